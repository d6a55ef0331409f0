"""Served form: a continuous-batching request loop over the batch layer.

Requests (products, squares, convolutions of mixed sizes) arrive over time. The
scheduler keeps up to `slots` batches in flight, each on its own CUDA stream and
batch executor (tables and arenas stay resident), and admits waiting requests in
arrival order into every free slot while the sum of the in-flight requests'
device bytes stays within the HBM budget. A request larger than the whole budget
runs alone once nothing else is in flight. Requests that arrive while batches run
join the next free slot, so work from different arrivals overlaps on the device.

The scheduler (`Scheduler`) is host logic only; `GpuExecutor` runs its batches on
the GPU through `nttanafis_gb300.GpuBatch`, and tests drive it with a fake
executor on the CPU.
"""
from __future__ import annotations

import time
from collections import deque
from dataclasses import dataclass, field
from typing import Callable, Optional


@dataclass
class Pending:
    rid: int
    arrival: float
    nbytes: int          # device bytes the request holds while in flight
    payload: object = None
    admitted: float = -1.0
    done: float = -1.0


@dataclass
class Slot:
    index: int
    busy: bool = False
    members: list = field(default_factory=list)
    handle: object = None  # executor-specific completion handle


class Scheduler:
    """Arrival-ordered admission of requests into free slots under a byte budget."""

    def __init__(self, budget_bytes: int, slots: int, max_batch: int = 512):
        if slots < 1 or budget_bytes <= 0:
            raise ValueError("need at least one slot and a positive budget")
        self.budget = budget_bytes
        self.max_batch = max_batch
        self.slots = [Slot(i) for i in range(slots)]
        self.queue: deque[Pending] = deque()
        self.in_flight_bytes = 0
        self.peak_bytes = 0
        self.max_queue = 0
        self.batches = 0

    def submit(self, p: Pending) -> None:
        self.queue.append(p)
        self.max_queue = max(self.max_queue, len(self.queue))

    def admit(self, slot: Slot) -> list[Pending]:
        """Requests for a free slot: FIFO while the budget allows."""
        take = []
        while self.queue and len(take) < self.max_batch:
            head = self.queue[0]
            fits = self.in_flight_bytes + head.nbytes <= self.budget
            alone = not take and self.in_flight_bytes == 0  # oversized request, GPU idle
            if not (fits or alone):
                break
            take.append(self.queue.popleft())
            self.in_flight_bytes += head.nbytes
        if take:
            slot.busy = True
            slot.members = take
            self.batches += 1
            self.peak_bytes = max(self.peak_bytes, self.in_flight_bytes)
        return take

    def release(self, slot: Slot) -> list[Pending]:
        done = slot.members
        for p in done:
            self.in_flight_bytes -= p.nbytes
        slot.busy = False
        slot.members = []
        slot.handle = None
        return done


def percentile(values: list[float], q: float) -> float:
    if not values:
        return float("nan")
    s = sorted(values)
    k = min(len(s) - 1, max(0, int(round(q / 100.0 * (len(s) - 1)))))
    return s[k]


def serve(stream: list, executor, budget_bytes: int, slots: int = 4, max_batch: int = 512,
          clock: Callable[[], float] = time.perf_counter, idle: Optional[Callable[[], None]] = None) -> dict:
    """Runs `stream` (objects with .arrival seconds) through `executor` and returns
    latency and throughput statistics. `executor` provides nbytes(item),
    prepare(item) -> payload, launch(slot, payloads) -> handle, ready(handle)."""
    sched = Scheduler(budget_bytes, slots, max_batch)
    future = deque(sorted(enumerate(stream), key=lambda t: t[1].arrival))
    n = len(future)
    finished: list[Pending] = []
    t0 = clock()
    while len(finished) < n:
        now = clock() - t0
        while future and future[0][1].arrival <= now:
            rid, item = future.popleft()
            sched.submit(Pending(rid, item.arrival, executor.nbytes(item), executor.prepare(item)))
        progressed = False
        for slot in sched.slots:
            if slot.busy and executor.ready(slot.handle):
                t = clock() - t0
                for p in sched.release(slot):
                    p.done = t
                    finished.append(p)
                progressed = True
        for slot in sched.slots:
            if not slot.busy and sched.queue:
                take = sched.admit(slot)
                if take:
                    t = clock() - t0
                    for p in take:
                        p.admitted = t
                    slot.handle = executor.launch(slot, [p.payload for p in take])
                    progressed = True
        if not progressed:
            if not future and not sched.queue and not any(s.busy for s in sched.slots):
                break
            if idle is not None:
                idle()
    span = max(p.done for p in finished) - min(p.arrival for p in finished) if finished else float("nan")
    lat = [1000.0 * (p.done - p.arrival) for p in finished]
    return {
        "requests": len(finished), "span_s": span, "requests_per_s": len(finished) / span if span > 0 else None,
        "p50_ms": percentile(lat, 50), "p99_ms": percentile(lat, 99), "mean_ms": sum(lat) / max(1, len(lat)),
        "batches": sched.batches, "mean_batch": len(finished) / max(1, sched.batches),
        "peak_budget_bytes": sched.peak_bytes, "budget_bytes": budget_bytes, "max_queue_depth": sched.max_queue,
        "order": [p.rid for p in finished],
        "finished": finished,
    }


class GpuExecutor:
    """Runs scheduler batches on the GPU: one GpuBatch and CUDA stream per slot.
    Operands of every request are slices of a few resident random pools (one per
    coefficient class), so the synthetic stream needs no per-request upload; each
    request gets its own result buffer."""

    def __init__(self, slots: int, device=None, pool_limbs: int = 1 << 22):
        import numpy as np
        import torch

        from .api import GpuBatch
        from .operands import operand

        self.torch = torch
        self.device = device or torch.device("cuda", torch.cuda.current_device())
        self.batches = [GpuBatch() for _ in range(slots)]
        self.streams = [torch.cuda.Stream(device=self.device) for _ in range(slots)]
        raw_a, raw_b = operand(pool_limbs, 101), operand(pool_limbs, 102)

        def signed32(x):
            m = (x & np.uint64((1 << 31) - 1)).astype(np.uint64)
            return np.where((x >> np.uint64(63)).astype(bool), np.uint64(0) - m, m).astype(np.uint64)

        def put(x):
            return torch.from_numpy(np.ascontiguousarray(x).view(np.int64)).to(self.device)

        self.pools = {
            64: (put(raw_a), put(raw_b)),
            16: (put(raw_a & np.uint64(0xFFFF)), put(raw_b & np.uint64(0xFFFF))),
            32: (put(raw_a & np.uint64(0xFFFFFFFF)), put(raw_b & np.uint64(0xFFFFFFFF))),
            -32: (put(signed32(raw_a)), put(signed32(raw_b))),
        }
        self.pool_limbs = pool_limbs

    def operands(self, item):
        key = -32 if item.signed else (item.bits if item.kind == "conv" else 64)
        pa, pb = self.pools[key]
        oa = item.seed_a % max(1, self.pool_limbs - item.la + 1)
        a = pa[oa:oa + item.la]
        if item.kind == "sqr":
            return a, a
        ob = item.seed_b % max(1, self.pool_limbs - item.lb + 1)
        return a, pb[ob:ob + item.lb]

    def nbytes(self, item) -> int:
        from .api import ConvPlan, MulPlan

        if item.kind == "conv":
            plan = ConvPlan.new(item.la, item.lb, item.max_a, item.max_a, item.signed)
            return 8 * (plan.scratch_len() + plan.output_len())
        plan = MulPlan.new(item.la, item.lb)
        scratch = plan.sqr_scratch_len() if item.kind == "sqr" else plan.scratch_len()
        return 8 * (scratch + item.la + item.lb)

    def _make(self, item):
        from .api import Request

        a, b = self.operands(item)
        dst = self.torch.empty(item.out_len(), dtype=self.torch.int64, device=self.device)
        return Request(dst, a, b, "conv" if item.kind == "conv" else "mul", item.max_a, item.max_a, item.signed)

    def preload(self, items) -> None:
        """Allocates the result buffers of `items` ahead of time (a server draws
        them from a pool; allocating on arrival would put the allocator's device
        synchronisations inside the loop)."""
        self._pre = {id(it): self._make(it) for it in items}

    def prepare(self, item):
        pre = getattr(self, "_pre", None)
        if pre is not None and id(item) in pre:
            return pre.pop(id(item))
        return self._make(item)

    def launch(self, slot: Slot, payloads):
        from .api import last_error

        st = self.streams[slot.index]
        if not self.batches[slot.index].run(payloads, st):
            raise RuntimeError(last_error())
        ev = self.torch.cuda.Event()
        ev.record(st)
        return ev

    def ready(self, handle) -> bool:
        return handle is None or handle.query()

    def alone(self, item):
        """The same request computed by itself through the single-call entry points."""
        from .api import ConvPlan, GpuConvWorkspace, GpuMulWorkspace

        torch = self.torch
        a, b = self.operands(item)
        dst = torch.empty(item.out_len(), dtype=torch.int64, device=self.device)
        if item.kind == "conv":
            ws = GpuConvWorkspace()
            ok = ws.prepare(ConvPlan.new(item.la, item.lb, item.max_a, item.max_a, item.signed)) and \
                ws.convolve_device(dst, a, b, torch.cuda.current_stream())
        else:
            ws = GpuMulWorkspace()
            ok = ws.mul_device(dst, a, b, torch.cuda.current_stream())
        torch.cuda.synchronize()
        ws.close()
        if not ok:
            raise RuntimeError("single call failed")
        return dst

    def close(self) -> None:
        for b in self.batches:
            b.close()
