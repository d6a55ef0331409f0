"""Throughput of exact 1,048,576 x 1,048,576-limb products on GB300.

One step = one exact product of two 1M-limb operands (SplitMix64 seeds 1 and 2
plus per-set offsets), the workload the reference's headline number is quoted on
(README.md:28 of the reference: 43.4 ms on one Zen 5 core). Products are
independent: consecutive steps alternate between `--streams` workspaces and CUDA
streams (default 2), so one product's kernel tails overlap the next one's
(`config.one_stream_products_per_s` keeps the single-stream figure). N GPUs run N
replicas ("scaling": "weak") with no collective on the data path; the timed region
is bracketed by a barrier and a device sync on every rank and the slowest rank's
time counts.

Printed keys beyond the base contract:
  e2e         the same metric through the host-pointer C ABI call
              (ntt_mul_workspace_mul) from pinned host buffers, copies included,
              made by `--e2e-threads` host threads (default 4) on their own
              workspaces, so one call's transfers overlap another's kernels
              (`one_thread_products_per_s` keeps the single-caller figure);
  roofline    algorithmic bytes of one product (operands in, product out, and the
              fused four-step spectrum traffic 8*S with S from the reference
              planner) over the measured device time per product;
  compute_roofline  the transforms' butterflies per product over the device time,
              against the butterfly rate of a register-only probe (no memory
              traffic) run on the same GPU: the integer-issue ceiling;
  kernels     per-kernel device times from CUDA events recorded between the
              library's launches on the launching stream;
  cpu_baseline  the oracle (a C restatement of the reference algorithm) timed
              on this host's cores on a bounded sample of the same workload.

`--impl reference` times that CPU restatement alone (the reference crate is Rust
and cannot be built here), with every host thread, on the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

LA = LB = 1 << 20
L2_BYTES = 129 * 2**20
WORKLOAD = "mul 1048576x1048576 u64 limbs (SplitMix64)"
METRIC = "products/s (1,048,576 x 1,048,576-limb exact products)"


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


def shard_units(units: int, rank: int, world: int) -> range:
    """Replica sharding: rank r runs units r, r+world, ... (no data exchange)."""
    return range(rank, units, world)


def max_over_ranks(value: float, world: int, device=None) -> float:
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist

    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def measured_peak_gbs() -> tuple[float, str]:
    path = ROOT / "MEASURED_PEAKS.json"
    if path.exists():
        try:
            return float(json.loads(path.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi while running."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = ROOT / "gpurun_out" / f"clocks_bench_{gpu_index}.csv"

    def __enter__(self):
        try:
            self.path.parent.mkdir(exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self) -> dict:
        if self.proc is None or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sms, maxes, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sms.append(float(parts[1]))
                maxes.append(float(parts[2]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower() == "active":
                    reasons.add(name)
        if not sms:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        loaded = sorted(sms)[len(sms) // 2:] or sms
        return {"sm_mhz": float(np.median(loaded)), "sm_max_mhz": max(maxes), "reasons": sorted(reasons),
                "samples": len(sms)}


def operand_sets(count: int):
    from nttanafis_gb300.operands import operand

    return [(operand(LA, 1 + 2 * i), operand(LB, 2 + 2 * i)) for i in range(count)]


def cpu_sample(threads: int, seconds: float = 12.0, max_products: int = 20, min_products: int = 5) -> dict:
    """Times the oracle on whole products (bounded sample): at least `min_products`
    after one warm-up product, then more until `seconds` elapse; the value is the
    median per-product time. A single-threaded sample runs pinned to one core."""
    import statistics

    import oracle

    from nttanafis_gb300.operands import operand

    a, b = operand(LA, 1), operand(LB, 2)
    pinned = None
    if threads == 1 and hasattr(os, "sched_getaffinity"):
        pinned = os.sched_getaffinity(0)
        os.sched_setaffinity(0, {min(pinned)})
    try:
        oracle.mul(a, b, threads)  # tables, page-in
        times, t0 = [], time.perf_counter()
        while len(times) < max_products and (len(times) < min_products or time.perf_counter() - t0 < seconds):
            t = time.perf_counter()
            oracle.mul(a, b, threads)
            times.append(time.perf_counter() - t)
    finally:
        if pinned is not None:
            os.sched_setaffinity(0, pinned)
    med = statistics.median(times)
    return {"value": 1.0 / med, "seconds_per_product": med, "products": len(times), "threads": threads,
            "pinned_core": min(pinned) if pinned is not None else None}


def cpu_model() -> str:
    try:
        for line in Path("/proc/cpuinfo").read_text().splitlines():
            if line.lower().startswith(("model name", "cpu part")):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform

    return platform.machine()


def run_reference(args) -> None:
    rank, world, local = dist_env()
    if rank != 0:
        return
    import oracle

    from nttanafis_gb300.operands import operand

    threads = os.cpu_count() or 1
    a, b = operand(LA, 1), operand(LB, 2)
    for _ in range(args.warmup):
        oracle.mul(a, b, threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        oracle.mul(a, b, threads)
    dt = time.perf_counter() - t0
    value = args.steps / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "products/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (SplitMix64 seeds 1, 2)",
        "config": {"workload": WORKLOAD, "la": LA, "lb": LB, "l2": "n/a (CPU)"},
        "cpu_baseline": {"value": value, "unit": "products/s", "cores": threads, "kind": "port",
                         "sample": f"{args.steps} whole 1M x 1M products, {threads} threads, {cpu_model()}"},
        "e2e": {"value": value, "unit": "products/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


KERNEL_NAMES = ["pack+column DIF (k_fwd_cols)", "row DIF+pointwise+DIT (k_rows)", "column DIT (k_inv_cols)",
                "CRT+window sums+look-back carry (k_crt_mul)"]


def kernel_breakdown(run, reps: int):
    """Device time of each of a four-step product's kernels, from CUDA events the
    library records between its launches (ntt_timing_start/stop), averaged over
    `reps` products; None if the call did not take the four-kernel path."""
    import ctypes

    import nttanafis_gb300 as ntt

    lib = ntt.library()
    stride = len(KERNEL_NAMES) + 1
    ms = (ctypes.c_float * (reps * stride))()
    lib.ntt_timing_start(reps * stride)
    for _ in range(reps):
        run()
    got = lib.ntt_timing_stop(ms, reps * stride)
    if got != reps * stride - 1:
        return None
    return {n: round(sum(ms[r * stride + k] for r in range(reps)) / reps, 5) for k, n in enumerate(KERNEL_NAMES)}


def configs_section(dev, stream, peak_gbs: float) -> list:
    """Device time per product of every plain configuration (inputs resident), with
    its algorithmic bytes and roofline fraction. Squares pass the same tensor twice."""
    import torch

    import oracle
    import nttanafis_gb300 as ntt
    from nttanafis_gb300.operands import operand, sparse_operand

    ones = lambda n, s: np.full(n, np.uint64(0xFFFFFFFFFFFFFFFF), dtype=np.uint64)  # noqa: E731
    cases = [
        ("mul 256x256", 256, 256, operand, 8000),
        ("mul 1024x1024", 1024, 1024, operand, 8000), ("sqr 1024", 1024, 0, operand, 8000),
        ("mul 4096x4096", 4096, 4096, operand, 4000),
        ("mul 16384x16384", 1 << 14, 1 << 14, operand, 4000), ("mul 65536x65536", 1 << 16, 1 << 16, operand, 2000),
        ("mul 262144x262144", 1 << 18, 1 << 18, operand, 400),
        ("mul 1048576x1048576", 1 << 20, 1 << 20, operand, 100), ("sqr 1048576", 1 << 20, 0, operand, 100),
        ("mul 1048576x131072", 1 << 20, 131072, operand, 100),
        ("mul 1048576^2 all-ones", 1 << 20, 1 << 20, ones, 50),
        ("mul 1048576^2 99% zero limbs", 1 << 20, 1 << 20, lambda n, s: sparse_operand(n, s, s + 1), 50),
        ("mul 4194304x4194304", 1 << 22, 1 << 22, operand, 20),
        ("mul 16777216x16777216", 1 << 24, 1 << 24, operand, 6), ("sqr 16777216", 1 << 24, 0, operand, 6),
    ]
    broken_down = {"mul 1048576x1048576", "sqr 1048576", "mul 16777216x16777216", "sqr 16777216"}
    ws = ntt.GpuMulWorkspace()
    out = []
    for name, la, lb, gen, reps in cases:
        a = torch.from_numpy(gen(la, 1).view(np.int64)).to(dev)
        b = a if lb == 0 else torch.from_numpy(gen(lb, 2).view(np.int64)).to(dev)
        n_out = la + (la if lb == 0 else lb)
        d = torch.empty(n_out, dtype=torch.int64, device=dev)
        for _ in range(3):
            assert ws.mul_device(d, a, b, stream), ntt.last_error()
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            ws.mul_device(d, a, b, stream)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1) / reps
        model = oracle.model_bytes("sqr" if lb == 0 else "mul", la, lb or la)
        row = {"config": name, "ms_per_product": round(ms, 5), "products_per_s": round(1000.0 / ms, 1),
               "algorithmic_bytes": model, "roofline_frac": round(model / (ms / 1000.0) / 1e9 / peak_gbs, 4)}
        if name in broken_down:
            row["kernels_ms"] = kernel_breakdown(lambda: ws.mul_device(d, a, b, stream), min(reps, 10))
        out.append(row)
        del a, b, d
    ws.close()
    # Convolutions of 16-bit coefficients (the reference's published conv sizes,
    # README.md:33-36 of the reference), operands resident.
    cws = ntt.GpuConvWorkspace()
    for n, reps in ((1024, 4000), (65536, 1000), (1 << 20, 100), (1 << 22, 20)):
        plan = ntt.ConvPlan.new(n, n, 0xFFFF, 0xFFFF, False)
        assert cws.prepare(plan), ntt.last_error()
        a = torch.from_numpy((operand(n, 1) & np.uint64(0xFFFF)).view(np.int64)).to(dev)
        b = torch.from_numpy((operand(n, 2) & np.uint64(0xFFFF)).view(np.int64)).to(dev)
        d = torch.empty(plan.output_len(), dtype=torch.int64, device=dev)
        for _ in range(3):
            assert cws.convolve_device(d, a, b, stream), ntt.last_error()
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            cws.convolve_device(d, a, b, stream)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1) / reps
        out.append({"config": f"conv 16-bit {n}", "ms_per_product": round(ms, 5),
                    "products_per_s": round(1000.0 / ms, 1), "primes": plan.primes,
                    "log_transform": plan.log_transform})
        del a, b, d
    cws.close()
    torch.cuda.empty_cache()
    return out


def batched_section(dev, stream, count: int = 4096, reps: int = 3) -> dict:
    """Batched configuration: `count` products (log-uniform 256..65536 limbs, ratio
    up to 8:1, 25% squares) through the batch layer in one enqueue, against the
    same products issued one workspace call each, on the same resident inputs."""
    import torch

    import nttanafis_gb300 as ntt
    from nttanafis_gb300.workloads import batched_shapes

    shapes = batched_shapes(count, seed=5)
    reqs, singles = [], []
    limbs = 0
    for s in shapes:
        a_h, b_h = s.operands()
        a = torch.from_numpy(a_h.view(np.int64)).to(dev)
        b = a if s.kind == "sqr" else torch.from_numpy(b_h.view(np.int64)).to(dev)
        d = torch.empty(s.out_len(), dtype=torch.int64, device=dev)
        reqs.append(ntt.Request(d, a, b))
        singles.append((d, a, b))
        limbs += s.la + s.lb
    batch = ntt.GpuBatch()
    direct = ntt.GpuBatch()  # one stream, no graph: the layer without its scheduler
    direct.set_graphs(False)
    direct.set_lanes(1)
    packed = ntt.GpuBatch.pack(reqs)
    ws = ntt.GpuMulWorkspace()
    # warm-up (tables, arenas) of every form; the batch tunes its lane count on runs
    # 2-7 of this composition and captures the winner into a graph at run 8
    for _ in range(8):
        assert batch.run(packed, stream), ntt.last_error()
    assert direct.run(packed, stream), ntt.last_error()
    for d, a, b in singles[:64]:
        assert ws.mul_device(d, a, b, stream), ntt.last_error()
    torch.cuda.synchronize(dev)

    def timed(fn) -> float:
        best = float("inf")
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize(dev)
            best = min(best, max(e0.elapsed_time(e1) / 1000.0, time.perf_counter() - t0))
        return best

    def steady(b, runs: int = 10) -> float:
        # back-to-back runs on one stream: the host plans run i+1 while run i executes
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        e0.record(stream)
        for _ in range(runs):
            b.run(packed, stream)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        return max(e0.elapsed_time(e1) / 1000.0, time.perf_counter() - t0) / runs

    launches0 = ntt.kernel_launches()
    replays0 = batch.graph_replays
    t_batch = timed(lambda: batch.run(packed, stream))
    batch_launches = (ntt.kernel_launches() - launches0) // reps
    graph_replays = batch.graph_replays - replays0
    t_direct = timed(lambda: direct.run(packed, stream))
    t_steady, t_steady_direct = steady(batch), steady(direct)
    stats = batch.stats()
    # parity of a sample of members against single calls
    sample_ok = True
    import random

    rnd = random.Random(1)
    for i in rnd.sample(range(count), 16):
        d, a, b = singles[i]
        got = d.clone()
        ref = torch.empty_like(d)
        assert ws.mul_device(ref, a, b, stream)
        torch.cuda.synchronize(dev)
        sample_ok &= bool(torch.equal(got, ref))
    launches0 = ntt.kernel_launches()
    t_plain = timed(lambda: [ws.mul_device(d, a, b, stream) for d, a, b in singles])
    plain_launches = (ntt.kernel_launches() - launches0) // reps
    batch.close()
    direct.close()
    ws.close()
    return {
        "workload": f"{count} products, log-uniform 256..65536 limbs, ratio <= 8:1, 25% squares (seed 5)",
        "products_per_s": count / t_batch, "plain_products_per_s": count / t_plain,
        "graph_replays": graph_replays, "tuned_lanes": stats["last_lanes"],
        "steady_products_per_s": count / t_steady,
        "one_stream_no_graph": {"products_per_s": count / t_direct, "steady_products_per_s": count / t_steady_direct},
        "speedup_vs_plain": t_plain / t_batch, "steady_speedup_vs_plain": t_plain / t_steady,
        "ms_batch": 1000 * t_batch, "ms_plain": 1000 * t_plain,
        "launches_batch": batch_launches, "launches_plain": plain_launches, "limbs_in": limbs,
        "parity_sample_ok": sample_ok,
        "timing": ("products_per_s: best of 3 single runs, max(device events, host wall) per enqueue+completion; "
                   "steady_products_per_s: 10 back-to-back runs"),
    }


def served_section(dev, count: int = 400, rates=(2000.0, 20000.0), budget_gb: float = 8.0, slots: int = 4) -> dict:
    """Served configuration: Poisson arrivals of products/squares (log-uniform
    192..4,194,304 limbs) and 16/32-bit unsigned and 32-bit signed convolutions
    (1,024..4,194,304 coefficients), continuous batching under an HBM budget, at a
    few arrival rates; against the same requests issued one call at a time."""
    import torch

    import nttanafis_gb300 as ntt
    from nttanafis_gb300.serve import GpuExecutor, serve
    from nttanafis_gb300.workloads import served_stream

    ex = GpuExecutor(slots, dev)
    out = {"workload": f"{count} requests per rate; mul/sqr 192..4194304 limbs, conv 1024..4194304 coefficients "
                       "(16-bit, 32-bit unsigned, 32-bit signed)", "budget_bytes": int(budget_gb * 2**30),
           "slots": slots, "rates": []}
    # Warm-up over the whole size range: root tables and batch arenas reach their
    # working sizes before the timed streams (a server starts warm).
    warm = served_stream(count, 1e9, seed=99)
    ex.preload(warm)
    serve(warm, ex, int(budget_gb * 2**30), slots)
    torch.cuda.synchronize(dev)
    for rate in rates:
        stream = served_stream(count, rate, seed=7)
        ex.preload(stream)
        torch.cuda.synchronize(dev)
        stats = serve(stream, ex, int(budget_gb * 2**30), slots)
        torch.cuda.synchronize(dev)
        finished = stats.pop("finished")
        stats.pop("order")
        # parity: a sample of results equals the same request computed alone
        ok = True
        for p in finished[:: max(1, len(finished) // 12)]:
            ok &= bool(torch.equal(p.payload.dst, ex.alone(stream[p.rid])))
        stats["rate_hz"] = rate
        stats["parity_sample_ok"] = ok
        out["rates"].append(stats)
    # plain: the same requests one call at a time on one stream
    stream = served_stream(count, rates[-1], seed=7)
    payloads = [ex.prepare(item) for item in stream]
    ws, cws = ntt.GpuMulWorkspace(), ntt.GpuConvWorkspace()
    st = torch.cuda.Stream(device=dev)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for item, r in zip(stream, payloads):
        if item.kind == "conv":
            cws.prepare(ntt.ConvPlan.new(item.la, item.lb, item.max_a, item.max_a, item.signed))
            cws.convolve_device(r.dst, r.a, r.b, st)
        else:
            ws.mul_device(r.dst, r.a, r.b, st)
    torch.cuda.synchronize(dev)
    plain = time.perf_counter() - t0
    out["plain_requests_per_s"] = count / plain
    best = max(r["requests_per_s"] for r in out["rates"])
    out["speedup_vs_plain"] = best / out["plain_requests_per_s"]
    ws.close()
    cws.close()
    ex.close()
    return out


def field_section(dev, n: int = 1 << 26, reps: int = 20) -> dict:
    """Batched PrimeField products (the catalog's first field) over n residues, with
    each product method: elements/s of out = a * b, inputs resident."""
    import torch

    import nttanafis_gb300 as ntt
    from nttanafis_gb300.field import mul_method

    f = next(ntt.PrimeField.catalog())
    gen = torch.Generator(device=dev).manual_seed(11)
    a = torch.randint(0, f.modulus, (n,), device=dev, generator=gen)
    b = torch.randint(0, f.modulus, (n,), device=dev, generator=gen)
    outs = {}
    result = {"workload": f"out = a * b mod p over {n} residues of p = {f.modulus}"}
    previous = mul_method()
    for name, m in (("barrett", 0), ("fp64", 1)):
        mul_method(m)
        out = torch.empty_like(a)
        f.mul(out, a, b)
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            f.mul(out, a, b)
        e1.record()
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1) / reps
        result[name] = {"elements_per_s": n / (ms / 1000.0), "ms": ms, "gb_per_s": 24 * n / (ms / 1000.0) / 1e9}
        outs[name] = out
    mul_method(previous)
    result["bit_identical"] = bool(torch.equal(outs["barrett"], outs["fp64"]))
    return result


def run_gpu(args) -> None:
    import torch

    import oracle
    import nttanafis_gb300 as ntt

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    lib = ntt.library()
    # Four-step split per transform length, measured on this GPU (a fraction of a second).
    splits = {}
    if not args.no_tune:
        try:
            splits = ntt.tune_splits(14, 23, reps=3, stream=torch.cuda.current_stream(dev))
        except RuntimeError as exc:  # e.g. no room for the tuning operands: default splits
            print(f"split tuning skipped: {exc}", file=sys.stderr)

    per_step_in = 8 * (LA + LB)
    nsets = max(2, -(-2 * L2_BYTES // per_step_in))  # rotating inputs larger than L2
    host_sets = operand_sets(nsets)
    d_a = [torch.from_numpy(a.view(np.int64)).to(dev) for a, _ in host_sets]
    d_b = [torch.from_numpy(b.view(np.int64)).to(dev) for _, b in host_sets]
    d_out = [torch.empty(LA + LB, dtype=torch.int64, device=dev) for _ in range(nsets)]
    plan = ntt.MulPlan.new(LA, LB)
    # Independent products run on `streams` workspaces and streams (product i on
    # stream i mod streams), so one product's kernel tails overlap the next one's.
    nstreams = max(1, args.streams)
    wss = [ntt.GpuMulWorkspace() for _ in range(nstreams)]
    for w in wss:
        assert w.prepare(plan), ntt.last_error()
    ws = wss[0]
    streams = [torch.cuda.Stream(device=dev) for _ in range(nstreams)]
    stream = streams[0]

    def step(i: int, n: int = nstreams) -> None:
        k = i % nsets
        if not wss[i % n].mul_device(d_out[k], d_a[k], d_b[k], streams[i % n]):
            raise RuntimeError(ntt.last_error())

    def timed(steps: int, n: int) -> float:
        """Device milliseconds of `steps` products spread over n streams."""
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(streams[0])
        for st in streams[1:n]:
            st.wait_event(e0)
        for i in range(steps):
            step(i, n)
        for st in streams[1:n]:
            ev = torch.cuda.Event()
            ev.record(st)
            streams[0].wait_event(ev)
        e1.record(streams[0])
        torch.cuda.synchronize(dev)
        return e0.elapsed_time(e1)

    for i in range(args.warmup):
        step(i)
    torch.cuda.synchronize(dev)

    # Parity of the timed configuration against exact fingerprints.
    from nttanafis_gb300.operands import to_int

    A, B = to_int(host_sets[0][0]), to_int(host_sets[0][1])
    C = to_int(d_out[0].cpu().numpy().view(np.uint64)) if args.warmup else None
    fingerprint_ok = None
    if C is not None:
        qs = [(1 << 61) - 1, (1 << 89) - 1, (1 << 107) - 1]
        fingerprint_ok = all((A % q) * (B % q) % q == C % q for q in qs)

    sampler = ClockSampler(local)
    launches0 = ntt.kernel_launches()
    with sampler:
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(dev)
        t_wall = time.perf_counter()
        dev_ms = timed(args.steps, nstreams)
        t_wall = time.perf_counter() - t_wall
        if world > 1:
            torch.distributed.barrier()
        launches = ntt.kernel_launches() - launches0
        one_stream_steps = min(args.steps, 100)
        one_stream_ms = timed(one_stream_steps, 1) / one_stream_steps

        # End to end through the host-pointer C ABI call, pinned host memory: each
        # of `e2e_threads` host threads calls ntt_mul_workspace_mul on its own
        # workspace (the call blocks until the product is in its pinned buffer).
        import threading

        nthreads = max(1, args.e2e_threads)
        e2e_steps = max(3, min(args.steps, 50)) * nthreads
        bufs = []
        for t in range(nthreads):
            h_a = torch.from_numpy(host_sets[t % nsets][0].view(np.int64)).pin_memory()
            h_b = torch.from_numpy(host_sets[t % nsets][1].view(np.int64)).pin_memory()
            h_dst = torch.empty(LA + LB, dtype=torch.int64).pin_memory()
            bufs.append((h_a, h_b, h_dst, *(x.numpy().view(np.uint64) for x in (h_a, h_b, h_dst))))
        e2e_ws = wss + [ntt.GpuMulWorkspace() for _ in range(nthreads - len(wss))]
        failures = []

        def caller(t: int, count: int) -> None:
            na, nb, nd = bufs[t][3:]
            for _ in range(count):
                if not e2e_ws[t].mul(nd, na, nb):
                    failures.append(ntt.last_error())

        def run_e2e(n: int, steps: int) -> float:
            threads = [threading.Thread(target=caller, args=(t, steps // n + (t < steps % n))) for t in range(n)]
            t0 = time.perf_counter()
            for th in threads:
                th.start()
            for th in threads:
                th.join()
            return time.perf_counter() - t0

        run_e2e(nthreads, 2 * nthreads)
        e2e_s = run_e2e(nthreads, e2e_steps)
        e2e_one_s = run_e2e(1, e2e_steps // nthreads) / (e2e_steps // nthreads)
        # One caller with pageable (ordinary) host buffers, what a drop-in caller
        # passing its own slices gives the library.
        pa, pb = host_sets[0][0].copy(), host_sets[0][1].copy()
        pd = np.empty(LA + LB, dtype=np.uint64)
        assert e2e_ws[0].mul(pd, pa, pb), ntt.last_error()
        pageable_steps = max(3, min(args.steps, 20))
        t0 = time.perf_counter()
        for _ in range(pageable_steps):
            if not e2e_ws[0].mul(pd, pa, pb):
                failures.append(ntt.last_error())
        e2e_pageable_s = (time.perf_counter() - t0) / pageable_steps
        assert not failures, failures[:1]
        e2e_ok = True
        for t in range(nthreads):
            At, Bt = to_int(host_sets[t % nsets][0]), to_int(host_sets[t % nsets][1])
            q = (1 << 61) - 1
            e2e_ok &= to_int(bufs[t][5]) % q == (At % q) * (Bt % q) % q

    max_ms = max_over_ranks(dev_ms, world, dev)
    ms_per_step = max_ms / args.steps
    value = world * args.steps / (max_ms / 1000.0)
    e2e_value = world * e2e_steps / max_over_ranks(e2e_s, world, dev)

    # Per-kernel device times: events recorded between the library's launches.
    kernel_names = KERNEL_NAMES
    import ctypes

    reps = 10
    stride = len(kernel_names) + 1
    per_kernel = [0.0] * len(kernel_names)
    ms = (ctypes.c_float * (reps * stride))()
    lib.ntt_timing_start(reps * stride)
    for r in range(reps):
        step(r, 1)
    got = lib.ntt_timing_stop(ms, reps * stride)
    timed_ok = got == reps * stride - 1
    if timed_ok:
        for r in range(reps):
            for k in range(len(kernel_names)):
                per_kernel[k] += ms[r * stride + k] / reps
    kernels = [{"kernel": n_, "ms": round(t, 5)} for n_, t in zip(kernel_names, per_kernel)]
    instrumented_ms = sum(per_kernel)
    dominant = max(range(len(per_kernel)), key=lambda k: per_kernel[k]) if timed_ok else None

    peak, peak_kind = measured_peak_gbs()
    model = oracle.model_bytes("mul", LA, LB)
    achieved = model / (ms_per_step / 1000.0) / 1e9
    traffic = None
    tpath = ROOT / "profiles" / "traffic_mul_1M.json"
    if tpath.exists():
        try:
            traffic = json.loads(tpath.read_text()).get("dram_bytes_per_product")
        except Exception:
            traffic = None

    # Compute ceiling: the transforms' butterflies against a register-only probe of
    # the same lazy butterfly (no memory traffic) measured now on this GPU.
    t_len = 1 << plan.log_transform
    butterflies = 3 * plan.primes * (t_len // 2) * plan.log_transform
    from nttanafis_gb300 import probe

    probe_rate = probe.butterfly_rate()
    bfly_rate = butterflies / (ms_per_step / 1000.0)
    # Per-butterfly cost of the candidate residue arithmetics (register-only probes):
    # the transforms' 32-bit Shoup butterfly against a 32-bit Montgomery one, a
    # 64-bit Shoup one over a 50-bit prime and the reference's f64 FMA one, and the
    # raw instruction rates behind them.
    arith = {name: probe.rate(v) for v, name in enumerate(probe.VARIANTS)}

    line = {
        "metric": METRIC, "value": value, "unit": "products/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32 modular (NTT primes < 2^31), u64 limbs", "data": "synthetic (SplitMix64)",
        "config": {"workload": WORKLOAD, "la": LA, "lb": LB, "primes": plan.primes,
                   "log_transform": plan.log_transform, "parallelism": f"replicas x{world}",
                   "streams": nstreams, "one_stream_products_per_s": 1000.0 / one_stream_ms,
                   "four_step_splits": {f"2^{t}": f"2^{r} x 2^{t - r}" for t, r in splits.items()},
                   "l2": f"inputs larger than L2: {nsets} rotating operand pairs ({nsets * per_step_in >> 20} MiB)"},
        "e2e": {"value": e2e_value, "unit": "products/s", "h2d_bytes_per_step": per_step_in,
                "d2h_bytes_per_step": 8 * (LA + LB), "api": "ntt_mul_workspace_mul (host pointers, pinned)",
                "host_threads": nthreads, "one_thread_products_per_s": 1.0 / e2e_one_s,
                "one_thread_pageable_products_per_s": 1.0 / e2e_pageable_s,
                "steps": e2e_steps, "parity_ok": bool(e2e_ok)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else peak_kind,
                     "traffic": traffic, "algorithmic_bytes": model,
                     "unit_of_launch": "one product (the fused kernel sequence below)",
                     "dominant_kernel": kernel_names[dominant] if dominant is not None else None},
        "compute_roofline": {"bound": "integer issue", "achieved": bfly_rate, "peak": probe_rate,
                             "unit": "butterflies/s", "frac": bfly_rate / probe_rate,
                             "butterflies_per_product": butterflies,
                             "floor_ms": butterflies / probe_rate * 1000.0,
                             "peak_kind": "measured now: register-only lazy-butterfly probe (ntt_probe_butterflies)"},
        "arith_probe": {"unit": "operations/s (butterflies for *_butterfly*, instructions otherwise)",
                        "rates": arith},
        "kernels": kernels, "kernels_ms_total": instrumented_ms,
        "gpu_launches": launches, "wall_s": t_wall,
        "parity": {"fingerprint_ok": fingerprint_ok, "lookback_timeouts": ntt.lookback_timeouts()},
    }
    line["clocks"] = sampler.summary()
    if rank == 0 and not args.no_configs:
        line["configs"] = configs_section(dev, stream, peak)
    if rank == 0 and not args.no_batched:
        line["batched"] = batched_section(dev, stream)
    if rank == 0 and not args.no_served:
        line["served"] = served_section(dev, slots=args.served_slots)
    if rank == 0 and not args.no_configs:
        line["field"] = field_section(dev)
    if rank == 0 and not args.no_cpu:
        cores = os.cpu_count() or 1
        multi = cpu_sample(cores, seconds=args.cpu_seconds)
        single = cpu_sample(1, seconds=args.cpu_seconds / 2, max_products=10)
        line["cpu_baseline"] = {
            "value": multi["value"], "unit": "products/s", "cores": cores, "kind": "port",
            "sample": (f"median of {multi['products']} whole 1M x 1M products on {cores} threads ({cpu_model()}); "
                       f"single thread pinned to core {single['pinned_core']}: {single['value']:.3f} products/s, "
                       f"median of {single['products']}"),
            "single_thread_value": single["value"],
            "single_thread_ms": 1000.0 * single["seconds_per_product"],
            "published_reference_single_core_ms": 43.4,
        }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-configuration section")
    ap.add_argument("--no-served", action="store_true", help="skip the served-configuration section")
    ap.add_argument("--no-configs", action="store_true", help="skip the per-configuration timings")
    ap.add_argument("--no-tune", action="store_true", help="keep the default four-step splits (no tuning run)")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--streams", type=int, default=2, help="streams (and workspaces) the timed products alternate on")
    ap.add_argument("--e2e-threads", type=int, default=4, help="host threads making the host-pointer calls")
    ap.add_argument("--served-slots", type=int, default=4, help="batches in flight in the served section")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
