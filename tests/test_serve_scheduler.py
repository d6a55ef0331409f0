"""Continuous-batching scheduler on the CPU with a fake executor: the byte budget
is never exceeded, admission is arrival-ordered, an oversized request runs alone,
and requests that arrive while batches run join later batches."""
from dataclasses import dataclass

from nttanafis_gb300.serve import Scheduler, Pending, serve


@dataclass
class Item:
    arrival: float
    nbytes: int
    work: float  # simulated device seconds


class FakeClock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t

    def tick(self):
        self.t += 0.0005


class FakeExecutor:
    """Completes a batch after the sum of its members' work on a simulated clock."""

    def __init__(self, clock, budget):
        self.clock = clock
        self.budget = budget
        self.in_flight = 0
        self.max_in_flight = 0
        self.launched = []

    def nbytes(self, item):
        return item.nbytes

    def prepare(self, item):
        return item

    def launch(self, slot, payloads):
        self.launched.append([p.arrival for p in payloads])
        self.in_flight += sum(p.nbytes for p in payloads)
        self.max_in_flight = max(self.max_in_flight, self.in_flight)
        return {"end": self.clock() + sum(p.work for p in payloads), "bytes": sum(p.nbytes for p in payloads),
                "counted": False}

    def ready(self, h):
        if h is None:
            return True
        if self.clock() >= h["end"]:
            if not h["counted"]:
                self.in_flight -= h["bytes"]
                h["counted"] = True
            return True
        return False


def test_budget_fifo_and_overlap():
    clock = FakeClock()
    items = [Item(arrival=0.0002 * i, nbytes=100 + 37 * (i % 7), work=0.002) for i in range(200)]
    ex = FakeExecutor(clock, 1000)
    stats = serve(items, ex, budget_bytes=1000, slots=3, max_batch=8, clock=clock, idle=clock.tick)
    assert stats["requests"] == 200
    assert ex.max_in_flight <= 1000 and stats["peak_budget_bytes"] <= 1000
    # arrival order is kept inside and across batches
    flat = [a for batch in ex.launched for a in batch]
    assert flat == sorted(flat)
    assert stats["batches"] > 1 and stats["mean_batch"] > 1.0
    assert stats["p99_ms"] >= stats["p50_ms"] > 0


def test_oversized_request_runs_alone_when_idle():
    sched = Scheduler(budget_bytes=100, slots=2)
    sched.submit(Pending(0, 0.0, 500))
    sched.submit(Pending(1, 0.0, 10))
    take = sched.admit(sched.slots[0])
    assert [p.rid for p in take] == [0]
    assert sched.admit(sched.slots[1]) == []  # nothing else fits next to it
    sched.release(sched.slots[0])
    assert [p.rid for p in sched.admit(sched.slots[1])] == [1]


def test_later_arrivals_join_free_slots():
    clock = FakeClock()
    items = [Item(arrival=0.0, nbytes=10, work=0.05)] + [Item(arrival=0.01 + 0.001 * i, nbytes=10, work=0.001)
                                                         for i in range(20)]
    ex = FakeExecutor(clock, 10_000)
    stats = serve(items, ex, budget_bytes=10_000, slots=2, max_batch=64, clock=clock, idle=clock.tick)
    # the long first batch is still running when the later ones are served on the other slot
    first_done = stats["order"].index(0)
    assert first_done > 0
