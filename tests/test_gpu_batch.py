"""Batched layer: every member of a mixed batch is bit-identical to the oracle and
to the same call made alone; an inadmissible member makes the batch launch
nothing."""
import os

import numpy as np
import pytest

import oracle
from nttanafis_gb300.operands import operand
from nttanafis_gb300.workloads import Shape, batched_shapes

pytestmark = pytest.mark.gpu
THREADS = os.cpu_count() or 1
MASK = (1 << 64) - 1


def device(torch, x):
    return torch.from_numpy(np.ascontiguousarray(x).view(np.int64)).cuda()


def expected(shape: Shape, a, b):
    if shape.kind == "conv":
        return oracle.conv(a, b, shape.max_a, shape.max_a, shape.signed, THREADS)
    if shape.kind == "sqr":
        return oracle.sqr(a, THREADS)
    return oracle.mul(a, b, THREADS)


def run_batch(gpu, torch, shapes):
    reqs, keep = [], []
    for s in shapes:
        a_h, b_h = s.operands()
        a = device(torch, a_h)
        b = a if s.kind == "sqr" else device(torch, b_h)
        dst = torch.full((s.out_len() + 1,), -1, dtype=torch.int64, device="cuda")
        reqs.append(gpu.Request(dst, a, b, "conv" if s.kind == "conv" else "mul", s.max_a, s.max_a, s.signed))
        keep.append((s, a_h, b_h, dst))
    return reqs, keep


def test_mixed_batch_matches_oracle(gpu):
    import torch

    rng = np.random.default_rng(3)
    shapes = []
    for i in range(160):
        kind = ["mul", "sqr", "conv"][i % 3]
        la = int(np.exp(rng.uniform(0, np.log(40000))))
        lb = int(np.exp(rng.uniform(0, np.log(40000))))
        if kind == "conv":
            bits, signed = [(16, False), (32, False), (32, True), (64, False)][i % 4]
            shapes.append(Shape("conv", la, lb, 11 + 2 * i, 12 + 2 * i, bits=bits, signed=signed))
        else:
            shapes.append(Shape(kind, la, la if kind == "sqr" else lb, 11 + 2 * i, 12 + 2 * i))
    shapes += [Shape("mul", 300000, 250000, 1, 2), Shape("sqr", 200000, 200000, 3, 3)]
    batch = gpu.GpuBatch()
    reqs, keep = run_batch(gpu, torch, shapes)
    assert batch.run(reqs, torch.cuda.current_stream()), gpu.last_error()
    torch.cuda.synchronize()
    for s, a, b, dst in keep:
        host = dst.cpu().numpy().view(np.uint64)
        assert host[-1] == MASK, s  # one limb past the result is untouched
        assert np.array_equal(host[:-1], expected(s, a, b)), s
    batch.close()


def test_batched_workload_sample_equals_single_calls(gpu):
    import torch

    shapes = batched_shapes(256, seed=5)
    batch = gpu.GpuBatch()
    reqs, keep = run_batch(gpu, torch, shapes)
    assert batch.run(reqs), gpu.last_error()
    ws = gpu.GpuMulWorkspace()
    torch.cuda.synchronize()
    for s, a_h, b_h, dst in keep:
        single = np.full(s.out_len(), MASK, dtype=np.uint64)
        ok = ws.sqr(single, a_h) if s.kind == "sqr" else ws.mul(single, a_h, b_h)
        assert ok
        assert np.array_equal(dst.cpu().numpy().view(np.uint64)[:-1], single), s
    ws.close()
    batch.close()


def test_inadmissible_member_launches_nothing(gpu):
    import torch

    a = device(torch, operand(1000, 1))
    b = device(torch, operand(900, 2))
    good = torch.full((1900,), 7, dtype=torch.int64, device="cuda")
    short = torch.full((1898,), 7, dtype=torch.int64, device="cuda")
    batch = gpu.GpuBatch()
    assert not batch.run([gpu.Request(good, a, b), gpu.Request(short, a, b)])
    torch.cuda.synchronize()
    assert bool((good == 7).all()) and bool((short == 7).all())
    # empty operands write zeros
    empty = torch.empty(0, dtype=torch.int64, device="cuda")
    z = torch.full((900,), 7, dtype=torch.int64, device="cuda")
    assert batch.run([gpu.Request(z, empty, b)])
    torch.cuda.synchronize()
    assert bool((z == 0).all())
    batch.close()


def check_batch(gpu, torch, batch, shapes, st):
    reqs, keep = run_batch(gpu, torch, shapes)
    assert batch.run(reqs, st), gpu.last_error()
    st.synchronize()
    for s, a, b, dst in keep:
        host = dst.cpu().numpy().view(np.uint64)
        assert host[-1] == MASK, s
        assert np.array_equal(host[:-1], expected(s, a, b)), s


def test_tuned_composition_replays_from_a_graph(gpu):
    # A repeated composition: run 1 direct, runs 2-7 time the lane counts, run 8
    # captures the fastest into a CUDA graph, later runs replay it with new
    # operands (new descriptors). Every run matches the oracle.
    import torch

    st = torch.cuda.Stream()
    lengths = [("mul", 700, 300), ("sqr", 1500, 1500), ("mul", 9000, 7000), ("conv", 3000, 2000),
               ("mul", 40000, 5000), ("sqr", 20000, 20000), ("mul", 100, 90), ("conv", 50000, 1000)]
    batch = gpu.GpuBatch()
    for run in range(9):
        shapes = [Shape(k, la, lb, 100 * run + 2 * i + 1, 100 * run + 2 * i + 2, bits=32, signed=True)
                  for i, (k, la, lb) in enumerate(lengths)]
        check_batch(gpu, torch, batch, shapes, st)
        stats = batch.stats()
        assert stats["tuned"] == (1 if run >= 7 else 0), (run, stats)
        assert stats["graph_replays"] == max(0, run - 6), (run, stats)
    assert batch.stats()["compositions"] == 1
    # graphs off: the tuned lane count, enqueued directly
    batch.set_graphs(False)
    shapes = [Shape(k, la, lb, 2 * i + 1, 2 * i + 2, bits=32, signed=True) for i, (k, la, lb) in enumerate(lengths)]
    check_batch(gpu, torch, batch, shapes, st)
    assert batch.stats()["graph_replays"] == 2
    batch.close()


@pytest.mark.parametrize("lanes", [1, 2, 4])
def test_fixed_lanes_capture_at_the_second_run(gpu, lanes):
    import torch

    st = torch.cuda.Stream()
    batch = gpu.GpuBatch()
    assert batch.set_lanes(lanes) == 0
    for run in range(3):
        shapes = [Shape("mul", 5000, 4000, 7 + run, 8), Shape("sqr", 300, 300, 9, 9), Shape("mul", 20, 33, 1, run),
                  Shape("conv", 4000, 4000, 3, 4 + run, bits=16)]
        check_batch(gpu, torch, batch, shapes, st)
        assert batch.stats()["graph_replays"] == run
        assert batch.stats()["tuned"] == 0
    # the legacy default stream runs directly
    check_batch(gpu, torch, batch, shapes, torch.cuda.default_stream())
    assert batch.stats()["graph_replays"] == 2
    batch.close()


def test_unbalanced_members_run_as_block_splits(gpu):
    """Members that the planner splits (src/multiply/execute.rs:114-209 of the
    reference) run as block splits inside the batch, beside ordinary classes, and
    stay exact over repeated runs (the ordinary classes replay from a graph)."""
    import torch

    shapes = [Shape("mul", 1 << 20, 1000, 41, 42), Shape("mul", 1500, (1 << 20) + 7, 43, 44),
              Shape("mul", 600000, 1000, 45, 46), Shape("mul", 5000, 4000, 47, 48), Shape("sqr", 3000, 3000, 49, 49),
              Shape("conv", 3000, 2000, 50, 51, bits=16, signed=False)]
    batch = gpu.GpuBatch()
    reqs, keep = run_batch(gpu, torch, shapes)
    want = [expected(s, a, b) for s, a, b, _ in keep]
    for run in range(3):
        for _, _, _, dst in keep:
            dst.fill_(-1)
        assert batch.run(reqs, torch.cuda.current_stream()), gpu.last_error()
        torch.cuda.synchronize()
        for (s, _, _, dst), w in zip(keep, want):
            host = dst.cpu().numpy().view(np.uint64)
            assert host[-1] == MASK, (run, s)
            assert np.array_equal(host[:-1], w), (run, s)
    assert batch.split_members == 9  # three split members per run
    assert batch.status() == 0
    batch.close()
