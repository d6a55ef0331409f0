"""Device-side coefficient admission of the device-pointer convolution calls
(the reference's ConvPlan::convolve rejects a coefficient above its bound and
leaves dst untouched, src/convolve.rs:169-184; src/tests/convolution.rs:310-350):
a rejected convolution is not written and its status says so, on the workspace,
plan and batch paths, for unsigned bounds and signed magnitudes, through the
transform and the schoolbook kernels."""
import os

import numpy as np
import pytest

import oracle
from nttanafis_gb300.operands import operand

pytestmark = pytest.mark.gpu
THREADS = os.cpu_count() or 1
MASK = (1 << 64) - 1


def dev(torch, x):
    return torch.from_numpy(np.ascontiguousarray(x).view(np.int64)).cuda()


def host(t):
    return t.cpu().numpy().view(np.uint64)


def operands(la, lb, mx, signed, seed):
    a, b = operand(la, seed) & np.uint64(mx), operand(lb, seed + 1) & np.uint64(mx)
    if signed:  # odd positions negative, magnitudes within the bound
        with np.errstate(over="ignore"):
            a[1::2] = np.uint64(0) - a[1::2]
            b[1::2] = np.uint64(0) - b[1::2]
    return a, b


def over_bound(x, mx, signed, pos):
    bad = x.copy()
    with np.errstate(over="ignore"):
        bad[pos] = np.uint64(0) - np.uint64(mx + 1) if signed else np.uint64(mx + 1)
    return bad


# (a_len, b_len, bound, signed): transform convolutions and a schoolbook one
CASES = [(3000, 2000, 0xFFFF, False), (5000, 4000, (1 << 31) - 1, True), (4000, 20, (1 << 32) - 1, False),
         (70000, 50000, 0xFFFF, False)]


@pytest.mark.parametrize("la,lb,mx,signed", CASES)
def test_workspace_device_call_rejects_over_bound(gpu, la, lb, mx, signed):
    import torch

    stream = torch.cuda.current_stream()
    w = gpu.GpuConvWorkspace()
    plan = gpu.ConvPlan.new(la, lb, mx, mx, signed)
    assert w.prepare(plan)
    a, b = operands(la, lb, mx, signed, 401)
    expected = oracle.conv(a, b, mx, mx, signed, THREADS)
    for bad_a, bad_b in [(over_bound(a, mx, signed, la // 2), b), (a, over_bound(b, mx, signed, lb - 1))]:
        dst = torch.full((plan.output_len() + 1,), -1, dtype=torch.int64, device="cuda")
        assert w.convolve_device(dst, dev(torch, bad_a), dev(torch, bad_b), stream)  # enqueued
        torch.cuda.synchronize()
        assert w.status() == gpu.STATUS_BOUND
        assert bool((dst == -1).all()), "a rejected convolution wrote its destination"
    assert w.status() == 0  # reading cleared it
    dst = torch.full((plan.output_len() + 1,), -1, dtype=torch.int64, device="cuda")
    assert w.convolve_device(dst, dev(torch, a), dev(torch, b), stream)
    torch.cuda.synchronize()
    assert w.status() == 0
    got = host(dst)
    assert np.array_equal(got[:-1], expected) and got[-1] == MASK
    w.close()


@pytest.mark.parametrize("la,lb,mx,signed", CASES[:3])
def test_plan_device_call_rejects_over_bound(gpu, la, lb, mx, signed):
    import torch

    stream = torch.cuda.current_stream()
    plan = gpu.ConvPlan.new(la, lb, mx, mx, signed)
    scratch = torch.full((plan.scratch_len(),), -1, dtype=torch.int64, device="cuda")
    a, b = operands(la, lb, mx, signed, 501)
    dst = torch.full((plan.output_len(),), -1, dtype=torch.int64, device="cuda")
    bad = dev(torch, over_bound(a, mx, signed, 0))
    assert plan.convolve_device(dst, bad, dev(torch, b), scratch, stream)
    assert plan.status(scratch, stream) == 0
    assert bool((dst == -1).all())
    assert plan.convolve_device(dst, dev(torch, a), dev(torch, b), scratch, stream)
    assert plan.status(scratch, stream) == 1
    assert np.array_equal(host(dst), oracle.conv(a, b, mx, mx, signed, THREADS))


def test_batch_member_over_bound_is_left_unwritten(gpu):
    import torch

    stream = torch.cuda.current_stream()
    batch = gpu.GpuBatch()
    members = [(3000, 2000, 0xFFFF, False, False), (3000, 2000, 0xFFFF, False, True),
               (5000, 20, (1 << 31) - 1, True, True), (6000, 5000, (1 << 32) - 1, False, False)]
    reqs, keep = [], []
    for i, (la, lb, mx, signed, bad) in enumerate(members):
        a, b = operands(la, lb, mx, signed, 601 + 2 * i)
        if bad:
            a = over_bound(a, mx, signed, la - 1)
        plan = gpu.ConvPlan.new(la, lb, mx, mx, signed)
        dst = torch.full((plan.output_len(),), -1, dtype=torch.int64, device="cuda")
        reqs.append(gpu.Request(dst, dev(torch, a), dev(torch, b), "conv", mx, mx, signed))
        keep.append((a, b, mx, signed, bad, dst))
    mul_a, mul_b = operand(4000, 7), operand(3000, 8)
    mul_dst = torch.empty(7000, dtype=torch.int64, device="cuda")
    reqs.append(gpu.Request(mul_dst, dev(torch, mul_a), dev(torch, mul_b)))
    assert batch.run(reqs, stream), gpu.last_error()
    torch.cuda.synchronize()
    assert batch.status() == gpu.STATUS_BOUND
    for a, b, mx, signed, bad, dst in keep:
        if bad:
            assert bool((dst == -1).all())
        else:
            assert np.array_equal(host(dst), oracle.conv(a, b, mx, mx, signed, THREADS))
    assert np.array_equal(host(mul_dst), oracle.mul(mul_a, mul_b))
    assert batch.status() == 0
    batch.close()


@pytest.mark.parametrize("la,lb,mx,signed", [(1 << 20, (1 << 20) - 5, 0xFFFF, False), (1 << 20, 3000, (1 << 31) - 1, True),
                                             (1 << 23, (1 << 23) - 3, 0xFFFF, False)])
def test_column_pass_admission_at_large_sizes(gpu, la, lb, mx, signed):
    # the two-pass 2^10-point column kernel (T = 2^21) and the radix-64 2^12-point
    # one (T = 2^24, wide primes) check the coefficients as they load them
    import torch

    stream = torch.cuda.current_stream()
    w = gpu.GpuConvWorkspace()
    plan = gpu.ConvPlan.new(la, lb, mx, mx, signed)
    assert w.prepare(plan)
    a, b = operands(la, lb, mx, signed, 701)
    for bad_a, bad_b in [(over_bound(a, mx, signed, la - 1), b), (a, over_bound(b, mx, signed, lb // 3))]:
        dst = torch.full((plan.output_len(),), -1, dtype=torch.int64, device="cuda")
        assert w.convolve_device(dst, dev(torch, bad_a), dev(torch, bad_b), stream)
        torch.cuda.synchronize()
        assert w.status() == gpu.STATUS_BOUND
        assert bool((dst == -1).all()), "a rejected convolution wrote its destination"
    dst = torch.full((plan.output_len(),), -1, dtype=torch.int64, device="cuda")
    assert w.convolve_device(dst, dev(torch, a), dev(torch, b), stream)
    torch.cuda.synchronize()
    assert w.status() == 0
    if la <= 1 << 20:
        assert np.array_equal(host(dst), oracle.conv(a, b, mx, mx, signed, THREADS))
    w.close()
