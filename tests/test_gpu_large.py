"""Parity at the largest served convolution sizes: 4,194,304 x 4,194,304
coefficients (T = 2^23) in each served class, and an unbalanced
4,194,304 x 1,024 convolution, bit-exact against the oracle on every host thread
(the reference's ConvPlan::convolve, src/convolve.rs:148-162, at the sizes of its
benchmark rows, README.md:33-36; value ranges as src/tests/convolution.rs:136-157
draws them)."""
import os

import numpy as np
import pytest

import oracle
from nttanafis_gb300.operands import operand

pytestmark = pytest.mark.gpu
MASK = (1 << 64) - 1
THREADS = os.cpu_count() or 1
N = 1 << 22


def signed_values(values: np.ndarray, mx: int) -> np.ndarray:
    """Magnitude below the bound, sign from each limb's top bit (vectorised)."""
    mag = values & np.uint64(mx)
    neg = (values >> np.uint64(63)) != 0
    with np.errstate(over="ignore"):
        return np.where(neg, np.uint64(0) - mag, mag).astype(np.uint64)


def operands(la: int, lb: int, bits: int, signed: bool, seed: int):
    mx = (1 << bits) - 1
    a, b = operand(la, seed), operand(lb, seed + 1)
    if signed:
        return signed_values(a, mx), signed_values(b, mx), 1 << bits
    return a & np.uint64(mx), b & np.uint64(mx), mx


@pytest.fixture(scope="module")
def cws(gpu):
    w = gpu.GpuConvWorkspace()
    yield w
    w.close()


def convolve(gpu, cws, a, b, mx, signed):
    plan = gpu.ConvPlan.new(a.size, b.size, mx, mx, signed)
    assert plan is not None and cws.prepare(plan)
    dst = np.full(plan.output_len() + 1, MASK, dtype=np.uint64)
    assert cws.convolve(dst, a, b), gpu.last_error()
    assert dst[-1] == MASK, "suffix was overwritten"
    return plan, dst[:-1]


@pytest.mark.parametrize("bits,signed", [(16, False), (32, False), (31, True)])
def test_served_classes_at_4m_coefficients(gpu, cws, bits, signed):
    # 16-bit unsigned (bound 2^16-1), 32-bit unsigned (2^32-1), 32-bit signed (2^31)
    a, b, mx = operands(N, N, bits, signed, 201 + bits)
    plan, got = convolve(gpu, cws, a, b, mx, signed)
    assert plan.log_transform == 23
    assert np.array_equal(got, oracle.conv(a, b, mx, mx, signed, THREADS)), (bits, signed)


@pytest.mark.parametrize("bits,signed", [(16, False), (31, True)])
def test_unbalanced_4m_by_1024(gpu, cws, bits, signed):
    a, b, mx = operands(N, 1024, bits, signed, 301 + bits)
    _, got = convolve(gpu, cws, a, b, mx, signed)
    assert np.array_equal(got, oracle.conv(a, b, mx, mx, signed, THREADS)), (bits, signed)
    _, swapped = convolve(gpu, cws, b, a, mx, signed)
    assert np.array_equal(swapped, got)


def test_wide_prime_convolution_at_2_pow_22(gpu, cws):
    # 64-bit unsigned coefficients, the shorter operand above 2^20 terms: the bound
    # needs 149 bits, five wide primes (five lazy ones hold 148 at 2^22); maximal
    # coefficients, exact against the oracle, and admission on the wide column pass
    import torch

    mx = (1 << 64) - 1
    la, lb = 3 * (1 << 20) - 7, (1 << 20) + 3
    a = np.full(la, MASK, dtype=np.uint64)
    b = operand(lb, 501)
    b[::3] = np.uint64(MASK)
    plan, got = convolve(gpu, cws, a, b, mx, False)
    assert plan.log_transform == 22 and plan.primes == 5 and plan.stride() == 3
    assert np.array_equal(got, oracle.conv(a, b, mx, mx, False, THREADS))
    # a bound one below the maximum rejects the all-ones operand on the device path
    stream = torch.cuda.current_stream()
    small = gpu.ConvPlan.new(la, lb, mx - 1, mx - 1, False)
    w = gpu.GpuConvWorkspace()
    assert w.prepare(small)
    dst = torch.full((small.output_len(),), -1, dtype=torch.int64, device="cuda")
    da = torch.from_numpy(a.view(np.int64)).cuda()
    db = torch.from_numpy((b & np.uint64(mx - 1)).view(np.int64)).cuda()
    assert w.convolve_device(dst, da, db, stream)
    torch.cuda.synchronize()
    assert w.status() == gpu.STATUS_BOUND and bool((dst == -1).all())
    w.close()
