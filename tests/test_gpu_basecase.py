"""The short-product basecase (direct column sums in one thread-block cluster):
bit-exact against the oracle over 1..=512 limbs in both operands (the proptest
range of src/tests/products.rs:134-135 widened to the basecase's range), through
its carry scan (all-ones operands, whose carries run through every limb:
src/tests/scheduling.rs:35-45), for squares and unbalanced shapes, and equal to
the transform path on the same operands."""
import numpy as np
import pytest

import oracle
from nttanafis_gb300.operands import operand

pytestmark = pytest.mark.gpu
MASK = (1 << 64) - 1


def all_ones_expected(la: int, lb: int) -> np.ndarray:
    left, right = max(la, lb), min(la, lb)
    out = np.zeros(la + lb, dtype=np.uint64)
    out[0] = 1
    out[right:] = MASK
    out[left] = MASK - 1
    return out


@pytest.fixture
def basecase(gpu):
    previous = gpu.set_basecase_limit(1 << 40)  # every product the basecase holds
    ws = gpu.GpuMulWorkspace()
    yield ws
    ws.close()
    gpu.set_basecase_limit(previous)


def mul(ws, a, b, extra=1):
    dst = np.full(a.size + b.size + extra, MASK, dtype=np.uint64)
    assert ws.mul(dst, a, b)
    assert np.all(dst[a.size + b.size:] == MASK), "suffix was overwritten"
    return dst[:a.size + b.size]


def test_every_length_up_to_512(basecase):
    rng = np.random.default_rng(101)
    lengths = list(range(1, 41)) + [63, 64, 65, 127, 128, 129, 191, 192, 193, 255, 256, 257, 383, 511, 512]
    for la in lengths:
        for lb in (1, 2, 7, 16, 33, 100, 256, 512):
            a = rng.integers(0, 2**64, la, dtype=np.uint64)
            b = rng.integers(0, 2**64, lb, dtype=np.uint64)
            assert np.array_equal(mul(basecase, a, b), oracle.schoolbook(a, b)), (la, lb)


def test_squares_and_aliases(basecase):
    for n in (1, 5, 64, 255, 256, 511, 512):
        a = operand(n, 7 + n)
        sq = np.full(2 * n + 1, MASK, dtype=np.uint64)
        assert basecase.sqr(sq, a) and sq[-1] == MASK
        assert np.array_equal(sq[:-1], oracle.sqr(a))
        assert np.array_equal(mul(basecase, a, a), oracle.sqr(a))


@pytest.mark.parametrize("la,lb", [(1, 1), (2, 3), (64, 64), (100, 33), (256, 256), (511, 513), (512, 512),
                                   (1000, 24), (1, 1023), (700, 300)])
def test_all_ones_carries_through_every_limb(basecase, la, lb):
    a = np.full(la, MASK, dtype=np.uint64)
    b = np.full(lb, MASK, dtype=np.uint64)
    assert np.array_equal(mul(basecase, a, b), all_ones_expected(la, lb)), (la, lb)


def test_unbalanced_and_random_shapes_match_the_transforms(gpu, basecase):
    rng = np.random.default_rng(103)
    ntt_ws = gpu.GpuMulWorkspace()
    try:
        for _ in range(24):
            la = int(rng.integers(1, 1000))
            lb = int(rng.integers(1, 1025 - la))
            a, b = operand(la, 2 * la + 1), operand(lb, 2 * lb + 2)
            got = mul(basecase, a, b)
            previous = gpu.set_basecase_limit(0)
            try:
                via_transforms = mul(ntt_ws, a, b)
            finally:
                gpu.set_basecase_limit(previous)
            assert np.array_equal(got, via_transforms), (la, lb)
            assert np.array_equal(got, oracle.mul(a, b)), (la, lb)
    finally:
        ntt_ws.close()


def test_device_and_plan_paths(gpu, basecase):
    import torch

    a_h, b_h = operand(700, 1), operand(300, 2)
    expected = oracle.mul(a_h, b_h)
    a = torch.from_numpy(a_h.view(np.int64)).cuda()
    b = torch.from_numpy(b_h.view(np.int64)).cuda()
    dst = torch.full((1001,), -1, dtype=torch.int64, device="cuda")
    stream = torch.cuda.current_stream()
    assert basecase.mul_device(dst, a, b, stream)
    plan = gpu.MulPlan.new(700, 300)
    scratch = torch.full((max(1, plan.scratch_len()),), -1, dtype=torch.int64, device="cuda")
    dst2 = torch.full((1000,), -1, dtype=torch.int64, device="cuda")
    assert plan.mul_device(dst2, a, b, scratch, stream)
    torch.cuda.synchronize()
    got = dst.cpu().numpy().view(np.uint64)
    assert np.array_equal(got[:1000], expected) and got[1000] == MASK
    assert np.array_equal(dst2.cpu().numpy().view(np.uint64), expected)
