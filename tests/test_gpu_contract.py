"""Public-contract behaviour of the GPU drop-in, mirroring the reference's
contract tests (src/tests/products.rs, src/tests/convolution.rs)."""
import os

import numpy as np
import pytest

import oracle
from nttanafis_gb300.operands import operand, to_int

pytestmark = pytest.mark.gpu
MASK = (1 << 64) - 1
THREADS = os.cpu_count() or 1


def bound_of(bits: int) -> int:
    return (1 << bits) - 1 if bits < 64 else MASK


def signed_values(values, mx):
    """Magnitude below the bound, sign from each limb's top bit (src/tests/convolution.rs:101-115)."""
    out = []
    for v in values:
        v = int(v)
        m = v & mx
        out.append(((-m) & MASK) if v >> 63 else m)
    return np.array(out, dtype=np.uint64)


def test_failure_leaves_destination_untouched(gpu):
    ws = gpu.GpuMulWorkspace()
    a, b = operand(100, 1), operand(50, 2)
    dst = np.full(149, MASK, dtype=np.uint64)  # one limb short
    assert not ws.mul(dst, a, b)
    assert np.all(dst == MASK)
    assert not ws.sqr(np.full(199, MASK, dtype=np.uint64), a)
    big = operand(1 << 25, 3)
    d2 = np.full(2, 7, dtype=np.uint64)
    assert not ws.mul(d2, big, operand(2, 1)) and np.all(d2 == 7)  # no plan
    ws.close()


def test_empty_operands_write_zero(gpu):
    # src/plan.rs:183-192
    ws = gpu.GpuMulWorkspace()
    dst = np.full(6, MASK, dtype=np.uint64)
    empty = np.zeros(0, dtype=np.uint64)
    assert ws.mul(dst, empty, operand(4, 1))
    assert np.all(dst[:4] == 0) and np.all(dst[4:] == MASK)
    assert not ws.mul(np.full(3, MASK, dtype=np.uint64), empty, operand(4, 1))
    assert ws.sqr(dst, empty) and dst[4] == MASK
    ws.close()


def test_alias_equals_distinct_copies(gpu):
    ws = gpu.GpuMulWorkspace()
    a = operand(3000, 9)
    copy = a.copy()
    assert np.array_equal(
        (lambda d: (ws.mul(d, a, a), d)[1])(np.zeros(6000, dtype=np.uint64)),
        (lambda d: (ws.mul(d, a, copy), d)[1])(np.zeros(6000, dtype=np.uint64)))
    ws.close()


def test_retained_workspace_serves_shapes_in_any_order(gpu):
    # src/tests/products.rs:203-217
    ws = gpu.GpuMulWorkspace()
    rng = np.random.default_rng(5)
    shapes = [(300, 300), (1, 1), (20000, 20000), (7, 300), (70000, 3), (128, 128), (1, 300), (5000, 4999)]
    plan = gpu.MulPlan.new(*shapes[0])
    assert ws.prepare(plan)
    for la, lb in shapes + shapes[::-1]:
        a = rng.integers(0, 2**64, la, dtype=np.uint64)
        b = rng.integers(0, 2**64, lb, dtype=np.uint64)
        dst = np.full(la + lb, MASK, dtype=np.uint64)
        assert ws.mul(dst, a, b)
        assert np.array_equal(dst, oracle.mul(a, b, THREADS)), (la, lb)
    ws.close()


@pytest.fixture(scope="module")
def cws(gpu):
    w = gpu.GpuConvWorkspace()
    yield w
    w.close()


def conv_gpu(gpu, cws, a, b, ma, mb, signed):
    plan = gpu.ConvPlan.new(a.size, b.size, ma, mb, signed)
    assert plan is not None
    assert cws.prepare(plan)
    dst = np.full(plan.output_len() + 2, MASK, dtype=np.uint64)
    assert cws.convolve(dst, a, b), gpu.last_error()
    assert dst[-1] == MASK and dst[-2] == MASK
    return dst[:plan.output_len()]


def test_conv_example_and_suffix(gpu, cws, golden):
    ex = golden["conv_example"]
    a = np.array(ex["a"], dtype=np.uint64)
    b = np.array(ex["b"], dtype=np.uint64)
    plan = gpu.ConvPlan.new(3, 2, 7, 7, False)
    assert cws.prepare(plan)
    dst = np.full(6, MASK, dtype=np.uint64)
    assert cws.convolve(dst, a, b)
    assert dst.tolist() == ex["expected"] + [MASK, MASK]


def test_golden_convolutions(gpu, cws, golden):
    for case in golden["convolutions"]["cases"]:
        a = np.array([int(v, 16) for v in case["a"]], dtype=np.uint64)
        b = np.array([int(v, 16) for v in case["b"]], dtype=np.uint64)
        mx = bound_of(case["bits"])
        got = conv_gpu(gpu, cws, a, b, mx, mx, case["signed"])
        stride = gpu.ConvPlan.new(a.size, b.size, mx, mx, case["signed"]).stride()
        for k, v in enumerate(case["coefficients"]):
            assert to_int(got[k * stride:(k + 1) * stride]) == int(v) % (1 << (64 * stride))


def test_conv_all_bounds_and_shapes_match_oracle(gpu, cws):
    # src/tests/convolution.rs:136-157 ranges: 1..=70 coefficients, every width
    rng = np.random.default_rng(21)
    for _ in range(160):
        la, lb = int(rng.integers(1, 71)), int(rng.integers(1, 71))
        ba, bb = int(rng.integers(0, 65)), int(rng.integers(0, 65))
        ma, mb = bound_of(ba), bound_of(bb)
        a = rng.integers(0, 2**64, la, dtype=np.uint64) & np.uint64(ma)
        b = rng.integers(0, 2**64, lb, dtype=np.uint64) & np.uint64(mb)
        assert np.array_equal(conv_gpu(gpu, cws, a, b, ma, mb, False), oracle.conv(a, b, ma, mb)), (la, lb, ba, bb)


def test_signed_conv_matches_oracle(gpu, cws):
    rng = np.random.default_rng(22)
    for _ in range(120):
        la, lb = int(rng.integers(1, 71)), int(rng.integers(1, 71))
        ba, bb = int(rng.integers(0, 64)), int(rng.integers(0, 64))
        ma, mb = bound_of(ba), bound_of(bb)
        a = signed_values(rng.integers(0, 2**64, la, dtype=np.uint64), ma)
        b = signed_values(rng.integers(0, 2**64, lb, dtype=np.uint64), mb)
        assert np.array_equal(conv_gpu(gpu, cws, a, b, ma, mb, True), oracle.conv(a, b, ma, mb, True)), (la, lb)


def test_signed_extremes_and_saturated_bounds(gpu, cws):
    # src/tests/convolution.rs:186-209 and :374-407
    for la, lb in [(1, 1), (8, 8), (24, 100), (25, 25), (33, 33), (1000, 25), (2048, 64)]:
        for ba, bb in [(0, 0), (1, 1), (63, 1), (63, 63)]:
            ma, mb = bound_of(ba), bound_of(bb)
            neg_a = np.full(la, (-ma) & MASK, dtype=np.uint64)
            neg_b = np.full(lb, (-mb) & MASK, dtype=np.uint64)
            assert np.array_equal(conv_gpu(gpu, cws, neg_a, neg_b, ma, mb, True),
                                  oracle.conv(neg_a, neg_b, ma, mb, True))
            alt = np.array([ma if i % 2 == 0 else (-ma) & MASK for i in range(la)], dtype=np.uint64)
            assert np.array_equal(conv_gpu(gpu, cws, alt, neg_b, ma, mb, True),
                                  oracle.conv(alt, neg_b, ma, mb, True))
        for ba, bb in [(0, 0), (32, 32), (32, 64), (64, 1), (64, 64)]:
            ma, mb = bound_of(ba), bound_of(bb)
            a = np.full(la, ma, dtype=np.uint64)
            b = np.full(lb, mb, dtype=np.uint64)
            assert np.array_equal(conv_gpu(gpu, cws, a, b, ma, mb, False), oracle.conv(a, b, ma, mb))


def test_conv_rejections_leave_destination(gpu):
    # src/tests/convolution.rs:310-350
    for la, lb in [(3, 2), (30, 30)]:
        w = gpu.GpuConvWorkspace()
        a, b = np.full(la, 7, dtype=np.uint64), np.full(lb, 7, dtype=np.uint64)
        plan = gpu.ConvPlan.new(la, lb, 7, 7, False)
        untouched = np.full(plan.output_len() + 1, MASK, dtype=np.uint64)
        assert not w.convolve(untouched, a, b)  # no plan prepared
        assert w.prepare(plan)
        above = a.copy()
        above[-1] = 8
        for x, y in [(a[1:], b), (a, b[1:]), (above, b)]:
            assert not w.convolve(untouched, x, y)
        assert not w.convolve(untouched[:plan.output_len() - 1], a, b)
        assert np.all(untouched == MASK)
        w.close()
    w = gpu.GpuConvWorkspace()
    plan = gpu.ConvPlan.new(4, 4, 3, 3, True)
    assert w.prepare(plan)
    dst = np.full(plan.output_len(), 7, dtype=np.uint64)
    beyond = np.array([1, MASK - 3, 0, 2], dtype=np.uint64)
    assert not w.convolve(dst, beyond, np.array([1, 2, 3, 0], dtype=np.uint64))
    assert np.all(dst == 7)
    w.close()


def test_conv_alias_and_large_shapes(gpu, cws):
    a = operand(5000, 3) & np.uint64(0xFFFF)
    assert np.array_equal(conv_gpu(gpu, cws, a, a, 0xFFFF, 0xFFFF, False),
                          conv_gpu(gpu, cws, a, a.copy(), 0xFFFF, 0xFFFF, False))
    # the served convolution classes at 1M coefficients: 16/32-bit unsigned, 32-bit signed
    n = 1 << 20
    for bits, signed in [(16, False), (32, False), (31, True)]:
        mx = bound_of(bits)
        if signed:
            a = signed_values(operand(n, 51), mx)
            b = signed_values(operand(n, 52), mx)
            mx = 1 << 31
        else:
            a = operand(n, 51) & np.uint64(mx)
            b = operand(n, 52) & np.uint64(mx)
        assert np.array_equal(conv_gpu(gpu, cws, a, b, mx, mx, signed),
                              oracle.conv(a, b, mx, mx, signed, THREADS)), (bits, signed)


@pytest.mark.parametrize("la,lb", [(4096, 3000), (2049, 2048), (6000, 2193), (8000, 193)])
def test_conv_single_transform_lengths_near_2_pow_13(gpu, cws, la, lb):
    # T = 2^12 (one CTA per prime) and T = 2^13 (four-step, 2^6-point columns, when
    # enqueued alone), at every coefficient class and sign
    for bits, signed in [(16, False), (32, False), (31, True), (64, False)]:
        mx = bound_of(bits)
        if signed:
            a, b = signed_values(operand(la, 61), mx), signed_values(operand(lb, 62), mx)
            mx = 1 << 31
        else:
            a, b = operand(la, 61) & np.uint64(mx), operand(lb, 62) & np.uint64(mx)
        assert np.array_equal(conv_gpu(gpu, cws, a, b, mx, mx, signed),
                              oracle.conv(a, b, mx, mx, signed, THREADS)), (la, lb, bits, signed)


def test_conv_device_paths(gpu):
    import torch

    la, lb, mx = 40000, 30000, (1 << 32) - 1
    a = operand(la, 61) & np.uint64(mx)
    b = operand(lb, 62) & np.uint64(mx)
    expected = oracle.conv(a, b, mx, mx, False, THREADS)
    plan = gpu.ConvPlan.new(la, lb, mx, mx, False)
    da = torch.from_numpy(a.view(np.int64)).cuda()
    db = torch.from_numpy(b.view(np.int64)).cuda()
    dst = torch.empty(plan.output_len(), dtype=torch.int64, device="cuda")
    scratch = torch.empty(plan.scratch_len(), dtype=torch.int64, device="cuda")
    stream = torch.cuda.current_stream()
    assert plan.convolve_device(dst, da, db, scratch, stream)
    torch.cuda.synchronize()
    assert np.array_equal(dst.cpu().numpy().view(np.uint64), expected)
    w = gpu.GpuConvWorkspace()
    assert w.prepare(plan)
    dst.zero_()
    assert w.convolve_device(dst, da, db, stream)
    torch.cuda.synchronize()
    assert np.array_equal(dst.cpu().numpy().view(np.uint64), expected)
    w.close()


def test_butterfly_probe_and_launch_counter(gpu):
    # the compute-ceiling probe runs (positive, plausible rate) and the launch
    # counter grows by the kernels a product enqueues
    from nttanafis_gb300 import probe

    rate = probe.butterfly_rate(152, 50)
    assert 1e11 < rate < 1e14
    for v in range(len(probe.VARIANTS)):
        assert probe.rate(v, 152, 20) > 1e9, probe.VARIANTS[v]
    import torch

    ws = gpu.GpuMulWorkspace()
    a = torch.from_numpy(operand(6000, 1).view(np.int64)).cuda()
    b = torch.from_numpy(operand(6000, 2).view(np.int64)).cuda()
    assert gpu.MulPlan.new(6000, 6000).blocks == 0
    dst = torch.empty(12000, dtype=torch.int64, device="cuda")
    assert ws.mul_device(dst, a, b)
    before = gpu.kernel_launches()
    assert ws.mul_device(dst, a, b)
    assert gpu.kernel_launches() - before == 4  # column, row, inverse column, CRT
    torch.cuda.synchronize()
    ws.close()
