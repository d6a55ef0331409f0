"""Bit-exact parity of the CUDA path (through the C ABI) with the oracle, the
golden Python-integer products, and modular fingerprints at full sizes."""
import hashlib
import os

import numpy as np
import pytest

import oracle
from nttanafis_gb300.operands import operand, sparse_operand, to_int

pytestmark = pytest.mark.gpu
MASK = (1 << 64) - 1
FINGERPRINT_PRIMES = [(1 << 61) - 1, (1 << 89) - 1, (1 << 107) - 1, (1 << 127) - 1]
THREADS = os.cpu_count() or 1


def hexlimbs(values):
    return np.array([int(v, 16) for v in values], dtype=np.uint64)


def all_ones_expected(la: int, lb: int) -> np.ndarray:
    """Limbs of (B^la - 1)(B^lb - 1), src/tests/scheduling.rs:35-45."""
    left, right = max(la, lb), min(la, lb)
    out = np.zeros(la + lb, dtype=np.uint64)
    out[0] = 1
    out[right:] = MASK
    out[left] = MASK - 1
    return out


def fingerprint_ok(a, b, c) -> bool:
    A, B, C = to_int(a), to_int(b), to_int(c)
    return all((A % q) * (B % q) % q == C % q for q in FINGERPRINT_PRIMES)


@pytest.fixture(scope="module")
def ws(gpu):
    w = gpu.GpuMulWorkspace()
    yield w
    w.close()


@pytest.fixture
def transforms_only(gpu):
    """Short products through the transforms (the basecase off), so that the
    one-CTA and fused transform kernels stay covered at every size."""
    previous = gpu.set_basecase_limit(0)
    yield
    gpu.set_basecase_limit(previous)


def gpu_mul(ws, a, b, extra=2):
    dst = np.full(a.size + b.size + extra, MASK, dtype=np.uint64)
    assert ws.mul(dst, a, b), "mul failed"
    assert np.all(dst[a.size + b.size:] == MASK), "suffix was overwritten"
    return dst[:a.size + b.size]


def gpu_sqr(ws, a):
    dst = np.full(2 * a.size + 1, MASK, dtype=np.uint64)
    assert ws.sqr(dst, a), "sqr failed"
    assert dst[-1] == MASK
    return dst[:2 * a.size]


def test_golden_products(ws, golden):
    for case in golden["products"]["cases"]:
        a, b = operand(case["la"], case["seed_a"]), operand(case["lb"], case["seed_b"])
        got = gpu_mul(ws, a, b)
        assert hashlib.sha256(got.astype("<u8").tobytes()).hexdigest() == case["sha256"], (case["la"], case["lb"])
        if "product" in case:
            assert np.array_equal(got, hexlimbs(case["product"]))


def test_golden_squares(ws, golden):
    for case in golden["squares"]["cases"]:
        a = operand(case["la"], case["seed"])
        assert np.array_equal(gpu_sqr(ws, a), hexlimbs(case["square"]))


@pytest.mark.parametrize("path", ["default", "transforms"])
def test_config_1024_mul_and_sqr_match_oracle(ws, gpu, path):
    previous = gpu.set_basecase_limit(0) if path == "transforms" else None
    try:
        a, b = operand(1024, 1), operand(1024, 2)
        assert np.array_equal(gpu_mul(ws, a, b), oracle.mul(a, b))
        assert np.array_equal(gpu_sqr(ws, a), oracle.sqr(a))
    finally:
        if previous is not None:
            gpu.set_basecase_limit(previous)


@pytest.mark.parametrize("path", ["default", "transforms"])
def test_small_shapes_every_length(ws, gpu, path):
    previous = gpu.set_basecase_limit(0) if path == "transforms" else None
    try:
        _small_shapes_every_length(ws)
    finally:
        if previous is not None:
            gpu.set_basecase_limit(previous)


def _small_shapes_every_length(ws):
    # proptest range of src/tests/products.rs:134-135: 1..=40 limbs each
    rng = np.random.default_rng(11)
    for la in range(1, 41):
        for lb in (1, 2, 7, 16, 33, 40):
            a = rng.integers(0, 2**64, la, dtype=np.uint64)
            b = rng.integers(0, 2**64, lb, dtype=np.uint64)
            assert np.array_equal(gpu_mul(ws, a, b), oracle.schoolbook(a, b)), (la, lb)
        assert np.array_equal(gpu_sqr(ws, a), oracle.schoolbook(a, a)), la


def test_unbalanced_either_order(ws):
    # src/tests/products.rs:180-201: 1..=40 short, 200..=1500 long, both orders
    rng = np.random.default_rng(12)
    for _ in range(24):
        short = rng.integers(0, 2**64, int(rng.integers(1, 41)), dtype=np.uint64)
        long = rng.integers(0, 2**64, int(rng.integers(200, 1501)), dtype=np.uint64)
        assert np.array_equal(gpu_mul(ws, long, short), oracle.mul(long, short))
        assert np.array_equal(gpu_mul(ws, short, long), oracle.mul(short, long))


@pytest.mark.parametrize("log_t", range(4, 14))
def test_fused_cluster_every_size(ws, transforms_only, log_t):
    # every single-product fused size (T = 2^4 .. 2^13): products that fill T,
    # squares, and all-ones operands whose carries run across every CRT tile
    half = 1 << (log_t - 1)
    a, b = operand(half, 31 + log_t), operand(half, 61 + log_t)
    assert np.array_equal(gpu_mul(ws, a, b), oracle.mul(a, b)), log_t
    assert np.array_equal(gpu_sqr(ws, a), oracle.sqr(a)), log_t
    ones = np.full(half, MASK, dtype=np.uint64)
    assert np.array_equal(gpu_mul(ws, ones, ones), all_ones_expected(half, half)), log_t
    assert np.array_equal(gpu_sqr(ws, ones), all_ones_expected(half, half)), log_t
    c = operand(half - 3, 91 + log_t)
    assert np.array_equal(gpu_mul(ws, a, c), oracle.mul(a, c)), log_t


@pytest.mark.parametrize("log_t", range(14, 24))
def test_every_four_step_split(ws, gpu, log_t):
    # every split T = R * C the kernels offer gives the same product and square
    lo, hi = gpu.split_range(log_t)
    n = 1 << (log_t - 1)
    a, b = operand(n, 71 + log_t), operand(n - 5, 72 + log_t)
    expected = oracle.mul(a, b, THREADS) if log_t <= 20 else None
    try:
        for r in range(lo, hi + 1):
            gpu.set_split(log_t, r)
            got = gpu_mul(ws, a, b)
            if expected is not None:
                assert np.array_equal(got, expected), (log_t, r)
            else:
                assert fingerprint_ok(a, b, got), (log_t, r)
            assert fingerprint_ok(a, a, gpu_sqr(ws, a)), (log_t, r)
    finally:
        gpu.set_split(log_t, 0)


def test_split_in_batches_and_convolutions(gpu):
    import torch

    from nttanafis_gb300.workloads import Shape

    # members with T = 2^18
    shapes = [Shape("mul", 140000, 100000, 1, 2), Shape("sqr", 100000, 100000, 3, 3),
              Shape("conv", 150000, 100000, 5, 6, bits=32, signed=True)]
    lo, hi = gpu.split_range(18)
    batch = gpu.GpuBatch()
    try:
        for r in range(lo, hi + 1):
            gpu.set_split(18, r)
            reqs, keep = [], []
            for s in shapes:
                a_h, b_h = s.operands()
                a = torch.from_numpy(a_h.view(np.int64)).cuda()
                b = a if s.kind == "sqr" else torch.from_numpy(b_h.view(np.int64)).cuda()
                d = torch.empty(s.out_len(), dtype=torch.int64, device="cuda")
                reqs.append(gpu.Request(d, a, b, "conv" if s.kind == "conv" else "mul", s.max_a, s.max_a, s.signed))
                keep.append((s, a_h, b_h, d))
            assert batch.run(reqs), gpu.last_error()
            torch.cuda.synchronize()
            for s, a_h, b_h, d in keep:
                got = d.cpu().numpy().view(np.uint64)
                if s.kind == "conv":
                    assert np.array_equal(got, oracle.conv(a_h, b_h, s.max_a, s.max_a, True, THREADS)), r
                else:
                    assert fingerprint_ok(a_h, b_h, got), (s, r)
    finally:
        gpu.set_split(18, 0)
        batch.close()


def test_split_tuner_keeps_results(ws, gpu):
    try:
        chosen = gpu.tune_splits(15, 19, reps=2)
        for t, r in chosen.items():
            lo, hi = gpu.split_range(t)
            assert lo <= r <= hi
        a, b = operand(1 << 18, 5), operand(1 << 18, 6)
        assert fingerprint_ok(a, b, gpu_mul(ws, a, b))
    finally:
        for t in range(15, 20):
            gpu.set_split(t, 0)


@pytest.mark.parametrize("la,lb", [(4096, 4096), (4097, 4096), (8192, 8191), (8193, 8192), (20000, 13000),
                                   (65536, 65536), (65536, 256), (131072, 131072), (300000, 250000),
                                   (1 << 20, 131072)])
def test_transform_classes_match_oracle(ws, la, lb):
    # crosses the one-CTA / four-step boundary (T = 2^13 / 2^14) and every split
    a, b = operand(la, 21), operand(lb, 22)
    assert np.array_equal(gpu_mul(ws, a, b), oracle.mul(a, b, THREADS)), (la, lb)


def test_config_1m_mul_and_sqr_match_oracle(ws):
    a, b = operand(1 << 20, 1), operand(1 << 20, 2)
    expected = oracle.mul(a, b, THREADS)
    assert np.array_equal(gpu_mul(ws, a, b), expected)
    assert np.array_equal(gpu_sqr(ws, a), oracle.sqr(a, THREADS))


def test_edge_operands_all_ones_and_sparse(ws):
    ones = np.full(1 << 20, MASK, dtype=np.uint64)
    assert np.array_equal(gpu_mul(ws, ones, ones), all_ones_expected(1 << 20, 1 << 20))
    a, b = sparse_operand(1 << 20, 3, 4), sparse_operand(1 << 20, 5, 6)
    assert np.array_equal(gpu_mul(ws, a, b), oracle.mul(a, b, THREADS))
    assert np.array_equal(gpu_sqr(ws, a), oracle.sqr(a, THREADS))
    z = np.zeros(5000, dtype=np.uint64)
    assert not np.any(gpu_mul(ws, z, operand(3000, 1)))


@pytest.mark.parametrize("la,lb", [(4096, 64), (4097, 64), (5000, 300), (8192, 25), (3000, 1), (1 << 17, 1 << 17)])
def test_all_ones_carries(ws, la, lb):
    # src/tests/products.rs:17-29 and the closed form of src/tests/scheduling.rs:35-45
    a = np.full(la, MASK, dtype=np.uint64)
    b = np.full(lb, MASK, dtype=np.uint64)
    assert np.array_equal(gpu_mul(ws, a, b), all_ones_expected(la, lb))
    assert np.array_equal(gpu_mul(ws, b, a), all_ones_expected(la, lb))


def test_wide_prime_class_2_pow_24(ws):
    # T = 2^24 runs on the primes below 2^31 (canonical arithmetic)
    a, b = operand(1 << 23, 31), operand((1 << 23) - 7, 32)
    assert fingerprint_ok(a, b, gpu_mul(ws, a, b))


def test_wide_block_split(ws, gpu):
    # blocks of 2^24-point transforms (wide primes) sharing the shorter operand's
    # spectrum: the 2^12-point column kernels in their one-operand spectrum mode;
    # blocks of 2^23 and 2^22 points on the wide primes: the 2^10-point ones
    for la, lb, log_t in [(40_000_000, 2_000_000, 24), (20_000_000, 1_500_000, 23), (12_000_000, 1_100_000, 22)]:
        plan = gpu.MulPlan.new(la, lb)
        assert plan.blocks > 1 and plan.log_transform == log_t and plan.primes == 5, (la, lb)
        a, b = operand(la, 33), operand(lb, 34)
        assert fingerprint_ok(a, b, gpu_mul(ws, a, b)), (la, lb)
        assert fingerprint_ok(a, b, gpu_mul(ws, b, a)), (la, lb)


def test_wide_class_in_a_batch(gpu):
    # T = 2^24 and T = 2^22 wide members beside a short one: the 2^12- and 2^10-point
    # column kernels of the wide arithmetic in batch mode
    import torch

    big_a, big_b = operand(1 << 23, 35), operand((1 << 23) - 7, 36)
    mid_a, mid_b = operand(1 << 21, 39), operand((1 << 21) - 5, 40)
    small_a, small_b = operand(3000, 37), operand(2000, 38)
    batch = gpu.GpuBatch()
    dev = [torch.from_numpy(x.view(np.int64)).cuda() for x in (big_a, big_b, mid_a, mid_b, small_a, small_b)]
    dsts = [torch.full((x.size + y.size + 1,), -1, dtype=torch.int64, device="cuda")
            for x, y in ((big_a, big_b), (mid_a, mid_b), (small_a, small_b))]
    reqs = [gpu.Request(dsts[i], dev[2 * i], dev[2 * i + 1]) for i in range(3)]
    assert batch.run(reqs, torch.cuda.current_stream()), gpu.last_error()
    torch.cuda.synchronize()
    big, mid, small = (d.cpu().numpy().view(np.uint64) for d in dsts)
    assert big[-1] == MASK and mid[-1] == MASK and small[-1] == MASK
    assert fingerprint_ok(big_a, big_b, big[:-1])
    assert np.array_equal(mid[:-1], oracle.mul(mid_a, mid_b, THREADS))
    assert np.array_equal(small[:-1], oracle.mul(small_a, small_b, THREADS))
    assert batch.status() == 0
    batch.close()


def test_config_16m_mul_and_sqr_exact(ws, golden):
    # bit-exact against the oracle's digests (tests/golden/make_big_digests.py),
    # with the Mersenne fingerprints as a second, independent check
    cases = {c["kind"]: c for c in golden["big_products"]["cases"]}
    a, b = operand(1 << 24, 1), operand(1 << 24, 2)
    c = gpu_mul(ws, a, b, extra=1)
    assert hashlib.sha256(c.astype("<u8").tobytes()).hexdigest() == cases["mul"]["sha256"]
    assert fingerprint_ok(a, b, c)
    s = gpu_sqr(ws, a)
    assert hashlib.sha256(s.astype("<u8").tobytes()).hexdigest() == cases["sqr"]["sha256"]
    assert fingerprint_ok(a, a, s)


def test_16m_all_ones(ws):
    n = 1 << 24
    ones = np.full(n, MASK, dtype=np.uint64)
    assert np.array_equal(gpu_mul(ws, ones, ones, extra=0), all_ones_expected(n, n))


def test_device_and_plan_scratch_paths(gpu):
    import torch

    la, lb = 70000, 50000
    a, b = operand(la, 41), operand(lb, 42)
    expected = oracle.mul(a, b, THREADS)
    da = torch.from_numpy(a.view(np.int64)).cuda()
    db = torch.from_numpy(b.view(np.int64)).cuda()
    dst = torch.full((la + lb + 3,), -1, dtype=torch.int64, device="cuda")
    plan = gpu.MulPlan.new(la, lb)
    scratch = torch.empty(plan.scratch_len(), dtype=torch.int64, device="cuda")
    stream = torch.cuda.current_stream()
    assert plan.mul_device(dst, da, db, scratch, stream)
    torch.cuda.synchronize()
    host = dst.cpu().numpy().view(np.uint64)
    assert np.array_equal(host[:la + lb], expected) and np.all(host[la + lb:] == MASK)
    # square through the plan with its smaller scratch
    sq_plan = gpu.MulPlan.new(la, la)
    sq_scratch = torch.empty(sq_plan.sqr_scratch_len(), dtype=torch.int64, device="cuda")
    sq = torch.empty(2 * la, dtype=torch.int64, device="cuda")
    assert sq_plan.sqr_device(sq, da, sq_scratch, stream)
    torch.cuda.synchronize()
    assert np.array_equal(sq.cpu().numpy().view(np.uint64), oracle.sqr(a, THREADS))
    # workspace device path, aliasing the same tensor squares it
    w = gpu.GpuMulWorkspace()
    sq.fill_(0)
    assert w.mul_device(sq, da, da, stream)
    torch.cuda.synchronize()
    assert np.array_equal(sq.cpu().numpy().view(np.uint64), oracle.sqr(a, THREADS))
    # short scratch is rejected before any write
    dst.fill_(-1)
    assert not plan.mul_device(dst, da, db, scratch[:-1], stream)
    torch.cuda.synchronize()
    assert bool((dst == -1).all())
    w.close()


@pytest.mark.parametrize("la,lb", [(1 << 20, 1024), (1024, 1 << 20), (1 << 20, 3001), (600000, 1000), (1 << 20, 300),
                                   (524288, 512), (1 << 20, 131072)])
def test_block_split_matches_oracle(ws, gpu, la, lb):
    # the longer operand in blocks times the shorter one, whose spectrum every block
    # shares (one-CTA block transforms at 2^11..2^13, four-step ones from 2^15),
    # block sums added with carries
    assert gpu.MulPlan.new(la, lb).blocks > 1
    a, b = operand(la, 51), operand(lb, 52)
    assert np.array_equal(gpu_mul(ws, a, b), oracle.mul(a, b, THREADS)), (la, lb)


def test_block_split_all_ones(ws, gpu):
    # every block sum carries through the whole odd-block addition
    for la, lb in [(1 << 20, 1000), ((1 << 20) + 7, 1500)]:
        assert gpu.MulPlan.new(la, lb).blocks > 1
        a = np.full(la, MASK, dtype=np.uint64)
        b = np.full(lb, MASK, dtype=np.uint64)
        assert np.array_equal(gpu_mul(ws, a, b), all_ones_expected(la, lb))


def test_block_split_beyond_one_transform(ws, gpu):
    # a + b - 1 > 2^25: no single transform holds it, the split does
    la, lb = (1 << 25) + 12345, 3000
    plan = gpu.MulPlan.new(la, lb)
    assert plan is not None and plan.blocks > 1
    a, b = operand(la, 61), operand(lb, 62)
    assert fingerprint_ok(a, b, gpu_mul(ws, b, a, extra=1))


def test_block_split_plan_scratch(gpu):
    import torch

    la, lb = 1 << 20, 2000
    plan = gpu.MulPlan.new(la, lb)
    assert plan.blocks > 1
    a, b = operand(la, 71), operand(lb, 72)
    da = torch.from_numpy(a.view(np.int64)).cuda()
    db = torch.from_numpy(b.view(np.int64)).cuda()
    dst = torch.full((la + lb + 2,), -1, dtype=torch.int64, device="cuda")
    scratch = torch.empty(plan.scratch_len(), dtype=torch.int64, device="cuda")
    stream = torch.cuda.current_stream()
    assert plan.mul_device(dst, da, db, scratch, stream)
    torch.cuda.synchronize()
    host = dst.cpu().numpy().view(np.uint64)
    assert np.array_equal(host[:la + lb], oracle.mul(a, b, THREADS)) and np.all(host[la + lb:] == MASK)
    dst.fill_(-1)
    assert not plan.mul_device(dst, da, db, scratch[:-1], stream)
    torch.cuda.synchronize()
    assert bool((dst == -1).all())


def test_no_lookback_timeouts(gpu):
    # every bounded look-back wait of the CRT carry scan completed
    assert gpu.lookback_timeouts() == 0


def test_concurrent_host_calls_and_streams(gpu):
    # several host threads on their own workspaces (the copy-out result path that
    # concurrent host-pointer calls take) and products on two streams at once
    import threading

    import torch

    shapes = [(70000, 50000), (1 << 16, 1 << 16), (30000, 3), (4096, 4096), (200000, 3001), (1 << 20, 1 << 20)]
    expected = {s: oracle.mul(operand(s[0], 81 + i), operand(s[1], 91 + i), THREADS) for i, s in enumerate(shapes)}
    errors = []

    def worker(t):
        w = gpu.GpuMulWorkspace()
        try:
            for r in range(3):
                for i, (la, lb) in enumerate(shapes[t::2]):
                    k = shapes.index((la, lb))
                    a, b = operand(la, 81 + k), operand(lb, 91 + k)
                    dst = torch.empty(la + lb, dtype=torch.int64).pin_memory().numpy().view(np.uint64)
                    if not w.mul(dst, a, b) or not np.array_equal(dst, expected[(la, lb)]):
                        errors.append((t, la, lb))
        finally:
            w.close()

    threads = [threading.Thread(target=worker, args=(t,)) for t in range(4)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    assert not errors, errors
    # device calls alternating on two streams with two workspaces
    wss = [gpu.GpuMulWorkspace() for _ in range(2)]
    sts = [torch.cuda.Stream() for _ in range(2)]
    outs = []
    for i, (la, lb) in enumerate(shapes * 2):
        k = shapes.index((la, lb))
        da = torch.from_numpy(operand(la, 81 + k).view(np.int64)).cuda()
        db = torch.from_numpy(operand(lb, 91 + k).view(np.int64)).cuda()
        out = torch.empty(la + lb, dtype=torch.int64, device="cuda")
        torch.cuda.synchronize()
        assert wss[i % 2].mul_device(out, da, db, sts[i % 2])
        outs.append(((la, lb), out, da, db))
    torch.cuda.synchronize()
    for (la, lb), out, _, _ in outs:
        assert np.array_equal(out.cpu().numpy().view(np.uint64), expected[(la, lb)]), (la, lb)
    for w in wss:
        w.close()


@pytest.mark.parametrize("log_t,lb", [(23, 1 << 19), (23, (1 << 19) + 1), (23, (1 << 20) + 1), (22, 1 << 20),
                                      (22, (1 << 20) + 1)])
def test_all_ones_at_the_lazy_wide_boundary(ws, gpu, log_t, lb):
    # 2^log_t points filled: a shorter operand of 2^19 limbs at 2^23 (2^20 at 2^22)
    # needs exactly the capacity of five lazy primes there (147, 148 bits); one limb
    # more takes five wide primes. All-ones operands give the largest coefficients
    # (closed form, src/tests/scheduling.rs:35-45).
    la = (1 << log_t) - lb
    plan = gpu.MulPlan.new(la, lb)
    assert plan.primes == 5 and plan.log_transform == log_t and plan.blocks == 0
    a = np.full(la, MASK, dtype=np.uint64)
    b = np.full(lb, MASK, dtype=np.uint64)
    assert np.array_equal(gpu_mul(ws, a, b), all_ones_expected(la, lb))


def test_wide_primes_at_2_pow_22_and_23(ws, gpu):
    # T = 2^22 and 2^23 with the shorter operand above 2^20 (2^19) limbs: five lazy
    # primes hold too few bits, five wide ones enough (canonical arithmetic on the
    # 2^10-point column kernels); exact against the oracle
    for la, lb in [(1 << 21, 1 << 21), (3 << 20, (1 << 21) + 3), (3_000_000, 1_500_000)]:
        plan = gpu.MulPlan.new(la, lb)
        assert plan.primes == 5 and plan.log_transform in (22, 23) and plan.blocks == 0, (la, lb)
        a, b = operand(la, 111), operand(lb, 112)
        assert np.array_equal(gpu_mul(ws, a, b), oracle.mul(a, b, THREADS)), (la, lb)
    ones = np.full(1 << 21, MASK, dtype=np.uint64)
    assert np.array_equal(gpu_mul(ws, ones, ones), all_ones_expected(1 << 21, 1 << 21))
    a = operand(3 << 20, 113)
    assert np.array_equal(gpu_sqr(ws, a), oracle.sqr(a, THREADS))


def test_poisoned_scratch_and_any_shape_order(gpu):
    # caller scratch full of ones (no kernel may rely on its contents), and one
    # workspace serving fused, four-step and split shapes in a shuffled order
    import torch

    shapes = [(3000, 2000), (70000, 50000), (600000, 1000), (1024, 1024), (5, 7), (1 << 17, 1 << 17), (40000, 300)]
    expected = {s: oracle.mul(operand(s[0], 121), operand(s[1], 122), THREADS) for s in shapes}
    stream = torch.cuda.current_stream()
    for la, lb in shapes:
        plan = gpu.MulPlan.new(la, lb)
        da = torch.from_numpy(operand(la, 121).view(np.int64)).cuda()
        db = torch.from_numpy(operand(lb, 122).view(np.int64)).cuda()
        scratch = torch.full((max(1, plan.scratch_len()),), -1, dtype=torch.int64, device="cuda")
        dst = torch.full((la + lb,), -1, dtype=torch.int64, device="cuda")
        assert plan.mul_device(dst, da, db, scratch, stream)
        torch.cuda.synchronize()
        assert np.array_equal(dst.cpu().numpy().view(np.uint64), expected[(la, lb)]), (la, lb)
    w = gpu.GpuMulWorkspace()
    rng = np.random.default_rng(5)
    for i in rng.permutation(len(shapes * 3)):
        la, lb = (shapes * 3)[i]
        dst = np.full(la + lb, MASK, dtype=np.uint64)
        assert w.mul(dst, operand(la, 121), operand(lb, 122))
        assert np.array_equal(dst, expected[(la, lb)]), (la, lb)
    w.close()
