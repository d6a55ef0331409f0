"""The oracle (C restatement of the reference algorithm) against the reference's
known answers and against independent Python-integer products."""
import numpy as np
import pytest

import oracle
from nttanafis_gb300.operands import operand, to_int

MASK = (1 << 64) - 1


def hexlimbs(values):
    return np.array([int(v, 16) for v in values], dtype=np.uint64)


def test_capacities_match_reference_property(golden):
    assert [oracle.capacity(c) for c in range(1, 9)] == golden["capacities"]["bits"]


def test_row_shapes_match_reference_table(golden):
    # for_residues at 8-bit values: the reference's rows for each shape
    for la, lb, t, c, tab in golden["row_shapes"]["cases"]:
        plan = oracle.conv_plan(la, lb, 255, 255, False)
        assert oracle.row_shape(la + lb - 1, max(la, lb)) == (t, c, tab), (la, lb)
        assert plan is not None


def test_strides_match_reference_table(golden):
    for terms, ma, mb, stride in golden["strides"]["cases"]:
        assert oracle.conv_plan(terms, terms, ma, mb, False)["stride"] == stride


def test_geometry_at_benchmark_shapes(golden):
    for case in golden["geometry"]["cases"]:
        plan = oracle.mul_plan(case["la"], case["lb"], 1)
        for key in ("primes", "chunk_bits", "digits_a", "conv_len", "transform_len"):
            assert plan[key] == case[key], (case, plan)


def test_conv_example(golden):
    ex = golden["conv_example"]
    a = np.array(ex["a"], dtype=np.uint64)
    b = np.array(ex["b"], dtype=np.uint64)
    assert oracle.conv(a, b, 3, 5).tolist() == ex["expected"]


def test_rejections(golden):
    for la, lb in golden["rejections"]["mul_none"]:
        assert oracle.mul_plan(la, lb) is None
    for la, lb, ma, mb, s in golden["rejections"]["conv_none"]:
        assert oracle.conv_plan(la, lb, ma, mb, bool(s)) is None
    sb = golden["rejections"]["signed_beyond"]
    a = np.array(sb["a"], dtype=np.uint64)
    b = np.array(sb["b"], dtype=np.uint64)
    assert oracle.conv(a, b, sb["max"], sb["max"], True) is None


def test_products_match_python_integers(golden):
    for case in golden["products"]["cases"]:
        a, b = operand(case["la"], case["seed_a"]), operand(case["lb"], case["seed_b"])
        got = oracle.mul(a, b)
        if "product" in case:
            assert np.array_equal(got, hexlimbs(case["product"])), (case["la"], case["lb"])
        import hashlib

        assert hashlib.sha256(got.astype("<u8").tobytes()).hexdigest() == case["sha256"]


def test_squares_match_python_integers(golden):
    for case in golden["squares"]["cases"]:
        a = operand(case["la"], case["seed"])
        assert np.array_equal(oracle.sqr(a), hexlimbs(case["square"]))


def test_convolutions_match_python_integers(golden):
    for case in golden["convolutions"]["cases"]:
        a, b = hexlimbs(case["a"]), hexlimbs(case["b"])
        mx = (1 << case["bits"]) - 1 if case["bits"] < 64 else MASK
        got = oracle.conv(a, b, mx, mx, case["signed"])
        stride = oracle.conv_plan(a.size, b.size, mx, mx, case["signed"])["stride"]
        for k, v in enumerate(case["coefficients"]):
            block = to_int(got[k * stride:(k + 1) * stride])
            assert block == int(v) % (1 << (64 * stride)), (case["la"], case["lb"], k)


def test_schoolbook_and_splitmix():
    a, b = operand(50, 1), operand(37, 2)
    assert np.array_equal(oracle.operand(50, 1), a)
    assert to_int(oracle.schoolbook(a, b)) == to_int(a) * to_int(b)


@pytest.mark.parametrize("la,lb", [(1, 40), (40, 1), (17, 23), (256, 256), (2000, 30), (5000, 300)])
def test_random_shapes_and_threads(la, lb):
    rng = np.random.default_rng(la * 7919 + lb)
    a = rng.integers(0, 2**64, la, dtype=np.uint64)
    b = rng.integers(0, 2**64, lb, dtype=np.uint64)
    exact = to_int(a) * to_int(b)
    for threads in (1, 4):
        assert to_int(oracle.mul(a, b, threads)) == exact


def test_all_ones_closed_form():
    # (B^l - 1)(B^r - 1), src/tests/scheduling.rs:35-45
    for la, lb in [(4096, 64), (5000, 300), (3000, 1)]:
        a = np.full(la, MASK, dtype=np.uint64)
        b = np.full(lb, MASK, dtype=np.uint64)
        assert to_int(oracle.mul(a, b)) == ((1 << (64 * la)) - 1) * ((1 << (64 * lb)) - 1)


def test_every_prefix_at_capacity():
    # src/tests/convolution.rs:244-281: a bound at each capacity selects that prefix
    for count in range(1, 9):
        cap = oracle.capacity(count)
        # max_a * max_b * terms with bit length exactly cap: terms=1, max_a=2^(cap//2)... use 64-bit bounds
        if cap <= 128:
            ma = (1 << min(64, cap - 64)) - 1 if cap > 64 else (1 << cap) - 1
            mb = (1 << 64) - 1 if cap > 64 else 1
            plan = oracle.conv_plan(1, 1, ma, mb, False)
            assert plan["primes"] <= count


def test_cache_blocked_transforms_equal_radix_2():
    # the timed CPU path's transforms (cache-blocked, radix-4 above the block, lazy
    # centred residues) against the plain radix-2 ones, bit for bit, across the
    # block boundary and for every catalog prime
    for prime in range(8):
        for log_n in (1, 2, 5, 11, 12, 13, 14, 15, 17):
            assert oracle.transform_check(prime, log_n, 7 + prime + log_n), (prime, log_n)
