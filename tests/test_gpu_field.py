"""Batched 50-bit prime-field arithmetic and CrtPair on the GPU against Python
integers (exact), over the catalog fields and the largest admitted prime, with
the reference's known answers (src/field/prime_field.rs:25-32,49-61 and
src/field/tests/prime_field.rs)."""
import numpy as np
import pytest

import nttanafis_gb300 as ntt

pytestmark = pytest.mark.gpu
MASK = (1 << 64) - 1


def fields():
    return list(ntt.PrimeField.catalog()) + [ntt.PrimeField.below(1 << 50)]


def dev(values):
    import torch

    arr = np.array([v & MASK for v in values], dtype=np.uint64)
    return torch.from_numpy(arr.view(np.int64)).cuda()


def host(t):
    import torch

    torch.cuda.synchronize()
    return [int(v) for v in t.cpu().numpy().view(np.uint64)]


def empty(n):
    import torch

    return torch.empty(n, dtype=torch.int64, device="cuda")


def residues(rng, p, n):
    edges = [0, 1, 2, p >> 1, (p >> 1) + 1, p - 1]
    return edges + [int(v) % p for v in rng.integers(0, 2**63, n - len(edges), dtype=np.int64)]


def test_known_answers():
    f = next(ntt.PrimeField.catalog())
    a, b, out = dev([100]), dev([25]), empty(1)
    f.add(out, a, b)
    assert host(out) == [125]
    f.mul(out, a, b)
    assert host(out) == [2500]
    f1, f2 = list(ntt.PrimeField.catalog())[:2]
    vals = [12345, -12345]
    r1, r2 = empty(2), empty(2)
    f1.reduce(r1, dev(vals))
    f2.reduce(r2, dev(vals))
    out = empty(4)
    ntt.CrtPair.new(f1, f2).combine(out, r1, r2)
    words = host(out)
    got = [(words[2 * i] | words[2 * i + 1] << 64) for i in range(2)]
    got = [g - (1 << 128) if g >> 127 else g for g in got]
    assert got == vals


@pytest.fixture(params=[0, 1], ids=["barrett", "fp64"])
def method(request):
    # both product methods (Barrett on integers, the reference's FP64 estimate)
    from nttanafis_gb300.field import mul_method

    previous = mul_method(request.param)
    yield request.param
    mul_method(previous)


@pytest.mark.parametrize("index", range(9))
def test_arithmetic_matches_integers(index, method):
    f = fields()[index]
    p = f.modulus
    rng = np.random.default_rng(100 + index)
    n = 4096
    A, B = residues(rng, p, n), residues(rng, p, n)[::-1]
    a, b, out = dev(A), dev(B), empty(n)
    f.add(out, a, b)
    assert host(out) == [(x + y) % p for x, y in zip(A, B)]
    f.sub(out, a, b)
    assert host(out) == [(x - y) % p for x, y in zip(A, B)]
    f.mul(out, a, b)
    assert host(out) == [x * y % p for x, y in zip(A, B)]
    f.neg(out, a)
    assert host(out) == [-x % p for x in A]
    for e in (0, 1, 2, 12345, p - 2, (1 << 64) - 1):
        f.pow(out, a, e)
        assert host(out) == [pow(x, e, p) for x in A], e
    import torch

    mask = torch.empty(n, dtype=torch.uint8, device="cuda")
    f.inv(out, a, mask)
    inv = host(out)
    m = mask.cpu().numpy()
    for x, y, k in zip(A, inv, m):
        assert (k == 1 and x * y % p == 1) or (k == 0 and x == 0 and y == 0)
    f.signed(out, a)
    s = [v - (1 << 64) if v >> 63 else v for v in host(out)]
    assert s == [x - p if x > p >> 1 else x for x in A]
    assert all(abs(v) <= (p - 1) >> 1 for v in s)
    raw = [int(v) for v in rng.integers(-(2**63), 2**63 - 1, n, dtype=np.int64)] + [-(2**63), 2**63 - 1, -1, 0]
    rv = dev(raw)
    out2 = empty(len(raw))
    f.reduce(out2, rv)
    assert host(out2) == [v % p for v in raw]
    f.reduce_u64(out2, rv)
    assert host(out2) == [(v & MASK) % p for v in raw]


@pytest.mark.parametrize("index", [0, 3, 8])
def test_slice_kernels(index, method):
    f = fields()[index]
    p = f.modulus
    rng = np.random.default_rng(7 + index)
    T, S = residues(rng, p, 3000), residues(rng, p, 3000)
    for factor in (0, 1, p - 1, p >> 1, int(rng.integers(0, p))):
        t = dev(T)
        f.scale(t, factor)
        assert host(t) == [x * factor % p for x in T]
        t = dev(T)
        f.mul_sub(t, dev(S), factor)
        assert host(t) == [(x - factor * y) % p for x, y in zip(T, S)]
    coeffs = residues(rng, p, 2500)  # crosses the 1024-coefficient chunks
    points = residues(rng, p, 700)
    out = empty(len(points))
    f.evaluate(out, dev(coeffs), dev(points))
    expect = []
    for x in points:
        v = 0
        for c in reversed(coeffs):
            v = (v * x + c) % p
        expect.append(v)
    assert host(out) == expect


def test_crt_pairs_recover_signed_integers():
    # src/field/tests/prime_field.rs: every pair of catalog fields (and the largest prime)
    rng = np.random.default_rng(21)
    vals = [int(v) for v in rng.integers(-(2**63), 2**63 - 1, 512, dtype=np.int64)] + [0, 1, -1, -(2**63)]
    fs = fields()
    for i, f1 in enumerate(fs):
        for f2 in fs[i + 1:]:
            r1, r2 = empty(len(vals)), empty(len(vals))
            f1.reduce(r1, dev(vals))
            f2.reduce(r2, dev(vals))
            out = empty(2 * len(vals))
            ntt.CrtPair.new(f1, f2).combine(out, r1, r2)
            w = host(out)
            got = [(w[2 * k] | w[2 * k + 1] << 64) for k in range(len(vals))]
            assert [g - (1 << 128) if g >> 127 else g for g in got] == vals, (f1.modulus, f2.modulus)


def test_rejections():
    f = next(ntt.PrimeField.catalog())
    a, out = dev([1, 2]), empty(2)
    with pytest.raises(RuntimeError):
        ntt.PrimeField(1 << 49).add(out, a, a)  # not an admitted modulus
    with pytest.raises(RuntimeError):
        f.scale(dev([1]), f.modulus)  # factor is not a residue
    with pytest.raises(ValueError):
        f.add(out, a, dev([1]))
