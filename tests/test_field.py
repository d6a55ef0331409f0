"""Host side of the 50-bit prime-field API: admission (2^49 < p < 2^50, prime by
the reference's Miller-Rabin bases), below(), and the catalog
(src/field/prime_field.rs:91-138, src/field/catalog.rs:19-25,67-76)."""
import numpy as np
import pytest

import nttanafis_gb300 as ntt


def test_catalog_matches_reference(golden):
    assert [f.modulus for f in ntt.PrimeField.catalog()] == golden["catalog"]["primes"]
    for f in ntt.PrimeField.catalog():
        assert ntt.PrimeField.new(f.modulus) == f


def test_admission_matches_primality():
    sympy = pytest.importorskip("sympy")
    rng = np.random.default_rng(9)
    lo, hi = (1 << 49) + 1, (1 << 50) - 1
    for _ in range(400):
        p = int(rng.integers(lo, hi)) | 1
        assert (ntt.PrimeField.new(p) is not None) == bool(sympy.isprime(p)), p
    for p in (0, 1, 2, 3, 1 << 49, (1 << 49) + 1, 1 << 50, (1 << 50) + 1, 2**61 - 1, (1 << 64) - 1):
        assert ntt.PrimeField.new(p) is None or sympy.isprime(p) and (1 << 49) < p < (1 << 50)


def test_below():
    sympy = pytest.importorskip("sympy")
    assert ntt.PrimeField.below(1 << 50).modulus == sympy.prevprime(1 << 50)
    assert ntt.PrimeField.below(1 << 62).modulus == sympy.prevprime(1 << 50)
    c = ntt.PrimeField.catalog().__next__().modulus
    assert ntt.PrimeField.below(c + 1).modulus == c
    assert ntt.PrimeField.below(1 << 49) is None
    assert ntt.PrimeField.below(0) is None


def test_crt_pair_needs_distinct_fields():
    f1, f2 = list(ntt.PrimeField.catalog())[:2]
    assert ntt.CrtPair.new(f1, f1) is None
    assert ntt.CrtPair.new(f1, f2).modulus() == f1.modulus * f2.modulus
