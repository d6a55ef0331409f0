"""Batched modular arithmetic in 50-bit prime fields on device arrays: the
PrimeField / CrtPair API of ntt_anafis (src/field/prime_field.rs) over CUDA
tensors of residues, one call per array operation.

A field is named by its modulus, a prime 2^49 < p < 2^50. Residues are int64
CUDA tensors holding canonical values 0 <= r < p (the uint64 bit patterns);
residues of another field give unspecified values, as in the reference.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import Iterator, Optional

from .api import _dev, _stream_handle, last_error, library

_ADD, _SUB, _MUL = 0, 1, 2
_NEG, _POW, _INV, _SIGNED, _REDUCE, _REDUCE_U64 = 0, 1, 2, 3, 4, 5


def mul_method(method: Optional[int] = None) -> int:
    """The product method of the field calls: 1 FP64 quotient estimate (the
    reference's), 0 Barrett; sets it when given and returns the previous one."""
    return int(library().ntt_field_mul_method(-1 if method is None else method))


def _check(ok: int) -> None:
    if not ok:
        raise RuntimeError(last_error())


@dataclass(frozen=True)
class PrimeField:
    """Z/pZ for a prime 2^49 < p < 2^50 (PrimeField, src/field/prime_field.rs:34)."""

    modulus: int

    @staticmethod
    def new(modulus: int) -> Optional["PrimeField"]:
        """The field of `modulus`, or None unless it is an admitted prime (:99)."""
        if not 0 <= modulus < 1 << 64:
            return None
        return PrimeField(modulus) if library().ntt_field_check(modulus) else None

    @staticmethod
    def below(bound: int) -> Optional["PrimeField"]:
        """The largest admitted prime below min(bound, 2^50), or None (:118)."""
        p = library().ntt_field_below(min(max(bound, 0), (1 << 64) - 1))
        return PrimeField(p) if p else None

    @staticmethod
    def catalog() -> Iterator["PrimeField"]:
        """The transform's catalog fields in reconstruction order (:131)."""
        n = library().ntt_field_catalog(None, 0)
        buf = (ctypes.c_uint64 * n)()
        library().ntt_field_catalog(buf, n)
        return iter([PrimeField(int(p)) for p in buf])

    def _binary(self, op: int, out, a, b, stream) -> None:
        po, n = _dev(out)
        pa, na = _dev(a)
        pb, nb = _dev(b)
        if not n == na == nb:
            raise ValueError("arrays differ in length")
        _check(library().ntt_field_binary_device(self.modulus, op, po, pa, pb, n, _stream_handle(stream)))

    def _unary(self, op: int, out, a, exponent: int = 0, mask=None, stream=None) -> None:
        po, n = _dev(out)
        pa, na = _dev(a)
        if n != na:
            raise ValueError("arrays differ in length")
        pm = 0
        if mask is not None:
            if mask.element_size() != 1 or mask.numel() != n or not mask.is_cuda or not mask.is_contiguous():
                raise TypeError("mask must be a contiguous uint8 CUDA tensor of the same length")
            pm = int(mask.data_ptr())
        _check(library().ntt_field_unary_device(self.modulus, op, po, pa, n, exponent, pm, _stream_handle(stream)))

    def add(self, out, a, b, stream=None) -> None:
        """out = a + b (:205)."""
        self._binary(_ADD, out, a, b, stream)

    def sub(self, out, a, b, stream=None) -> None:
        """out = a - b (:215)."""
        self._binary(_SUB, out, a, b, stream)

    def mul(self, out, a, b, stream=None) -> None:
        """out = a * b (:232)."""
        self._binary(_MUL, out, a, b, stream)

    def neg(self, out, a, stream=None) -> None:
        """out = -a (:225)."""
        self._unary(_NEG, out, a, stream=stream)

    def pow(self, out, base, exponent: int, stream=None) -> None:
        """out = base^exponent with 0^0 = 1 (:249)."""
        self._unary(_POW, out, base, exponent, stream=stream)

    def inv(self, out, a, mask=None, stream=None) -> None:
        """out = a^-1; zero gives 0 and mask 0 where a mask is given (:271)."""
        self._unary(_INV, out, a, mask=mask, stream=stream)

    def signed(self, out, a, stream=None) -> None:
        """out = the representative in -(p-1)/2..(p-1)/2, as int64 (:193)."""
        self._unary(_SIGNED, out, a, stream=stream)

    def reduce(self, out, values, stream=None) -> None:
        """out = values mod p for int64 values (:158)."""
        self._unary(_REDUCE, out, values, stream=stream)

    def reduce_u64(self, out, values, stream=None) -> None:
        """out = values mod p for the uint64 bit patterns of values (:173)."""
        self._unary(_REDUCE_U64, out, values, stream=stream)

    def scale(self, target, factor: int, stream=None) -> None:
        """target = factor * target (:304)."""
        pt, n = _dev(target)
        _check(library().ntt_field_scale_device(self.modulus, pt, 0, n, factor, _stream_handle(stream)))

    def mul_sub(self, target, source, factor: int, stream=None) -> None:
        """target = target - factor * source over equal lengths (:296)."""
        pt, n = _dev(target)
        ps, ns = _dev(source)
        if n != ns:
            raise ValueError("arrays differ in length")
        _check(library().ntt_field_scale_device(self.modulus, pt, ps, n, factor, _stream_handle(stream)))

    def evaluate(self, out, coefficients, points, stream=None) -> None:
        """out[j] = sum_i coefficients[i] * points[j]^i (:313, at many points)."""
        po, n = _dev(out)
        pc, nc = _dev(coefficients)
        pp, npts = _dev(points)
        if n != npts:
            raise ValueError("out and points differ in length")
        _check(library().ntt_field_evaluate_device(self.modulus, po, pc, nc, pp, n, _stream_handle(stream)))


@dataclass(frozen=True)
class CrtPair:
    """Chinese remaindering over two distinct fields (CrtPair, prime_field.rs:63)."""

    first: PrimeField
    second: PrimeField

    @staticmethod
    def new(first: PrimeField, second: PrimeField) -> Optional["CrtPair"]:
        """The pair, or None when the fields coincide (:407)."""
        return None if first.modulus == second.modulus else CrtPair(first, second)

    def modulus(self) -> int:
        return self.first.modulus * self.second.modulus

    def combine(self, out, first, second, stream=None) -> None:
        """out[2i], out[2i+1] = low and high words of the int128 congruent to
        first[i] and second[i] in -(M-1)/2..(M-1)/2 (:428)."""
        po, n2 = _dev(out)
        pa, n = _dev(first)
        pb, nb = _dev(second)
        if n != nb or n2 != 2 * n:
            raise ValueError("out must hold two words per element")
        _check(library().ntt_crt_pair_combine_device(self.first.modulus, self.second.modulus, po, pa, pb, n,
                                                     _stream_handle(stream)))
