"""Seeded operands with the reference benchmarks' distribution.

SplitMix64 (Steele, Lea and Flood 2014), as bench/src/lib.rs:13-29 of the
reference uses it: `operand(len, seed)` returns `len` uniformly distributed
64-bit limbs. Vectorised with numpy's wrapping uint64 arithmetic.
"""
from __future__ import annotations

import numpy as np

_GAMMA = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def operand(length: int, seed: int) -> np.ndarray:
    """Returns `length` SplitMix64 limbs of stream `seed` as a uint64 array."""
    with np.errstate(over="ignore"):
        idx = np.arange(1, length + 1, dtype=np.uint64)
        state = np.uint64(seed) + idx * _GAMMA
        z = state
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def sparse_operand(length: int, keep_seed: int = 3, value_seed: int = 4, per: int = 100) -> np.ndarray:
    """Operand whose limb i is nonzero iff stream `keep_seed` gives 0 mod `per`;
    nonzero values come from stream `value_seed` (forced odd so they are nonzero)."""
    keep = operand(length, keep_seed) % np.uint64(per) == 0
    vals = operand(length, value_seed) | np.uint64(1)
    return np.where(keep, vals, np.uint64(0)).astype(np.uint64)


def to_int(limbs: np.ndarray) -> int:
    """Integer value of little-endian uint64 limbs."""
    return int.from_bytes(np.ascontiguousarray(limbs, dtype="<u8").tobytes(), "little")


def from_int(value: int, length: int) -> np.ndarray:
    """`length` little-endian uint64 limbs of a nonnegative integer."""
    return np.frombuffer(value.to_bytes(8 * length, "little"), dtype="<u8").astype(np.uint64)
