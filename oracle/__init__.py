"""ctypes binding of the oracle: TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs may use it,
as the checker or the timed CPU reference; the product never imports it.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .build import OUT, build

_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        l = ctypes.CDLL(str(OUT))
        vp, u64, i32 = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int
        l.oracle_mul.argtypes = [vp, vp, u64, vp, u64, i32]
        l.oracle_sqr.argtypes = [vp, vp, u64, i32]
        l.oracle_conv.argtypes = [vp, vp, u64, vp, u64, u64, u64, i32, i32]
        l.oracle_mul_plan.argtypes = [u64, u64, i32, vp]
        l.oracle_conv_plan.argtypes = [u64, u64, u64, u64, i32, vp]
        l.oracle_row_shape.argtypes = [u64, u64, vp]
        l.oracle_capacity.argtypes = [i32]
        l.oracle_schoolbook.argtypes = [vp, vp, u64, vp, u64]
        l.oracle_operand.argtypes = [vp, u64, u64]
        l.oracle_transform_check.argtypes = [i32, i32, u64]
        l.oracle_transform_check.restype = i32
        for name in ("oracle_mul", "oracle_sqr", "oracle_conv", "oracle_mul_plan", "oracle_conv_plan",
                     "oracle_row_shape", "oracle_capacity"):
            getattr(l, name).restype = i32
        l.oracle_schoolbook.restype = None
        l.oracle_operand.restype = None
        _lib = l
    return _lib


def _p(a: np.ndarray) -> int:
    return a.ctypes.data if a.size else 0


def default_threads() -> int:
    return os.cpu_count() or 1


def mul(a: np.ndarray, b: np.ndarray, threads: int = 1) -> np.ndarray:
    out = np.zeros(a.size + b.size, dtype=np.uint64)
    if not lib().oracle_mul(_p(out), _p(a), a.size, _p(b), b.size, threads):
        raise ValueError("no plan")
    return out


def sqr(a: np.ndarray, threads: int = 1) -> np.ndarray:
    out = np.zeros(2 * a.size, dtype=np.uint64)
    if not lib().oracle_sqr(_p(out), _p(a), a.size, threads):
        raise ValueError("no plan")
    return out


def conv(a: np.ndarray, b: np.ndarray, max_a: int, max_b: int, signed: bool = False,
         threads: int = 1) -> np.ndarray | None:
    plan = conv_plan(a.size, b.size, max_a, max_b, signed)
    if plan is None:
        return None
    out = np.zeros(plan["output_len"], dtype=np.uint64)
    if not lib().oracle_conv(_p(out), _p(a), a.size, _p(b), b.size, max_a, max_b, int(signed), threads):
        return None
    return out


def mul_plan(la: int, lb: int, crt_cost: int = 1) -> dict | None:
    out = np.zeros(8, dtype=np.int64)
    if not lib().oracle_mul_plan(la, lb, crt_cost, _p(out)):
        return None
    keys = ["primes", "chunk_bits", "digits_a", "digits_b", "conv_len", "transform_len", "cyclic_len", "table_len"]
    return dict(zip(keys, map(int, out)))


def conv_plan(la: int, lb: int, max_a: int, max_b: int, signed: bool = False) -> dict | None:
    out = np.zeros(8, dtype=np.int64)
    if not lib().oracle_conv_plan(la, lb, max_a, max_b, int(signed), _p(out)):
        return None
    keys = ["primes", "stride", "bound_bits", "schoolbook", "transform_len", "cyclic_len", "table_len",
            "output_len"]
    return dict(zip(keys, map(int, out)))


def row_shape(conv_len: int, longest: int) -> tuple[int, int, int]:
    out = np.zeros(3, dtype=np.uint64)
    lib().oracle_row_shape(conv_len, longest, _p(out))
    return tuple(int(x) for x in out)


def capacity(count: int) -> int:
    return int(lib().oracle_capacity(count))


def schoolbook(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    out = np.zeros(a.size + b.size, dtype=np.uint64)
    lib().oracle_schoolbook(_p(out), _p(a), a.size, _p(b), b.size)
    return out


def transform_check(prime: int, log_n: int, seed: int = 1) -> bool:
    """The cache-blocked transforms equal the radix-2 ones bit for bit."""
    return lib().oracle_transform_check(prime, log_n, seed) == 1


def operand(length: int, seed: int) -> np.ndarray:
    out = np.zeros(length, dtype=np.uint64)
    lib().oracle_operand(_p(out), length, seed)
    return out


def model_bytes(kind: str, la: int, lb: int = 0, stride: int = 1, max_a: int = 0, max_b: int = 0,
                signed: bool = False) -> int:
    """Algorithmic HBM bytes of one call: operands in, result out, and the fused
    four-step spectrum traffic 8*S (product) or 4*S (square), S = np*T*8 bytes of
    the reference planner's whole plan at crt_cost 1 (no block split)."""
    if kind == "conv":
        plan = conv_plan(la, lb, max_a, max_b, signed)
        s = plan["primes"] * plan["transform_len"] * 8
        return 8 * (la + lb) + 8 * (la + lb - 1) * plan["stride"] + 8 * s
    plan = mul_plan(la, la if kind == "sqr" else lb, 1)
    s = plan["primes"] * plan["transform_len"] * 8
    if kind == "sqr":
        return 8 * la + 16 * la + 4 * s
    return 16 * (la + lb) + 8 * s
