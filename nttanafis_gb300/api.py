"""Python mirror of the reference's multiplication API over the GB300 C ABI.

`MulPlan`, `GpuMulWorkspace`, `ConvPlan` and `GpuConvWorkspace` follow the call
shapes of `ntt_anafis::{MulPlan, MulWorkspace, ConvPlan, ConvWorkspace}`
(src/plan.rs:34-205, src/convolve.rs:52-281): operands and destinations are
little-endian `uint64` limb vectors, calls return `True` on success and `False`
on failure with the destination untouched, success preserves the destination's
suffix, and passing the same array as both operands squares it.

Host arrays are numpy `uint64` arrays (C-contiguous); device tensors are torch
`int64`/`uint64` CUDA tensors, passed to the `*_device` methods together with a
CUDA stream. There is no CPU fallback: without the compiled library every call
raises.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from pathlib import Path
from typing import Optional

import numpy as np

_LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libntt_gb300.so"
_lib: Optional[ctypes.CDLL] = None

u64p = ctypes.POINTER(ctypes.c_uint64)


class NttMulPlan(ctypes.Structure):
    _fields_ = [
        ("len_a", ctypes.c_uint64),
        ("len_b", ctypes.c_uint64),
        ("primes", ctypes.c_uint32),
        ("log_transform", ctypes.c_uint32),
        ("scratch_len", ctypes.c_uint64),
        ("sqr_scratch_len", ctypes.c_uint64),
        ("block_len", ctypes.c_uint64),
        ("blocks", ctypes.c_uint64),
    ]


class NttConvPlan(ctypes.Structure):
    _fields_ = [
        ("len_a", ctypes.c_uint64),
        ("len_b", ctypes.c_uint64),
        ("max_a", ctypes.c_uint64),
        ("max_b", ctypes.c_uint64),
        ("is_signed", ctypes.c_uint32),
        ("primes", ctypes.c_uint32),
        ("log_transform", ctypes.c_uint32),
        ("schoolbook", ctypes.c_uint32),
        ("stride", ctypes.c_uint64),
        ("output_len", ctypes.c_uint64),
        ("scratch_len", ctypes.c_uint64),
    ]


# (name, restype, argtypes) of every exported entry point of include/ntt_gb300.h.
_SIGNATURES = [
    ("ntt_mul_plan_new", ctypes.c_int, [ctypes.c_uint64, ctypes.c_uint64, ctypes.POINTER(NttMulPlan)]),
    ("ntt_mul_plan_mul_device", ctypes.c_uint8,
     [ctypes.POINTER(NttMulPlan), ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t,
      ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    ("ntt_mul_plan_sqr_device", ctypes.c_uint8,
     [ctypes.POINTER(NttMulPlan), ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t,
      ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    ("ntt_mul_workspace_new", ctypes.c_void_p, []),
    ("ntt_mul_workspace_free", None, [ctypes.c_void_p]),
    ("ntt_mul_workspace_prepare", ctypes.c_uint8, [ctypes.c_void_p, ctypes.POINTER(NttMulPlan)]),
    ("ntt_mul_workspace_mul", ctypes.c_uint8,
     [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t,
      ctypes.c_void_p, ctypes.c_size_t]),
    ("ntt_mul_workspace_sqr", ctypes.c_uint8,
     [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t]),
    ("ntt_mul_workspace_mul_device", ctypes.c_uint8,
     [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t,
      ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    ("ntt_mul_workspace_sqr_device", ctypes.c_uint8,
     [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    ("ntt_conv_plan_new", ctypes.c_int,
     [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int,
      ctypes.POINTER(NttConvPlan)]),
    ("ntt_conv_plan_convolve_device", ctypes.c_uint8,
     [ctypes.POINTER(NttConvPlan), ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t,
      ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    ("ntt_conv_plan_status", ctypes.c_int,
     [ctypes.POINTER(NttConvPlan), ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    ("ntt_mul_workspace_status", ctypes.c_uint32, [ctypes.c_void_p]),
    ("ntt_conv_workspace_status", ctypes.c_uint32, [ctypes.c_void_p]),
    ("ntt_conv_workspace_new", ctypes.c_void_p, []),
    ("ntt_conv_workspace_free", None, [ctypes.c_void_p]),
    ("ntt_conv_workspace_prepare", ctypes.c_uint8, [ctypes.c_void_p, ctypes.POINTER(NttConvPlan)]),
    ("ntt_conv_workspace_convolve", ctypes.c_uint8,
     [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t,
      ctypes.c_void_p, ctypes.c_size_t]),
    ("ntt_conv_workspace_convolve_device", ctypes.c_uint8,
     [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t,
      ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    ("ntt_batch_new", ctypes.c_void_p, []),
    ("ntt_batch_free", None, [ctypes.c_void_p]),
    ("ntt_batch_run_device", ctypes.c_uint8, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    ("ntt_batch_set_graphs", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    ("ntt_batch_set_lanes", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    ("ntt_batch_stats", None, [ctypes.c_void_p, ctypes.c_void_p]),
    ("ntt_batch_status", ctypes.c_uint32, [ctypes.c_void_p]),
    ("ntt_batch_split_members", ctypes.c_uint64, [ctypes.c_void_p]),
    ("ntt_mul_noalloc_device", ctypes.c_uint8,
     [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t,
      ctypes.c_void_p]),
    ("ntt_timing_start", ctypes.c_int, [ctypes.c_int]),
    ("ntt_timing_stop", ctypes.c_int, [ctypes.POINTER(ctypes.c_float), ctypes.c_int]),
    ("ntt_lookback_timeouts", ctypes.c_uint32, []),
    ("ntt_debug_stall_lookback", ctypes.c_int, [ctypes.c_int]),
    ("ntt_school_set", ctypes.c_uint64, [ctypes.c_uint64]),
    ("ntt_split_set", ctypes.c_int, [ctypes.c_int, ctypes.c_int]),
    ("ntt_split_get", ctypes.c_int, [ctypes.c_int]),
    ("ntt_split_range", ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]),
    ("ntt_tune_splits", ctypes.c_uint8, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]),
    ("ntt_field_check", ctypes.c_int, [ctypes.c_uint64]),
    ("ntt_field_mul_method", ctypes.c_int, [ctypes.c_int]),
    ("ntt_field_below", ctypes.c_uint64, [ctypes.c_uint64]),
    ("ntt_field_catalog", ctypes.c_size_t, [ctypes.c_void_p, ctypes.c_size_t]),
    ("ntt_field_binary_device", ctypes.c_uint8,
     [ctypes.c_uint64, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
      ctypes.c_void_p]),
    ("ntt_field_unary_device", ctypes.c_uint8,
     [ctypes.c_uint64, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_uint64,
      ctypes.c_void_p, ctypes.c_void_p]),
    ("ntt_field_scale_device", ctypes.c_uint8,
     [ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_uint64, ctypes.c_void_p]),
    ("ntt_field_evaluate_device", ctypes.c_uint8,
     [ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t,
      ctypes.c_void_p]),
    ("ntt_crt_pair_combine_device", ctypes.c_uint8,
     [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
      ctypes.c_void_p]),
    ("ntt_last_error", ctypes.c_char_p, []),
    ("ntt_kernel_launches", ctypes.c_uint64, []),
    ("ntt_version", ctypes.c_char_p, []),
]


def library() -> ctypes.CDLL:
    """Loads libntt_gb300.so (building it first if nvcc is present); raises if absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not _LIB_PATH.exists():
        from . import build_ext

        try:
            build_ext.build()
        except Exception as exc:  # no toolkit: fail loudly, never fall back
            raise RuntimeError(f"libntt_gb300.so is not built and cannot be built: {exc}") from exc
    lib = ctypes.CDLL(str(_LIB_PATH))
    for name, restype, argtypes in _SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = restype
        fn.argtypes = argtypes
    _lib = lib
    return lib


def exported_symbols() -> list[str]:
    return [name for name, _, _ in _SIGNATURES]


def last_error() -> str:
    return library().ntt_last_error().decode()


def kernel_launches() -> int:
    return int(library().ntt_kernel_launches())


def lookback_timeouts() -> int:
    """Bounded look-back waits of the CRT carry scan that gave up (expected 0)."""
    return int(library().ntt_lookback_timeouts())


# Status bits of device-pointer calls (NTT_STATUS_* in include/ntt_gb300.h).
STATUS_LOOKBACK = 1  # a carry look-back wait gave up: that product is wrong
STATUS_BOUND = 2     # a convolution coefficient exceeded its bound: not written


def debug_stall_lookback(count: int) -> int:
    """Test hook: the next `count` look-back CRT launches start with their tile
    counter at 1, so the bounded wait for tile 0 runs out. Returns the previous count."""
    return int(library().ntt_debug_stall_lookback(int(count)))


def set_basecase_limit(max_products: int) -> int:
    """Single-call products with a_len * b_len <= max_products take the direct
    column-sum basecase (0: never); returns the previous limit."""
    return int(library().ntt_school_set(int(max_products)))


def split_range(log_t: int) -> Optional[tuple[int, int]]:
    """(lowest, highest) log2 R of the four-step split of 2^log_t points, or None
    when that length has no choice of split."""
    lo, hi = ctypes.c_int(0), ctypes.c_int(0)
    if not library().ntt_split_range(log_t, ctypes.byref(lo), ctypes.byref(hi)):
        return None
    return lo.value, hi.value


def get_split(log_t: int) -> int:
    """log2 R of the four-step split in use for 2^log_t points (0: no four-step form)."""
    return int(library().ntt_split_get(log_t))


def set_split(log_t: int, log_r: int) -> int:
    """Sets log2 R for 2^log_t points (0: the default); returns the previous one."""
    prev = int(library().ntt_split_set(log_t, log_r))
    if prev < 0:
        raise ValueError(f"no split 2^{log_r} for transforms of 2^{log_t} points")
    return prev


def tune_splits(min_log_t: int = 14, max_log_t: int = 23, reps: int = 5, stream=None) -> dict:
    """Times every four-step split of each transform length on the current GPU and
    keeps the fastest (see ntt_tune_splits); returns {log_t: log_r} in use after it."""
    if not library().ntt_tune_splits(min_log_t, max_log_t, reps, _stream_handle(stream)):
        raise RuntimeError(last_error())
    return {t: get_split(t) for t in range(max(min_log_t, 14), min(max_log_t, 23) + 1)}


def save_splits(path) -> None:
    """Writes the splits in use to a JSON file (tuning results for the next run)."""
    import json

    data = {str(t): get_split(t) for t in range(14, 24) if split_range(t)}
    with open(path, "w") as f:
        json.dump(data, f, indent=1)


def load_splits(path) -> dict:
    """Applies splits saved by save_splits; returns them."""
    import json

    with open(path) as f:
        data = {int(k): int(v) for k, v in json.load(f).items()}
    for t, r in data.items():
        set_split(t, r)
    return data


def _host(arr: np.ndarray, name: str) -> np.ndarray:
    if not isinstance(arr, np.ndarray) or arr.dtype != np.uint64 or arr.ndim != 1:
        raise TypeError(f"{name} must be a 1-D numpy uint64 array")
    if not arr.flags["C_CONTIGUOUS"]:
        raise TypeError(f"{name} must be contiguous")
    return arr


def _ptr(arr: np.ndarray) -> int:
    return arr.ctypes.data if arr.size else 0


def _dev(t) -> tuple[int, int]:
    """(device pointer, element count) of a 1-D 64-bit CUDA tensor."""
    if t.element_size() != 8 or t.dim() != 1 or not t.is_contiguous() or not t.is_cuda:
        raise TypeError("device operands must be contiguous 1-D 64-bit CUDA tensors")
    return int(t.data_ptr()), int(t.numel())


def _stream_handle(stream) -> int:
    if stream is None:
        return 0
    return int(getattr(stream, "cuda_stream", stream))


@dataclass(frozen=True)
class MulPlan:
    """An admitted product shape (ntt_anafis MulPlan, src/plan.rs:34-114)."""

    len_a: int
    len_b: int
    primes: int
    log_transform: int
    scratch_len_limbs: int
    sqr_scratch_len_limbs: int
    block_len: int = 0  # block split: limbs per block of the longer operand (0: none)
    blocks: int = 0

    @staticmethod
    def new(len_a: int, len_b: int) -> Optional["MulPlan"]:
        raw = NttMulPlan()
        if not library().ntt_mul_plan_new(len_a, len_b, ctypes.byref(raw)):
            return None
        return MulPlan(raw.len_a, raw.len_b, raw.primes, raw.log_transform, raw.scratch_len,
                       raw.sqr_scratch_len, raw.block_len, raw.blocks)

    def scratch_len(self) -> int:
        return self.scratch_len_limbs

    def sqr_scratch_len(self) -> int:
        return self.sqr_scratch_len_limbs

    def _raw(self) -> NttMulPlan:
        return NttMulPlan(self.len_a, self.len_b, self.primes, self.log_transform, self.scratch_len_limbs,
                          self.sqr_scratch_len_limbs, self.block_len, self.blocks)

    def mul_device(self, dst, a, b, scratch, stream=None) -> bool:
        """a*b on device tensors with caller-owned device scratch (MulPlan::mul)."""
        d, nd = _dev(dst)
        pa, na = _dev(a)
        pb, nb = _dev(b)
        ps, ns = _dev(scratch)
        return bool(library().ntt_mul_plan_mul_device(ctypes.byref(self._raw()), d, nd, pa, na, pb, nb, ps, ns,
                                                      _stream_handle(stream)))

    def sqr_device(self, dst, a, scratch, stream=None) -> bool:
        d, nd = _dev(dst)
        pa, na = _dev(a)
        ps, ns = _dev(scratch)
        return bool(library().ntt_mul_plan_sqr_device(ctypes.byref(self._raw()), d, nd, pa, na, ps, ns,
                                                      _stream_handle(stream)))


class GpuMulWorkspace:
    """Retained device tables and arenas (ntt_anafis MulWorkspace, src/plan.rs:135-205)."""

    def __init__(self) -> None:
        self._lib = library()
        self._ws = self._lib.ntt_mul_workspace_new()
        if not self._ws:
            raise RuntimeError(f"cannot create a GPU workspace: {last_error()}")

    def close(self) -> None:
        if getattr(self, "_ws", None):
            self._lib.ntt_mul_workspace_free(self._ws)
            self._ws = None

    def __del__(self) -> None:
        try:
            self.close()
        except Exception:
            pass

    def prepare(self, plan: MulPlan) -> bool:
        return bool(self._lib.ntt_mul_workspace_prepare(self._ws, ctypes.byref(plan._raw())))

    def mul(self, dst: np.ndarray, a: np.ndarray, b: np.ndarray) -> bool:
        _host(dst, "dst"), _host(a, "a"), _host(b, "b")
        return bool(self._lib.ntt_mul_workspace_mul(self._ws, _ptr(dst), dst.size, _ptr(a), a.size, _ptr(b),
                                                    b.size))

    def sqr(self, dst: np.ndarray, a: np.ndarray) -> bool:
        _host(dst, "dst"), _host(a, "a")
        return bool(self._lib.ntt_mul_workspace_sqr(self._ws, _ptr(dst), dst.size, _ptr(a), a.size))

    def mul_device(self, dst, a, b, stream=None) -> bool:
        d, nd = _dev(dst)
        pa, na = _dev(a)
        pb, nb = _dev(b)
        return bool(self._lib.ntt_mul_workspace_mul_device(self._ws, d, nd, pa, na, pb, nb,
                                                           _stream_handle(stream)))

    def sqr_device(self, dst, a, stream=None) -> bool:
        d, nd = _dev(dst)
        pa, na = _dev(a)
        return bool(self._lib.ntt_mul_workspace_sqr_device(self._ws, d, nd, pa, na, _stream_handle(stream)))

    def status(self) -> int:
        """STATUS_* bits of the device-pointer calls since the last query (0: all
        succeeded); read after their streams have completed. Reading clears them."""
        return int(self._lib.ntt_mul_workspace_status(self._ws))


@dataclass(frozen=True)
class ConvPlan:
    """An admitted convolution (ntt_anafis ConvPlan, src/convolve.rs:52-217)."""

    len_a: int
    len_b: int
    max_a: int
    max_b: int
    signed: bool
    primes: int
    log_transform: int
    schoolbook: bool
    stride_limbs: int
    output_limbs: int
    scratch_limbs: int

    @staticmethod
    def new(len_a: int, len_b: int, max_a: int, max_b: int, signed: bool = False) -> Optional["ConvPlan"]:
        raw = NttConvPlan()
        if not library().ntt_conv_plan_new(len_a, len_b, max_a, max_b, int(signed), ctypes.byref(raw)):
            return None
        return ConvPlan(raw.len_a, raw.len_b, raw.max_a, raw.max_b, bool(raw.is_signed), raw.primes,
                        raw.log_transform, bool(raw.schoolbook), raw.stride, raw.output_len, raw.scratch_len)

    def stride(self) -> int:
        return self.stride_limbs

    def output_len(self) -> int:
        return self.output_limbs

    def scratch_len(self) -> int:
        return self.scratch_limbs

    def _raw(self) -> NttConvPlan:
        return NttConvPlan(self.len_a, self.len_b, self.max_a, self.max_b, int(self.signed), self.primes,
                           self.log_transform, int(self.schoolbook), self.stride_limbs, self.output_limbs,
                           self.scratch_limbs)

    def convolve_device(self, dst, a, b, scratch, stream=None) -> bool:
        d, nd = _dev(dst)
        pa, na = _dev(a)
        pb, nb = _dev(b)
        ps, ns = _dev(scratch) if scratch is not None else (0, 0)
        return bool(library().ntt_conv_plan_convolve_device(ctypes.byref(self._raw()), d, nd, pa, na, pb, nb,
                                                            ps, ns, _stream_handle(stream)))

    def status(self, scratch, stream=None) -> int:
        """Outcome of the last convolve_device that used `scratch` (waits for
        `stream`): 1 written, 0 a coefficient exceeded its bound (dst untouched),
        -1 error."""
        ps, ns = _dev(scratch)
        return int(library().ntt_conv_plan_status(ctypes.byref(self._raw()), ps, ns, _stream_handle(stream)))


class GpuConvWorkspace:
    """Retained convolution storage (ntt_anafis ConvWorkspace, src/convolve.rs:229-281)."""

    def __init__(self) -> None:
        self._lib = library()
        self._ws = self._lib.ntt_conv_workspace_new()
        if not self._ws:
            raise RuntimeError(f"cannot create a GPU workspace: {last_error()}")

    def close(self) -> None:
        if getattr(self, "_ws", None):
            self._lib.ntt_conv_workspace_free(self._ws)
            self._ws = None

    def __del__(self) -> None:
        try:
            self.close()
        except Exception:
            pass

    def prepare(self, plan: ConvPlan) -> bool:
        return bool(self._lib.ntt_conv_workspace_prepare(self._ws, ctypes.byref(plan._raw())))

    def convolve(self, dst: np.ndarray, a: np.ndarray, b: np.ndarray) -> bool:
        _host(dst, "dst"), _host(a, "a"), _host(b, "b")
        return bool(self._lib.ntt_conv_workspace_convolve(self._ws, _ptr(dst), dst.size, _ptr(a), a.size,
                                                          _ptr(b), b.size))

    def convolve_device(self, dst, a, b, stream=None) -> bool:
        d, nd = _dev(dst)
        pa, na = _dev(a)
        pb, nb = _dev(b)
        return bool(self._lib.ntt_conv_workspace_convolve_device(self._ws, d, nd, pa, na, pb, nb,
                                                                 _stream_handle(stream)))

    def status(self) -> int:
        """STATUS_* bits of the device-pointer calls since the last query (0: all
        succeeded); read after their streams have completed. Reading clears them."""
        return int(self._lib.ntt_conv_workspace_status(self._ws))


class NttRequest(ctypes.Structure):
    _fields_ = [
        ("dst", ctypes.c_void_p),
        ("dst_len", ctypes.c_uint64),
        ("a", ctypes.c_void_p),
        ("b", ctypes.c_void_p),
        ("a_len", ctypes.c_uint64),
        ("b_len", ctypes.c_uint64),
        ("kind", ctypes.c_uint32),
        ("is_signed", ctypes.c_uint32),
        ("max_a", ctypes.c_uint64),
        ("max_b", ctypes.c_uint64),
    ]


@dataclass
class Request:
    """One batch member on device tensors: a product (kind "mul"; the same tensor
    twice squares it) or a convolution (kind "conv") under ConvPlan's bounds."""

    dst: object
    a: object
    b: object
    kind: str = "mul"
    max_a: int = 0
    max_b: int = 0
    signed: bool = False

    def raw(self) -> NttRequest:
        d, nd = _dev(self.dst)
        pa, na = _dev(self.a)
        pb, nb = _dev(self.b)
        return NttRequest(d, nd, pa, pb, na, nb, 0 if self.kind == "mul" else 1, int(self.signed), self.max_a,
                          self.max_b)


class GpuBatch:
    """Batched executor: many exact products/convolutions per enqueue, grouped by
    transform class (one launch per kernel and class). Calls on one object must be
    ordered on one stream."""

    def __init__(self) -> None:
        self._lib = library()
        self._b = self._lib.ntt_batch_new()
        if not self._b:
            raise RuntimeError(f"cannot create a batch: {last_error()}")

    def close(self) -> None:
        if getattr(self, "_b", None):
            self._lib.ntt_batch_free(self._b)
            self._b = None

    def __del__(self) -> None:
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def pack(requests) -> ctypes.Array:
        arr = (NttRequest * len(requests))()
        for i, r in enumerate(requests):
            arr[i] = r.raw() if isinstance(r, Request) else r
        return arr

    def run(self, requests, stream=None) -> bool:
        """Enqueues `requests` (Request objects or a packed array) on `stream`."""
        arr = requests if isinstance(requests, ctypes.Array) else self.pack(requests)
        return bool(self._lib.ntt_batch_run_device(self._b, ctypes.cast(arr, ctypes.c_void_p), len(arr),
                                                   _stream_handle(stream)))

    def set_graphs(self, on: bool) -> bool:
        """Turns CUDA-graph replay of repeated batch compositions on or off; returns
        the previous setting."""
        return bool(self._lib.ntt_batch_set_graphs(self._b, 1 if on else 0))

    def set_lanes(self, lanes: int) -> int:
        """Fixes the streams (1, 2 or 4) the classes of a run spread over, or with 0
        lets the batch tune them per composition; returns the previous setting."""
        return int(self._lib.ntt_batch_set_lanes(self._b, int(lanes)))

    def stats(self) -> dict:
        """Graph replays, compositions tuned, lanes of the last enqueued run and
        compositions held by this batch object."""
        out = (ctypes.c_uint64 * 4)()
        self._lib.ntt_batch_stats(self._b, out)
        return {"graph_replays": out[0], "tuned": out[1], "last_lanes": out[2], "compositions": out[3]}

    def status(self) -> int:
        """STATUS_* bits of this batch's runs since the last query (0: every member
        succeeded); read after the runs' stream has completed. Reading clears them."""
        return int(self._lib.ntt_batch_status(self._b))

    @property
    def split_members(self) -> int:
        """Products of this batch object's runs that ran as block splits."""
        return int(self._lib.ntt_batch_split_members(self._b))

    @property
    def graph_replays(self) -> int:
        """Runs of this batch object served from a captured CUDA graph."""
        return self.stats()["graph_replays"]
