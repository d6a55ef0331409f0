"""ctypes binding of libntt_probe.so (include/ntt_probe.h): register-only
arithmetic probes for measurement tools. The product path never loads it."""
from __future__ import annotations

import ctypes
from pathlib import Path

_PATH = Path(__file__).resolve().parent / "_lib" / "libntt_probe.so"
_lib = None

# Variant names of ntt_probe_arith, in order.
VARIANTS = ["shoup32_butterfly", "montgomery32_butterfly", "shoup64_butterfly_50bit", "f64_fma_butterfly_50bit",
            "imad", "imad_hi", "iadd3", "imul64", "dfma", "imad_wide", "i2f",
            "shoup32_wide_quotient_butterfly", "shoup32_c64_quotient_butterfly"]


def library() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not _PATH.exists():
            from . import build_ext

            build_ext.build()
        lib = ctypes.CDLL(str(_PATH))
        lib.ntt_probe_variants.restype = ctypes.c_int
        lib.ntt_probe_variants.argtypes = []
        lib.ntt_probe_arith.restype = ctypes.c_uint8
        lib.ntt_probe_arith.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_float),
                                        ctypes.POINTER(ctypes.c_double)]
        lib.ntt_probe_butterflies.restype = ctypes.c_uint8
        lib.ntt_probe_butterflies.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_float)]
        _lib = lib
    return _lib


def exported_symbols() -> list[str]:
    return ["ntt_probe_arith", "ntt_probe_butterflies", "ntt_probe_variants"]


def rate(variant: int, blocks: int = 152 * 8, iters: int = 2000) -> float:
    """Operations per second of probe `variant` (butterflies or instructions)."""
    ms, ops = ctypes.c_float(0.0), ctypes.c_double(0.0)
    if not library().ntt_probe_arith(variant, blocks, iters, ctypes.byref(ms), ctypes.byref(ops)):
        raise RuntimeError(f"probe variant {variant} failed")
    return ops.value / (ms.value * 1e-3)


def butterfly_rate(blocks: int = 152 * 8, iters: int = 2000) -> float:
    """Lazy 32-bit butterflies per second with no memory traffic: the
    integer-issue ceiling of the transform kernels on this GPU."""
    return rate(0, blocks, iters)
