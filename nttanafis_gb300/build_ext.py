"""Builds the sm_103a shared libraries in-tree with nvcc:

  _lib/libntt_gb300.so  the product: the C ABI of include/ntt_gb300.h;
  _lib/libntt_probe.so  a measurement tool (include/ntt_probe.h): register-only
                        arithmetic probes that bench.py loads for its compute
                        ceiling. The product never loads it.

Each translation unit compiles in its own nvcc process (in parallel), then one
link step per library. Only `-gencode arch=compute_103a,code=sm_103a` is emitted:
the libraries target GB300 alone.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
LIBDIR = HERE / "_lib"
LIB = LIBDIR / "libntt_gb300.so"
PROBE_LIB = LIBDIR / "libntt_probe.so"
SOURCES = ["api.cu", "plan.cu", "exec.cu", "batch.cu", "transform.cu", "small.cu", "crt.cu", "school.cu",
           "noalloc.cu", "field.cu"]
PROBE_SOURCES = ["probe.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    found = shutil.which("nvcc")
    if found:
        return found
    default = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(default):
        return default
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libntt_gb300.so")


def _inputs() -> list[Path]:
    files = [CSRC / s for s in SOURCES + PROBE_SOURCES]
    files += sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h"))
    files += sorted((HERE.parent / "include").glob("*.h"))
    return files


def up_to_date() -> bool:
    if not LIB.exists() or not PROBE_LIB.exists():
        return False
    mtime = min(LIB.stat().st_mtime, PROBE_LIB.stat().st_mtime)
    return all(f.stat().st_mtime <= mtime for f in _inputs())


def build(force: bool = False, verbose: bool = False, extra_flags: list[str] | None = None) -> Path:
    """Compiles both libraries unless they are newer than every source; returns the
    product library's path."""
    if not force and up_to_date():
        return LIB
    LIBDIR.mkdir(exist_ok=True)
    obj_dir = LIBDIR / "obj"
    obj_dir.mkdir(exist_ok=True)
    cc = nvcc()
    common = [
        cc, "-O3", "-std=c++17", "-lineinfo", *ARCH,
        "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
        "-I", str(CSRC), "-I", str(HERE.parent / "include"),
        *(extra_flags or []),
    ]

    def compile_one(src: str) -> Path:
        obj = obj_dir / (Path(src).stem + ".o")
        cmd = common + ["-c", str(CSRC / src), "-o", str(obj)]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or res.returncode:
            sys.stderr.write(res.stdout + res.stderr)
        if res.returncode:
            raise RuntimeError(f"nvcc failed on {src}")
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES) + len(PROBE_SOURCES)) as pool:
        objs = list(pool.map(compile_one, SOURCES + PROBE_SOURCES))
    for lib, part in ((LIB, objs[:len(SOURCES)]), (PROBE_LIB, objs[len(SOURCES):])):
        tmp = lib.with_suffix(".so.tmp")
        cmd = [cc, "-shared", *ARCH, "-o", str(tmp), *map(str, part), "-lcudart"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode:
            sys.stderr.write(res.stdout + res.stderr)
            raise RuntimeError(f"nvcc link failed for {lib.name}")
        os.replace(tmp, lib)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
