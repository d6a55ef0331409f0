"""Builds the sm_103a shared library `_lib/libntt_gb300.so` in-tree with nvcc.

Each translation unit compiles in its own nvcc process (in parallel), then one
link step produces the library. Only `-gencode arch=compute_103a,code=sm_103a` is
emitted: the library targets GB300 alone.
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
SOURCES = ["api.cu", "plan.cu", "exec.cu", "batch.cu", "transform.cu", "small.cu", "crt.cu", "noalloc.cu",
           "field.cu", "probe.cu"]
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
    files = [CSRC / s for s in SOURCES]
    files += sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h"))
    files.append(HERE.parent / "include" / "ntt_gb300.h")
    return files


def up_to_date() -> bool:
    if not LIB.exists():
        return False
    mtime = LIB.stat().st_mtime
    return all(f.stat().st_mtime <= mtime for f in _inputs())


def build(force: bool = False, verbose: bool = False, extra_flags: list[str] | None = None) -> Path:
    """Compiles the library unless it is newer than every source; returns its path."""
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

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as pool:
        objs = list(pool.map(compile_one, SOURCES))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cc, "-shared", *ARCH, "-o", str(tmp), *map(str, objs), "-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode:
        sys.stderr.write(res.stdout + res.stderr)
        raise RuntimeError("nvcc link failed")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
