"""Compiles the oracle (test infrastructure) into oracle/_build/libntt_oracle.so.

Plain gcc on one C file; portable flags only (the same source builds on x86-64
and aarch64). -ffp-contract=off keeps every product that the exact-remainder
argument needs separately rounded, with fma() written out where it is meant.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build" / "libntt_oracle.so"
SRC = HERE / "ntt_oracle.c"


def build(force: bool = False) -> Path:
    if not force and OUT.exists() and OUT.stat().st_mtime >= max(SRC.stat().st_mtime,
                                                                  (HERE / "ntt_oracle.h").stat().st_mtime):
        return OUT
    OUT.parent.mkdir(exist_ok=True)
    tmp = OUT.with_suffix(".so.tmp")
    cmd = [os.environ.get("CC", "gcc"), "-O3", "-std=gnu11", "-ffp-contract=off", "-fno-fast-math", "-fPIC",
           "-shared", "-pthread", "-o", str(tmp), str(SRC), "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode:
        sys.stderr.write(res.stdout + res.stderr)
        raise RuntimeError("oracle build failed")
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
