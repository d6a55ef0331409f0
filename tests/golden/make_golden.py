"""Writes tests/golden/golden.json: known answers for the multiplication path.

Sources:
  * facts transcribed from the reference crate's own tests (paths relative to
    its root), cited per entry;
  * exact products and convolutions of SplitMix64 operands (bench/src/lib.rs:13-29
    of the reference) computed with Python's arbitrary-precision integers, which
    share no code with the oracle or the GPU library.

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from nttanafis_gb300.operands import operand  # noqa: E402  (pure-numpy SplitMix64)

MASK = (1 << 64) - 1


def to_int(limbs) -> int:
    v = 0
    for x in reversed([int(t) for t in limbs]):
        v = (v << 64) | x
    return v


def limbs(value: int, n: int) -> list[str]:
    return [format((value >> (64 * i)) & MASK, "016x") for i in range(n)]


def digest(value: int, n: int) -> str:
    return hashlib.sha256(value.to_bytes(8 * n, "little")).hexdigest()


def main() -> None:
    g: dict = {}
    # src/field/catalog.rs:67-76
    g["catalog"] = {
        "source": "src/field/catalog.rs:67-76",
        "primes": [1108307720798209, 1086317488242689, 910395627798529, 659706976665601, 699289395265537,
                   1022545813831681, 1013749720809473, 868614185943041],
        "generators": [11, 3, 7, 11, 5, 7, 3, 3],
    }
    # capacity c: 3*2^(c-1) <= P < 3*2^c (src/limb/tests/coefficients.rs:72-105)
    caps, P = [], 1
    for p in g["catalog"]["primes"]:
        P *= p
        c = 1
        while 3 * (1 << c) <= P:
            c += 1
        caps.append(c)
    g["capacities"] = {"source": "src/limb/tests/coefficients.rs:72-105 (property)", "bits": caps}
    # src/tests/plans.rs:46-80: for_residues at 8-bit values, bound 16, stride 64
    g["row_shapes"] = {
        "source": "src/tests/plans.rs:46-80",
        "cases": [[1, 1, 32, 32, 16], [30, 30, 64, 64, 32], [40, 40, 96, 64, 64], [49, 48, 96, 64, 64],
                  [49, 49, 128, 128, 64], [64, 33, 96, 64, 64], [65, 32, 128, 128, 64], [70, 20, 128, 128, 64],
                  [80, 80, 160, 128, 128], [100, 100, 224, 128, 128], [2100, 2100, 5120, 4096, 4096],
                  [3000, 2500, 6144, 4096, 4096], [3600, 3400, 7168, 4096, 4096], [4097, 1000, 8192, 8192, 4096]],
    }
    half = (1 << 32) - 1
    # src/tests/convolution.rs:283-298: stride(terms, max_a, max_b)
    g["strides"] = {
        "source": "src/tests/convolution.rs:283-298",
        "cases": [[1, 0, 0, 1], [1, 0, MASK, 1], [1, MASK, 1, 1], [1, half, half, 1], [2, half, half, 2],
                  [1, MASK, MASK, 2], [2, MASK, MASK, 3]],
    }
    g["conv_example"] = {"source": "src/lib.rs:89-102, src/tests/convolution.rs:300-308",
                         "a": [1, 2, 3], "b": [4, 5], "max_a": 7, "max_b": 7, "expected": [4, 13, 22, 15]}
    g["rejections"] = {
        "source": "src/tests/plans.rs:101-115, src/tests/convolution.rs:351-357,409-425",
        "mul_none": [[0, 1], [1, 0]],
        "conv_none": [[0, 1, 1, 1, 0], [1, 0, 1, 1, 0], [4, 4, (1 << 63), 1, 1]],
        "signed_beyond": {"a": [1, (MASK - 3), 0, 2], "b": [1, 2, 3, 0], "max": 3},
    }
    # Reference planner geometry at the benchmark shapes (crt_cost 1)
    g["geometry"] = {
        "source": "reference planner (src/profile/planner.rs:147-183,558-591) at crt_cost 1",
        "cases": [
            {"la": 1024, "lb": 1024, "primes": 6, "chunk_bits": 144, "digits_a": 456, "conv_len": 911,
             "transform_len": 1024},
            {"la": 1 << 20, "lb": 1 << 20, "primes": 6, "chunk_bits": 139, "digits_a": 482798,
             "conv_len": 965595, "transform_len": 1 << 20},
            {"la": 1 << 20, "lb": 131072, "primes": 7, "chunk_bits": 165, "digits_a": 406721,
             "conv_len": 457561, "transform_len": 1 << 19},
            {"la": 1 << 24, "lb": 1 << 24, "primes": 6, "chunk_bits": 137, "digits_a": 7837532,
             "conv_len": 15675063, "transform_len": 1 << 24},
        ],
    }
    prods = []
    for la, lb, sa, sb in [(1, 1, 1, 2), (3, 7, 1, 2), (40, 33, 1, 2), (64, 48, 1, 2), (300, 257, 5, 6),
                           (1024, 1024, 1, 2), (4097, 64, 1, 2), (3000, 1, 3, 4)]:
        a, b = operand(la, sa), operand(lb, sb)
        c = to_int(a) * to_int(b)
        entry = {"la": la, "lb": lb, "seed_a": sa, "seed_b": sb, "sha256": digest(c, la + lb)}
        if la + lb <= 4096:
            entry["product"] = limbs(c, la + lb)
        prods.append(entry)
    g["products"] = {"source": "Python integers on SplitMix64 operands", "cases": prods}
    sqrs = []
    for la, s in [(1, 1), (96, 1), (1024, 1)]:
        a = operand(la, s)
        c = to_int(a) ** 2
        sqrs.append({"la": la, "seed": s, "square": limbs(c, 2 * la)})
    g["squares"] = {"source": "Python integers", "cases": sqrs}
    convs = []
    for la, lb, bits, signed, sa, sb in [(30, 30, 16, False, 7, 8), (70, 1, 64, False, 9, 10),
                                          (100, 100, 32, True, 11, 12), (25, 25, 63, True, 13, 14),
                                          (24, 100, 8, False, 15, 16)]:
        mx = (1 << bits) - 1 if bits < 64 else MASK
        ra, rb = operand(la, sa), operand(lb, sb)
        if signed:
            # magnitude below the bound, sign from the limb's top bit
            av = [(-(int(x) & mx)) if int(x) >> 63 else (int(x) & mx) for x in ra]
            bv = [(-(int(x) & mx)) if int(x) >> 63 else (int(x) & mx) for x in rb]
        else:
            av = [int(x) & mx for x in ra]
            bv = [int(x) & mx for x in rb]
        coeffs = [0] * (la + lb - 1)
        for i, x in enumerate(av):
            for j, y in enumerate(bv):
                coeffs[i + j] += x * y
        convs.append({"la": la, "lb": lb, "bits": bits, "signed": signed,
                      "a": [format(v & MASK, "016x") for v in av], "b": [format(v & MASK, "016x") for v in bv],
                      "coefficients": [str(v) for v in coeffs]})
    g["convolutions"] = {"source": "Python integers", "cases": convs}
    out = Path(__file__).with_name("golden.json")
    out.write_text(json.dumps(g, indent=1))
    print(out, out.stat().st_size)


if __name__ == "__main__":
    main()
