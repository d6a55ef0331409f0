"""Adds exact SHA-256 digests of the largest benchmark products to golden.json.

The 16,777,216 x 16,777,216-limb product and square of SplitMix64 operands
(seeds 1 and 2, as the reference benchmarks draw them: bench/src/lib.rs:13-29 of
the reference) are too large for Python's integer multiplication, so the oracle
(the C restatement of the reference algorithm, oracle/ntt_oracle.c) computes them
once, on every host thread. Before a digest is written, each result is checked
against four Mersenne-prime fingerprints computed with Python integers, which
share no code with the oracle:  A*B = C (mod q) for q = 2^61-1, 2^89-1, 2^107-1,
2^127-1. The GPU tests then compare the GPU products with these digests.

Run from the repository root:  python tests/golden/make_big_digests.py
(about a minute on 8 x86 cores).
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402  (test infrastructure: the checker)
from nttanafis_gb300.operands import operand, to_int  # noqa: E402

FINGERPRINT_PRIMES = [(1 << 61) - 1, (1 << 89) - 1, (1 << 107) - 1, (1 << 127) - 1]
GOLDEN = Path(__file__).with_name("golden.json")


def fingerprints_agree(a, b, c) -> bool:
    A, B, C = to_int(a), to_int(b), to_int(c)
    return all((A % q) * (B % q) % q == C % q for q in FINGERPRINT_PRIMES)


def digest(limbs) -> str:
    return hashlib.sha256(limbs.astype("<u8").tobytes()).hexdigest()


def main() -> None:
    threads = os.cpu_count() or 1
    n = 1 << 24
    a, b = operand(n, 1), operand(n, 2)
    cases = []
    t0 = time.time()
    c = oracle.mul(a, b, threads)
    assert fingerprints_agree(a, b, c), "oracle product disagrees with the fingerprints"
    cases.append({"kind": "mul", "la": n, "lb": n, "seed_a": 1, "seed_b": 2, "sha256": digest(c)})
    s = oracle.sqr(a, threads)
    assert fingerprints_agree(a, a, s), "oracle square disagrees with the fingerprints"
    cases.append({"kind": "sqr", "la": n, "lb": n, "seed_a": 1, "seed_b": 1, "sha256": digest(s)})
    g = json.loads(GOLDEN.read_text())
    g["big_products"] = {
        "source": "oracle/ntt_oracle.c on every host thread, each result checked against Mersenne-prime "
                  "fingerprints (2^61-1, 2^89-1, 2^107-1, 2^127-1) computed with Python integers",
        "cases": cases,
    }
    GOLDEN.write_text(json.dumps(g, indent=1))
    print(f"{GOLDEN}: {len(cases)} digests in {time.time() - t0:.1f} s on {threads} threads")


if __name__ == "__main__":
    main()
