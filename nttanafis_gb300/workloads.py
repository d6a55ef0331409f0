"""Seeded synthetic workloads for the batched and served forms.

* `batched_shapes`: independent products with log-uniform operand lengths in
  [256, 65536] limbs, a log-uniform length ratio up to 8:1 on a random side and
  25% squares (the batched configuration).
* `served_stream`: Poisson arrivals of products/squares with log-uniform lengths
  192..4,194,304 limbs and dense convolutions of 16-bit unsigned, 32-bit unsigned
  and 32-bit two's complement coefficients (1,024..4,194,304 coefficients), with
  the bounds 2^16-1, 2^32-1 and 2^31.
Operand limbs come from SplitMix64 streams (nttanafis_gb300.operands.operand).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .operands import operand


@dataclass(frozen=True)
class Shape:
    kind: str  # "mul" | "sqr" | "conv"
    la: int
    lb: int
    seed_a: int
    seed_b: int
    bits: int = 64        # coefficient bits of a convolution
    signed: bool = False
    arrival: float = 0.0  # seconds from the start of a served stream

    @property
    def max_a(self) -> int:
        if self.kind != "conv":
            return 0
        return 1 << 31 if self.signed else (1 << self.bits) - 1

    def out_len(self) -> int:
        if self.kind == "conv":
            from .api import ConvPlan

            return ConvPlan.new(self.la, self.lb, self.max_a, self.max_a, self.signed).output_len()
        return self.la + (self.la if self.kind == "sqr" else self.lb)

    def operands(self) -> tuple[np.ndarray, np.ndarray]:
        a = operand(self.la, self.seed_a)
        if self.kind == "sqr":
            return a, a
        b = operand(self.lb, self.seed_b)
        if self.kind == "conv":
            if self.signed:
                mag = np.uint64((1 << 31) - 1)
                def signed(x):
                    m = (x & mag).astype(np.uint64)
                    neg = (x >> np.uint64(63)).astype(bool)
                    return np.where(neg, (np.uint64(0) - m), m).astype(np.uint64)
                return signed(a), signed(b)
            mask = np.uint64((1 << self.bits) - 1)
            return a & mask, b & mask
        return a, b


def _log_uniform(rng: np.random.Generator, lo: float, hi: float) -> float:
    return float(np.exp(rng.uniform(np.log(lo), np.log(hi))))


def batched_shapes(count: int = 4096, seed: int = 5) -> list[Shape]:
    rng = np.random.default_rng(seed)
    shapes = []
    for i in range(count):
        la = int(round(_log_uniform(rng, 256, 65536)))
        if rng.uniform() < 0.25:
            shapes.append(Shape("sqr", la, la, 1000 + 2 * i, 1000 + 2 * i))
            continue
        lb = max(1, int(round(la / _log_uniform(rng, 1, 8))))
        if rng.uniform() < 0.5:
            la, lb = lb, la
        shapes.append(Shape("mul", la, lb, 1000 + 2 * i, 1001 + 2 * i))
    return shapes


def served_stream(count: int, rate_hz: float, seed: int = 7, max_limbs: int = 4194304) -> list[Shape]:
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(count):
        t += float(rng.exponential(1.0 / rate_hz))
        r = rng.uniform()
        if r < 0.5:
            la = int(round(_log_uniform(rng, 192, max_limbs)))
            lb = max(1, int(round(_log_uniform(rng, 192, max_limbs))))
            if la + lb - 1 > (1 << 25):
                lb = (1 << 25) + 1 - la
            out.append(Shape("mul", la, lb, 5000 + 2 * i, 5001 + 2 * i, arrival=t))
        elif r < 0.65:
            la = int(round(_log_uniform(rng, 192, max_limbs)))
            out.append(Shape("sqr", la, la, 5000 + 2 * i, 5000 + 2 * i, arrival=t))
        else:
            n = int(round(_log_uniform(rng, 1024, max_limbs)))
            m = int(round(_log_uniform(rng, 1024, max_limbs)))
            if n + m - 1 > (1 << 25):
                m = (1 << 25) + 1 - n
            kind = rng.integers(0, 3)
            bits, signed = [(16, False), (32, False), (32, True)][int(kind)]
            out.append(Shape("conv", n, m, 5000 + 2 * i, 5001 + 2 * i, bits=bits, signed=signed, arrival=t))
    return out
