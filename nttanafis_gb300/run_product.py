"""Runs exact products of one shape on the device a few times, for profilers.

    python -m nttanafis_gb300.run_product --la 8388608 --lb 8388608 --reps 3
    python -m nttanafis_gb300.run_product --la 16777216 --square --reps 3

Operands are SplitMix64 limbs (seeds 1 and 2) made on the host and copied to the
device once; each repetition is one ntt_mul_workspace_mul_device call on the
current stream. The last product is checked against the fingerprint
A*B = C (mod 2^61 - 1) with Python integers, so a profile is only taken of a run
that computed the right product. Exit status 0 on success.
"""
from __future__ import annotations

import argparse
import sys


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--la", type=int, required=True)
    ap.add_argument("--lb", type=int, default=0, help="0 with --square")
    ap.add_argument("--square", action="store_true")
    ap.add_argument("--reps", type=int, default=3)
    args = ap.parse_args(argv)

    import numpy as np
    import torch

    from . import api as ntt
    from .operands import operand, to_int

    lb = args.la if args.square else args.lb
    if args.la <= 0 or lb <= 0:
        ap.error("operand lengths must be positive")
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream(dev)
    a_h = operand(args.la, 1)
    b_h = a_h if args.square else operand(lb, 2)
    a = torch.from_numpy(a_h.view(np.int64)).to(dev)
    b = a if args.square else torch.from_numpy(b_h.view(np.int64)).to(dev)
    d = torch.empty(args.la + lb, dtype=torch.int64, device=dev)
    ws = ntt.GpuMulWorkspace()
    for _ in range(args.reps):
        if not ws.mul_device(d, a, b, stream):
            print(ntt.last_error(), file=sys.stderr)
            return 1
    torch.cuda.synchronize(dev)
    q = (1 << 61) - 1
    c = d.cpu().numpy().view(np.uint64)
    ok = to_int(c) % q == (to_int(a_h) % q) * (to_int(b_h) % q) % q
    ws.close()
    print(f"{args.reps} products {args.la} x {lb}: fingerprint {'ok' if ok else 'WRONG'}")
    return 0 if ok else 2


if __name__ == "__main__":
    sys.exit(main())
