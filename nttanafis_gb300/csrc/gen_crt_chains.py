"""Writes crt_chains.cuh: the multiword carry chains of the CRT, one inline-PTX
block per chain, specialised for 1..8 primes.

A carry chain (add.cc / addc / mad.lo.cc / madc.hi.cc ...) passes the carry flag
from one instruction to the next. The flag is not a C++ value, so nothing keeps
the compiler from placing other instructions between two separate asm statements;
each chain is therefore emitted whole inside one asm statement. The operand lists
grow with the prime count, hence one specialisation per count.

Run from this directory:  python gen_crt_chains.py
"""
from __future__ import annotations

from pathlib import Path

MAX_PRIMES = 8


def accumulate(np_: int) -> str:
    """S[0..NP] += y * M[0..MW-1]: low halves into word w, high halves into w+1."""
    mw = np_ - 1 if np_ > 1 else 1
    s = lambda w: f"%{w}"            # S[w]: operands 0..NP
    y = f"%{np_ + 1}"
    m = lambda w: f"%{np_ + 2 + w}"  # M[w]
    lines = []
    # low halves
    lines.append(f"mad.lo.cc.u32 {s(0)}, {y}, {m(0)}, {s(0)};")
    for w in range(1, mw):
        lines.append(f"madc.lo.cc.u32 {s(w)}, {y}, {m(w)}, {s(w)};")
    for w in range(mw, np_ + 1):
        op = "addc.cc.u32" if w < np_ else "addc.u32"
        lines.append(f"{op} {s(w)}, {s(w)}, 0;")
    # high halves (a second chain)
    tail = list(range(2, mw + 1))
    lines.append(f"mad.hi.cc.u32 {s(1)}, {y}, {m(0)}, {s(1)};")
    for w in tail:
        lines.append(f"madc.hi.cc.u32 {s(w)}, {y}, {m(w - 1)}, {s(w)};")
    for w in range(mw + 1, np_ + 1):
        op = "addc.cc.u32" if w < np_ else "addc.u32"
        lines.append(f"{op} {s(w)}, {s(w)}, 0;")
    outs = ", ".join(f'"+r"(S[{w}])' for w in range(np_ + 1))
    ins = ", ".join(['"r"(y)'] + [f'"r"(M[{w}])' for w in range(mw)])
    body = "\n".join(f'        "{l}\\n\\t"' for l in lines)
    return (f"    static __device__ __forceinline__ void accumulate(u32 (&S)[{np_ + 1}], u32 y, const u32* M) {{\n"
            f"        asm(\n{body}\n        : {outs}\n        : {ins});\n    }}\n")


def subtract(np_: int) -> str:
    """x[0..NP] = S[0..NP] - U[0..NP] with borrows."""
    n = np_ + 1
    x = lambda w: f"%{w}"
    s = lambda w: f"%{n + w}"
    u = lambda w: f"%{2 * n + w}"
    lines = [f"sub.cc.u32 {x(0)}, {s(0)}, {u(0)};"]
    for w in range(1, n):
        op = "subc.cc.u32" if w < n - 1 else "subc.u32"
        lines.append(f"{op} {x(w)}, {s(w)}, {u(w)};")
    outs = ", ".join(f'"=r"(x[{w}])' for w in range(n))
    ins = ", ".join([f'"r"(S[{w}])' for w in range(n)] + [f'"r"(U[{w}])' for w in range(n)])
    body = "\n".join(f'        "{l}\\n\\t"' for l in lines)
    return (f"    static __device__ __forceinline__ void subtract(u32 (&x)[{n}], const u32 (&S)[{n}], "
            f"const u32 (&U)[{n}]) {{\n"
            f"        asm(\n{body}\n        : {outs}\n        : {ins});\n    }}\n")


def main() -> None:
    parts = [
        "// Generated by gen_crt_chains.py: multiword carry chains of the CRT, one\n"
        "// inline-PTX statement per chain (the carry flag never crosses statements).\n"
        "#pragma once\n#include \"ntt_arith.cuh\"\n\nnamespace ntt {\n\n"
        "template <int NP>\nstruct CrtChains;\n\n"
    ]
    for np_ in range(1, MAX_PRIMES + 1):
        parts.append(f"template <>\nstruct CrtChains<{np_}> {{\n")
        parts.append(accumulate(np_))
        parts.append(subtract(np_))
        parts.append("};\n\n")
    parts.append("}  // namespace ntt\n")
    out = Path(__file__).with_name("crt_chains.cuh")
    out.write_text("".join(parts))
    print(out)


if __name__ == "__main__":
    main()
