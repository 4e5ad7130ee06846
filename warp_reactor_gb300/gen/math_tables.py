"""Generate csrc/wr_math_tables.h: fixed-point tables for the portable exp/log.

Every entry is the correctly rounded value of a mathematical constant, computed with
mpmath at 200 bits, so the header is reproducible.  Run
``python -m warp_reactor_gb300.gen.math_tables`` to rewrite it (needs mpmath; the
header is committed so builds do not).

Tables
  WR_EXP_T1[i] = round(2^(i/64)   * 2^63), i = 0..63
  WR_EXP_T2[i] = round(2^(i/4096) * 2^63), i = 0..63
  WR_LOG_R[i]  = r_i, an integer in [1024, 2048] with r_i/2048 ~ 1/(1+(i+1/2)/512);
                 r_0 = 2048 and r_511 = 1024 exactly (the near-1 intervals)
  WR_LOG_NL[i] = -log(r_i / 2048) as a signed Q96 number in two words (hi, lo)
Constants
  WR_L2E_Q127  = floor(log2(e) * 2^127) in two words
  WR_LN2_Q64   = round(ln(2) * 2^64)
  WR_LN2_Q96   = round(ln(2) * 2^96) in two words (WR_LOG_NL[511] equals it)
  WR_INV_Q62[k]= round(2^62 / k), k = 1..7
"""
from __future__ import annotations

import os

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(os.path.dirname(HERE), "csrc", "wr_math_tables.h")


def build() -> str:
    import mpmath as mp

    mp.mp.prec = 200

    def rnd(x):
        return int(mp.nint(x))

    t1 = [rnd(mp.power(2, mp.mpf(i) / 64) * mp.power(2, 63)) for i in range(64)]
    t2 = [rnd(mp.power(2, mp.mpf(i) / 4096) * mp.power(2, 63)) for i in range(64)]
    assert all(2**63 <= v < 2**64 for v in t1 + t2)
    rs = []
    for i in range(512):
        if i == 0:
            r = 2048
        elif i == 511:
            r = 1024
        else:
            c = 1 + (mp.mpf(i) + mp.mpf(0.5)) / 512
            r = rnd(2048 / c)
        rs.append(r)
    ln2_q96 = rnd(mp.log(2) * mp.power(2, 96))
    nl = []
    for i, r in enumerate(rs):
        if i == 511:
            v = ln2_q96  # -log(1/2) shares the rounding of ln2 so that E*ln2 cancels
        else:
            v = rnd(-mp.log(mp.mpf(r) / 2048) * mp.power(2, 96))
        nl.append(v)
    l2e = int(mp.floor(mp.log(mp.e, 2) * mp.power(2, 127)))
    ln2_q64 = rnd(mp.log(2) * mp.power(2, 64))
    inv = [rnd(mp.power(2, 62) / k) for k in range(1, 8)]

    def words(v):
        v &= (1 << 128) - 1
        return f"0x{v >> 64:016x}ULL, 0x{v & ((1 << 64) - 1):016x}ULL"

    lines = [
        "// Generated by warp_reactor_gb300/gen/math_tables.py (mpmath, 200-bit); do not edit.",
        "// Fixed-point tables of the portable exp/log in wr_math.h.",
        "#pragma once",
        "#define WR_EXP_T1_INIT { \\",
    ]
    for i in range(0, 64, 4):
        lines.append("    " + ", ".join(f"0x{v:016x}ULL" for v in t1[i:i + 4]) + ", \\")
    lines.append("}")
    lines.append("#define WR_EXP_T2_INIT { \\")
    for i in range(0, 64, 4):
        lines.append("    " + ", ".join(f"0x{v:016x}ULL" for v in t2[i:i + 4]) + ", \\")
    lines.append("}")
    lines.append("#define WR_LOG_R_INIT { \\")
    for i in range(0, 512, 16):
        lines.append("    " + ", ".join(str(v) for v in rs[i:i + 16]) + ", \\")
    lines.append("}")
    lines.append("// (hi, lo) words of signed Q96 values")
    lines.append("#define WR_LOG_NL_INIT { \\")
    for i in range(512):
        lines.append(f"    {words(nl[i])}, \\")
    lines.append("}")
    lines.append(f"#define WR_L2E_Q127_HI 0x{l2e >> 64:016x}ULL")
    lines.append(f"#define WR_L2E_Q127_LO 0x{l2e & ((1 << 64) - 1):016x}ULL")
    lines.append(f"#define WR_LN2_Q64 0x{ln2_q64:016x}ULL")
    lines.append(f"#define WR_LN2_Q96_HI 0x{ln2_q96 >> 64:016x}ULL")
    lines.append(f"#define WR_LN2_Q96_LO 0x{ln2_q96 & ((1 << 64) - 1):016x}ULL")
    for k, v in enumerate(inv, 1):
        lines.append(f"#define WR_INV{k}_Q62 0x{v:016x}LL")
    return "\n".join(lines) + "\n"


if __name__ == "__main__":
    text = build()
    with open(OUT, "w") as f:
        f.write(text)
    print(OUT)
