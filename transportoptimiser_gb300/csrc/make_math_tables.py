"""Writes to_math_tables.h: the 128-entry tables of the table-assisted log
and sine/cosine that Box-Muller uses in to_math.h.

    python transportoptimiser_gb300/csrc/make_math_tables.py

log: for the mantissa m in [1, 2) of a float, entry i = the top 7 mantissa
bits covers [1 + i/128, 1 + (i+1)/128) with centre c_i = 1 + (i + 1/2)/128;
R_i = 1/c_i rounded to float and G_i = -log(R_i), less log 2 for the
entries with c_i > sqrt(2) (whose mantissa is then read as m/2 in
[sqrt(1/2), 1) with the exponent one higher, so that log(x) near 1 is a sum
of small terms).  log(x) = E log 2 + G_i + log1p(m R_i - 1), |m R_i - 1| < 1/200.

sin/cos: entry j = sin and cos of 2 pi j / 128.

Every value is computed in double and rounded once to float.  The same
literals serve the CUDA kernels and the C oracle.
"""
from __future__ import annotations

import math
from pathlib import Path

import numpy as np

OUT = Path(__file__).resolve().parent / "to_math_tables.h"
N = 128
SPLIT = next(i for i in range(N) if 1.0 + (i + 0.5) / N > math.sqrt(2.0))


def c_float(v: float) -> str:
    f = float(np.float32(v))
    if f == 0.0:
        return "0.0f"
    s = f.hex()                      # e.g. 0x1.6a09e60000000p-1
    mant, exp = s.split("p")
    mant = mant.rstrip("0")
    if mant.endswith("."):
        mant += "0"
    return "%sp%sf" % (mant, exp)


def main():
    rows = []
    for i in range(N):
        c = 1.0 + (i + 0.5) / N
        r = float(np.float32(1.0 / c))
        g = -math.log(r) - (math.log(2.0) if i >= SPLIT else 0.0)
        rows.append((r, g))
    sc = [(math.sin(2.0 * math.pi * j / N), math.cos(2.0 * math.pi * j / N)) for j in range(N)]
    lines = [
        "/* to_math_tables.h - written by make_math_tables.py; do not edit. */",
        "#ifndef TO_MATH_TABLES_H",
        "#define TO_MATH_TABLES_H",
        "/* first log entry whose centre exceeds sqrt(2) */",
        "#define TO_LOG_SPLIT %d" % SPLIT,
        "/* {R_i, G_i}: 1 / centre of mantissa interval i, -log(R_i) (less log 2 from TO_LOG_SPLIT on) */",
        "#define TO_LOG_TABLE_INIT { \\",
    ]
    lines += ["    {%s, %s}, \\" % (c_float(r), c_float(g)) for r, g in rows]
    lines += ["}", "/* {sin, cos} of 2 pi j / 128 */", "#define TO_SINCOS_TABLE_INIT { \\"]
    lines += ["    {%s, %s}, \\" % (c_float(s), c_float(c)) for s, c in sc]
    lines += ["}", "#endif /* TO_MATH_TABLES_H */", ""]
    OUT.write_text("\n".join(lines))
    print("wrote", OUT, "split", SPLIT)


if __name__ == "__main__":
    main()
