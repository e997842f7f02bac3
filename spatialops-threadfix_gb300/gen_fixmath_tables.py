"""Writes include/spatialops/detail/NeboFixMathTables.h: the tables of the fixed-point FP64 exp
and sin (include/spatialops/NeboFixMath.h) as literals, so that no run-time set-up or upload is
needed wherever the header is compiled.

    python spatialops-threadfix_gb300/gen_fixmath_tables.py

  exp2j[j] = round(2^(j/256) * 2^62),      j = 0..255  (Tang's table, ACM TOMS 15(2), 1989)
  sinj[j]  = round(sin(j pi/256) * 2^62),  j = 0..127
  cosj[j]  = round(cos(j pi/256) * 2^62),  j = 0..127
Each is rounded to nearest from 400-bit arithmetic (mpmath).
"""
import os

import mpmath

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(os.path.dirname(HERE), "include", "spatialops", "detail", "NeboFixMathTables.h")


def tables():
    mpmath.mp.prec = 400
    s62 = mpmath.mpf(2) ** 62
    exp2j = [int(mpmath.nint(mpmath.power(2, mpmath.mpf(j) / 256) * s62)) for j in range(256)]
    sinj = [int(mpmath.nint(mpmath.sin(j * mpmath.pi / 256) * s62)) for j in range(128)]
    cosj = [int(mpmath.nint(mpmath.cos(j * mpmath.pi / 256) * s62)) for j in range(128)]
    return exp2j, sinj, cosj


def _init(name, vals):
    rows = []
    for i in range(0, len(vals), 4):
        rows.append("    " + ", ".join(f"{v}LL" for v in vals[i:i + 4]) + ",")
    return f"#define {name} \\\n  {{ \\\n" + " \\\n".join(rows) + " \\\n  }\n"


def main():
    exp2j, sinj, cosj = tables()
    text = ("// Generated by spatialops-threadfix_gb300/gen_fixmath_tables.py -- do not edit.\n"
            "// Initialisers of the fixed-point exp / sin tables at 2^62 (see NeboFixMath.h).\n"
            "#pragma once\n\n" + _init("NEBO_FIX_EXP2J", exp2j) + "\n" + _init("NEBO_FIX_SINJ", sinj) + "\n" +
            _init("NEBO_FIX_COSJ", cosj))
    with open(OUT, "w") as f:
        f.write(text)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
