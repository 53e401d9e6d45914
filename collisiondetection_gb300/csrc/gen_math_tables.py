"""Writes ccd_math_tables.h: the exact constants of the table-driven exp/log.

  log table, j = 0..127:  m in [1 + j/128, 1 + (j+1)/128) is reduced by
      inv_j = fl(1 / c_j),  c_j = 1 + (j + 1/2)/128  (j = 1..63)
                            c_j = (1 + (j + 1/2)/128) / 2 applied to m/2  (j = 64..126)
                            c_0 = 1, c_127 = 1 (no reduction next to 1, so that
                            log(1 + d) keeps full relative accuracy)
      and stores nlog_j = -log(inv_j) as a double-double.
  exp table, j = 0..31:  2^(j/32) as a double-double.

Needs mpmath (development only; the header is committed):
    python collisiondetection_gb300/csrc/gen_math_tables.py
"""
import os
from fractions import Fraction

import mpmath

mpmath.mp.prec = 400


def dd(x):
    x = mpmath.mpf(x)
    hi = float(x)
    lo = float(x - mpmath.mpf(hi))
    return hi, lo


def main():
    lines = ["// Generated by gen_math_tables.py -- exact constants of the table-driven",
             "// exp/log in ccd_math.h.  Do not edit.", "#pragma once", "",
             "// log: {inv_j, -log(inv_j) hi, -log(inv_j) lo}, j = 0..127",
             "#define CCD_LOG_TABLE_DATA { \\"]
    for j in range(128):
        if j == 0 or j == 127:
            inv = 1.0
        elif j < 64:
            c = Fraction(1) + Fraction(2 * j + 1, 256)
            inv = float(1 / mpmath.mpf(c.numerator) * c.denominator)
        else:
            c = (Fraction(1) + Fraction(2 * j + 1, 256)) / 2
            inv = float(1 / mpmath.mpf(c.numerator) * c.denominator)
        hi, lo = dd(-mpmath.log(mpmath.mpf(inv)))
        lines.append(f"  {inv.hex()}, {hi.hex()}, {lo.hex()}, \\")
    lines.append("}")
    lines.append("")
    lines.append("// exp: {2^(j/32) hi, lo}, j = 0..31")
    lines.append("#define CCD_EXP_TABLE_DATA { \\")
    for j in range(32):
        hi, lo = dd(mpmath.power(2, mpmath.mpf(j) / 32))
        lines.append(f"  {hi.hex()}, {lo.hex()}, \\")
    lines.append("}")
    # ln2/32 split: L1, L2 with 36 significant bits (exact products with |N| < 2^17), L3 the rest
    v = mpmath.log(2) / 32
    parts = []
    for _ in range(2):
        f = float(v)
        m, e = mpmath.frexp(mpmath.mpf(f))
        q = mpmath.mpf(2) ** (e - 36)
        f = float(mpmath.floor(mpmath.mpf(f) / q + mpmath.mpf(0.5)) * q)
        parts.append(f)
        v = v - mpmath.mpf(f)
    parts.append(float(v))
    lines.append("")
    lines.append("// ln2/32 = L1 + L2 + L3, L1 and L2 with 36 significant bits")
    for name, p in zip(("L1", "L2", "L3"), parts):
        lines.append(f"#define CCD_LN2_32_{name} {p.hex()}")
    lines.append(f"#define CCD_32_OVER_LN2 {float(32 / mpmath.log(2)).hex()}")
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ccd_math_tables.h")
    with open(out, "w") as fh:
        fh.write("\n".join(lines) + "\n")
    print("wrote", out)


if __name__ == "__main__":
    main()
