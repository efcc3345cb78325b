"""Write the tables of the double-float logarithm and exponential in
likelihood.cu.

Nodes c_i = 0.75 + i / 128, i = 0..96 (exact in float), cover the reduced
argument f in [0.75, 1.5); the table holds ln(c_i) as a float pair
(high part the nearest float, low part the nearest float to the remainder),
computed here to 50 digits.  For the exponential: 1 / n!, n = 0..13, as
float pairs (the Taylor coefficients of exp on |r| <= ln 2 / 2), and
ln 2 in three parts for the argument reduction k ln 2 (the first two with
12 significant bits, so that k times each is exact for |k| < 2^11).

Usage:  python gen_log_table.py OUT.h
"""
import sys
import mpmath as mp
import numpy as np

mp.mp.dps = 50


def pair(v):
    hi = np.float32(float(v))
    lo = np.float32(float(v - mp.mpf(float(hi))))
    return hi, lo


def main(out):
    lines = ["// generated by gen_log_table.py: ln(0.75 + i / 128) as float pairs",
             "#pragma once", "", "#define XG_LOGT_N 97",
             "static __constant__ const float XG_LOGT[XG_LOGT_N][2] = {"]
    for i in range(97):
        c = mp.mpf(3) / 4 + mp.mpf(i) / 128
        hi, lo = pair(mp.log(c))
        lines.append("    {%.9ef, %.9ef}," % (hi, lo))
    lines.append("};")
    lines.append("")
    lines.append("#define XG_EXPT_N 14")
    lines.append("static __constant__ const float XG_EXPT[XG_EXPT_N][2] = {")
    for n in range(14):
        hi, lo = pair(1 / mp.factorial(n))
        lines.append("    {%.9ef, %.9ef}," % (hi, lo))
    lines.append("};")
    ln2 = mp.log(2)
    c1 = mp.mpf(round(float(ln2) * 2**12)) / 2**12
    c2 = mp.mpf(round(float(ln2 - c1) * 2**24)) / 2**24
    c3 = ln2 - c1 - c2
    lines.append("// ln 2 = XG_LN2_1 + XG_LN2_2 + XG_LN2_3")
    lines.append("#define XG_LN2_1 %.9ef" % float(c1))
    lines.append("#define XG_LN2_2 %.9ef" % float(c2))
    h3, l3 = pair(c3)
    lines.append("#define XG_LN2_3 %.9ef" % h3)
    lines.append("#define XG_LN2_4 %.9ef" % l3)
    with open(out, "w") as f:
        f.write("\n".join(lines) + "\n")


if __name__ == "__main__":
    main(sys.argv[1])
