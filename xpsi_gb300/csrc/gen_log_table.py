"""Write the table of the double-float natural logarithm in likelihood.cu.

Nodes c_i = 0.75 + i / 128, i = 0..96 (exact in float), cover the reduced
argument f in [0.75, 1.5); the table holds ln(c_i) as a float pair
(high part the nearest float, low part the nearest float to the remainder),
computed here to 50 digits.

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
    with open(out, "w") as f:
        f.write("\n".join(lines) + "\n")


if __name__ == "__main__":
    main(sys.argv[1])
