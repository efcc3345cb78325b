"""Compute Gauss-Kronrod (G_n, K_{2n+1}) nodes and weights in high precision.

Nodes for the ray (61-point) and window (21-point) quadratures; it writes the 61-point
Kronrod extension of the 30-point Gauss-Legendre rule (the rule the ray
integrals use, QUADPACK key 6) and the 21-point extension of the 10-point
rule.  They are derived here from their definition, not taken from any
library table:

* Gauss nodes are the roots of P_n, weights 2 / ((1 - x^2) P_n'(x)^2).
* Kronrod nodes add the n+1 roots of the Stieltjes polynomial E_{n+1},
  defined by  int_{-1}^{1} P_n(x) E_{n+1}(x) x^k dx = 0,  k = 0..n.
* Kronrod weights make the 2n+1 point rule exact for P_0..P_{2n}.

Usage:  python gen_gk_nodes.py OUT.h PREFIX
"""
import sys
import mpmath as mp
import numpy as np

mp.mp.dps = 60


def legendre_all(x, nmax):
    p = [mp.mpf(1), x]
    for k in range(1, nmax):
        p.append(((2 * k + 1) * x * p[k] - k * p[k - 1]) / (k + 1))
    return p[: nmax + 1]


def gauss(n):
    xs, ws = [], []
    for i in range(1, n + 1):
        x = mp.cos(mp.pi * (i - mp.mpf(1) / 4) / (n + mp.mpf(1) / 2))
        for _ in range(100):
            p = legendre_all(x, n)
            dp = n * (x * p[n] - p[n - 1]) / (x * x - 1)
            dx = p[n] / dp
            x -= dx
            if abs(dx) < mp.mpf(10) ** (-55):
                break
        p = legendre_all(x, n)
        dp = n * (x * p[n] - p[n - 1]) / (x * x - 1)
        xs.append(x)
        ws.append(2 / ((1 - x * x) * dp * dp))
    return xs, ws


def kronrod(n):
    gx, gw = gauss(n)
    # a Gauss rule exact to high degree for the moment integrals
    qx, qw = gauss(3 * n + 8)
    # E(x) = sum_{k=0}^{n+1} e_k P_k(x), e_{n+1} = 1
    Pq = [legendre_all(x, n + 1) for x in qx]
    A = mp.matrix(n + 1, n + 1)
    b = mp.matrix(n + 1, 1)
    for j in range(n + 1):
        for k in range(n + 1):
            A[j, k] = mp.fsum(qw[m] * Pq[m][n] * Pq[m][j] * Pq[m][k] for m in range(len(qx)))
        b[j] = -mp.fsum(qw[m] * Pq[m][n] * Pq[m][j] * Pq[m][n + 1] for m in range(len(qx)))
    e = list(mp.lu_solve(A, b)) + [mp.mpf(1)]

    def E(x):
        p = legendre_all(x, n + 1)
        return mp.fsum(e[k] * p[k] for k in range(n + 2))

    # roots of E interlace the Gauss nodes (sorted descending), plus the two ends
    edges = [mp.mpf(1)] + sorted(gx, reverse=True) + [mp.mpf(-1)]
    kx = []
    for i in range(len(edges) - 1):
        hi, lo = edges[i], edges[i + 1]
        r = mp.findroot(E, (lo + mp.mpf(10) ** -40, hi - mp.mpf(10) ** -40), solver="anderson")
        kx.append(r)
    nodes = sorted(kx + list(gx), reverse=True)
    N = len(nodes)
    M = mp.matrix(N, N)
    rhs = mp.matrix(N, 1)
    Pn = [legendre_all(x, N - 1) for x in nodes]
    for j in range(N):
        for i in range(N):
            M[j, i] = Pn[i][j]
        rhs[j] = 2 if j == 0 else 0
    kw = list(mp.lu_solve(M, rhs))
    return nodes, kw, gx, gw


def main():
    out, prefix = sys.argv[1], sys.argv[2]
    lines = ["/* Generated by gen_gk_nodes.py: Gauss-Kronrod nodes derived in",
             " * 60-digit arithmetic from the definitions in that script. */",
             "#pragma once",
             "#ifdef __CUDACC__",
             "#define GK_TABLE static __constant__ const double",
             "#define GK_TABLE_F static __constant__ const float",
             "#else",
             "#define GK_TABLE static const double",
             "#define GK_TABLE_F static const float",
             "#endif", ""]
    for n in (10, 30):
        nodes, kw, gx, gw = kronrod(n)
        # keep x >= 0 half: index 0 = largest node; the centre node is last
        half = n + 1
        xk = nodes[:half]
        wk = kw[:half]
        isg = [any(abs(x - g) < mp.mpf(10) ** -40 for g in gx) for x in xk]
        wg = []
        for x, g in zip(xk, isg):
            if g:
                j = min(range(len(gx)), key=lambda t: abs(gx[t] - x))
                wg.append(gw[j])
            else:
                wg.append(mp.mpf(0))
        K = 2 * n + 1
        tag = f"{prefix}K{K}"
        lines.append(f"#define {tag}_HALF {half}")
        # values below 1e-30 are round-off of exact zeros
        fmt = lambda v: mp.nstr(v if abs(v) > mp.mpf(10) ** -30 else mp.mpf(0), 25,
                                min_fixed=1, max_fixed=0)
        lines.append(f"GK_TABLE {tag}_X[{half}] = {{")
        lines += [f"    {fmt(v)}," for v in xk] + ["};"]
        lines.append(f"GK_TABLE {tag}_WK[{half}] = {{")
        lines += [f"    {fmt(v)}," for v in wk] + ["};"]
        lines.append(f"/* Gauss weight of the node, 0 where the node is Kronrod-only */")
        lines.append(f"GK_TABLE {tag}_WG[{half}] = {{")
        lines += [f"    {fmt(v)}," for v in wg] + ["};"]
        # the same values as float pairs hi + lo (hi the nearest float, lo the
        # nearest float to the remainder) for double-float arithmetic
        lines.append(f"/* float pairs (hi, lo) of _X, _WK, _WG */")
        for nm, vals in (("X", xk), ("WK", wk), ("WG", wg)):
            lines.append(f"GK_TABLE_F {tag}_{nm}2[{2 * half}] = {{")
            for v in vals:
                v = v if abs(v) > mp.mpf(10) ** -30 else mp.mpf(0)
                hi = float(np.float32(float(v)))
                lo = float(np.float32(float(v - mp.mpf(hi))))
                lines.append(f"    {hi!r}f, {lo!r}f,")
            lines.append("};")
        lines.append("")
        # self-check: exactness of the Kronrod rule to degree 3n+1, Gauss to 2n-1
        for deg in range(0, 3 * n + 2):
            s = mp.fsum(w * x ** deg for w, x in zip(kw, nodes))
            exact = mp.mpf(2) / (deg + 1) if deg % 2 == 0 else 0
            assert abs(s - exact) < mp.mpf(10) ** -40, (n, deg)
    with open(out, "w") as fh:
        fh.write("\n".join(lines) + "\n")


if __name__ == "__main__":
    main()
