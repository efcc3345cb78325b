// num4d_walk.cuh -- the numerical 4-D atmosphere evaluated with the
// reference's cached stencil walk (hot_Num4D.pyx:248-439), for kernels that
// visit the evaluations in the reference's call order and carry the previous
// call's coordinates.
#pragma once

#include "common.cuh"
#include "kernels.h"

namespace xg {

// base node of one dimension of the reference's cached stencil walk, given
// the previous call's coordinate vp on that dimension; v is clamped to the
// grid end when the walk that reaches the end moves the node (:300-351)
__device__ __forceinline__ int walk_base(const double *P, int n, double vp, double &v) {
  if (v > P[n - 1]) {
    if (!(vp >= P[n - 3])) v = P[n - 1];
    return n - 4;
  }
  if (v < P[0]) {
    if (!(vp < P[2])) v = P[0];
    return 0;
  }
  return stencil_base(P, n, v);
}

// hot_Num4D.pyx:248-439 for coordinates v[4] = (log T, log g, mu,
// log10(E / E_eff)) after a call at vp[4]
__device__ inline double num4d_walk(const Atmos4D &A, const double vp[4], double v0, double v1,
                             double v2, double v3) {
  double v[4] = {v0, v1, v2, v3};
  const double *g[4] = {A.logT, A.logg, A.mu, A.logE};
  const int n[4] = {A.nT, A.ng, A.nmu, A.nE};
  int b[4];
  double w[4][4];
#pragma unroll
  for (int d = 0; d < 4; d++) {
    b[d] = walk_base(g[d], n[d], vp[d], v[d]);
    lagrange4(g[d], b[d], v[d], w[d]);
  }
  const size_t S2 = (size_t)A.nE, S1 = (size_t)A.nmu * S2, S0 = (size_t)A.ng * S1;
  double I = 0.0;
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) {
      const double wij = w[0][i] * w[1][j];
      const double *base = A.I + (size_t)(b[0] + i) * S0 + (size_t)(b[1] + j) * S1 + b[3];
#pragma unroll
      for (int k = 0; k < 4; k++) {
        const double *p = base + (size_t)(b[2] + k) * S2;
        const double wijk = wij * w[2][k];
        I += wijk * w[3][0] * __ldg(p) + wijk * w[3][1] * __ldg(p + 1) +
             wijk * w[3][2] * __ldg(p + 2) + wijk * w[3][3] * __ldg(p + 3);
      }
    }
  if (I < 0.0) return 0.0;
  return I * pow(10.0, 3.0 * v[0]);
}

}  // namespace xg
