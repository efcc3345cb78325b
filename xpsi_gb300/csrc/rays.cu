// rays.cu -- K1: Schwarzschild ray tables (deflection, cos alpha, lag) per
// mesh parallel.  Replaces xpsi/cellmesh/rays.pyx:249-390 (compute_rays) and
// its per-ray quadrature rayIntegrator (:90-247).
//
// Work decomposition: one CTA per mesh row ("parallel"), one thread per ray;
// each thread runs its 2 or 4 QUADPACK-QAG / Gauss-Kronrod-61 integrals to
// epsrel 1e-12, the reference's quadrature problem: interval bookkeeping and
// error control in FP64, every panel's integrand evaluations and weighted
// sums in double-float arithmetic (FP32 pipes, ~1e-14 relative).  The
// row's NaN repair (:333-369) is a short sequential walk done by one thread
// after the CTA barrier.  Optionally the lag is calibrated in the same pass
// (HotRegion.py:880-901: lag -= C(r), lag *= 2 pi f_mode).
#include "common.cuh"
#include "kernels.h"

namespace xg {

// The integrands of rays.pyx:60-88 in double-float arithmetic (values of
// order one on [0, 1], inside the float exponent range).  q is the
// reciprocal of (Rr - 1) or (rc - 1), formed once per ray in FP64.
struct OutDef {
  DF oms, sas, q;  // 1 - sin^2 alpha, sin^2 alpha, 1 / (1/u - 1)
  __device__ __forceinline__ DF root(DF x) const {
    const DF x2 = df_mul(x, x);
    const DF u = df_sub(DF{1.0f, 0.0f}, x2);
    const DF w = df_sub(df_sub(DF{2.0f, 0.0f}, x2), df_mul(df_mul(u, u), q));
    return df_sqrt(df_add(oms, df_mul(df_mul(x2, sas), w)));
  }
  __device__ DF operator()(DF x) const { return df_div(x, root(x)); }
};
struct OutLag {
  OutDef d;
  __device__ DF operator()(DF x) const {
    const DF f = d.root(x);
    return df_div(x, df_fma(f, f, f));
  }
};
struct InDef {
  DF q;  // 1 / (rc - 1)
  __device__ __forceinline__ DF value(DF x) const {
    const DF x2 = df_mul(x, x);
    const DF u = df_sub(DF{1.0f, 0.0f}, x2);
    const DF w = df_sub(df_sub(DF{2.0f, 0.0f}, x2), df_mul(df_mul(u, u), q));
    return df_div(DF{1.0f, 0.0f}, df_sqrt(w));
  }
  __device__ DF operator()(DF x) const { return value(x); }
};
struct InLag {
  InDef d;
  __device__ DF operator()(DF x) const {
    const DF X = d.value(x);
    return df_div(df_mul(X, X), df_add(x, X));
  }
};

// QUADPACK QAG with the 61-point rule at relative 1e-12, limit 100
// (rays.pyx:140-236), panels in double-float arithmetic
template <typename F>
__device__ __forceinline__ int q61(const F &f, double a, double b, double &r) {
  double e;
  auto panel = [&](double lo, double hi, double &res, double &err, double &ra, double &rc) {
    gk_panel_df<XG_K61_HALF>(f, XG_K61_X2, XG_K61_WK2, XG_K61_WG2, lo, hi, res, err, ra, rc);
  };
  return qag_panels<100>(panel, a, b, 0.0, 1.0e-12, r, e);
}

// rays.pyx:90-247; returns deflection in d, lag in seconds in l
__device__ void ray_integrate(double cos_alpha, double r_s, double u, double &d, double &l) {
  const int EFAILED = 5;
  int status = 0;
  double sas = 1.0 - cos_alpha * cos_alpha;
  double sa = sqrt(sas);
  double alpha = acos(cos_alpha);
  double b = sa / (u * sqrt(1.0 - u));
  d = 0.0;
  l = 0.0;
  if (b <= kBPhotonSphere) {
    const OutDef fd{df_split(1.0 - sas), df_split(sas), df_split(1.0 / (1.0 / u - 1.0))};
    const OutLag fl{fd};
    status = q61(fd, 0.0, 1.0, d);
    if (status == EFAILED) d = nan("");
    if (status != EFAILED) {
      status = q61(fl, 0.0, 1.0, l);
      if (status == EFAILED) d = nan("");
    }
    if (status != EFAILED) {
      d *= 2.0 * b * u;
      l *= 2.0 * b * b * u * r_s;
    }
  } else if (alpha <= kPi / 2.0) {
    double rc, wR;
    if (are_equal(sa, 1.0)) {
      rc = 1.0 / u;
      wR = 0.0;
    } else {
      rc = 2.0 * b * cos((atan(sqrt(4.0 * b * b / 27.0 - 1.0)) - kPi) / 3.0) / sqrt(3.0);
      wR = sqrt(1.0 - rc * u);
    }
    if (isnan(wR)) wR = 0.0;
    const InDef fd{df_split(1.0 / (rc - 1.0))};
    const InLag fl{fd};
    status = q61(fd, wR, 1.0, d);
    if (status == EFAILED) d = nan("");
    if (status != EFAILED) {
      status = q61(fl, wR, 1.0, l);
      if (status == EFAILED) d = nan("");
    }
    if (status != EFAILED) {
      d *= 2.0 * b / rc;
      l *= 2.0 * b * b * r_s / rc;
    }
  } else if (alpha > kPi / 2.0) {
    double rc = 2.0 * b * cos((atan(sqrt(4.0 * b * b / 27.0 - 1.0)) - kPi) / 3.0) / sqrt(3.0);
    double wR = sqrt(1.0 - rc * u);
    if (isnan(wR)) wR = 0.0;
    const InDef fd{df_split(1.0 / (rc - 1.0))};
    const InLag fl{fd};
    double d1, d0, l1, l0;
    status = q61(fd, 0.0, 1.0, d1);
    if (status == EFAILED) d = nan("");
    if (status != EFAILED) {
      status = q61(fd, wR, 1.0, d0);
      if (status == EFAILED) d = nan("");
    }
    if (status != EFAILED) {
      status = q61(fl, 0.0, 1.0, l1);
      if (status == EFAILED) d = nan("");
    }
    if (status != EFAILED) {
      status = q61(fl, wR, 1.0, l0);
      if (status == EFAILED) d = nan("");
    }
    if (status != EFAILED) {
      d = 2.0 * b * (2.0 * d1 - d0) / rc;
      l = 2.0 * b * b * r_s * (2.0 * l1 - l0) / rc;
      double cor = 1.0 / u - rc + log((1.0 / u - 1.0) / (rc - 1.0));
      l += 2.0 * r_s * cor;
    }
  }
  if (status != EFAILED) l /= kC;
}

__global__ void __launch_bounds__(128) rays_kernel(RaysArgs a) {
  const int row = blockIdx.x;
  if (row >= a.n_rows) return;
  const int N_R = a.N_R;
  const double u = a.u[row];
  const double r_s = a.r_s_row[row];
  double *D = a.deflection + (size_t)row * N_R;
  double *CA = a.cos_alpha + (size_t)row * N_R;
  double *L = a.lag + (size_t)row * N_R;
  __shared__ double s_inc;
  if (threadIdx.x == 0) {
    // rays.pyx:310-320
    double extreme = 0.0;
    if (u < 2.0 / 3.0)
      extreme = kPi - asin(sqrt(1.0 - u) * kBPhotonSphere * u);
    else if (are_equal(u, 2.0 / 3.0))
      extreme = kPi / 2.0;
    else if (2.0 / 3.0 < u && u < 1.0)
      extreme = asin(sqrt(1.0 - u) * kBPhotonSphere * u);
    double ma = a.maxAlpha[row];
    const double eps = 1.0e-8;
    if (ma >= (1.0 - eps) * extreme) ma = (1.0 - eps) * extreme;
    a.maxAlpha[row] = ma;
    s_inc = (1.0 - cos(ma)) / ((double)N_R - 1.0);
  }
  __syncthreads();
  const double inc = s_inc;
  for (int j = threadIdx.x; j < N_R; j += blockDim.x) {
    double ca = 1.0 - (double)j * inc;
    if (j == 0) {
      CA[0] = 1.0;
      D[0] = 0.0;
      L[0] = 0.0;
      continue;
    }
    CA[j] = ca;
    double d, l;
    ray_integrate(ca, r_s, u, d, l);
    D[j] = d;  // raw values; repaired below
    L[j] = l;
  }
  __syncthreads();
  // rays.pyx:322-371: a row whose values are all finite, in [0, 100 pi] and
  // rising at the last ray needs no repair (the walk below changes nothing
  // there); the CTA checks that in parallel and only other rows take the
  // sequential walk
  int bad = 0;
  for (int j = 1 + threadIdx.x; j < N_R; j += blockDim.x) {
    const double rp = D[j];
    bad |= (isnan(rp) || rp < 0.0 || rp > 100.0 * kPi) ? 1 : 0;
  }
  const int any_bad = __syncthreads_or(bad);
  if (!any_bad && threadIdx.x == 0) {
    const int term = N_R >= 2 && !(D[N_R - 1] > D[N_R - 2]);
    a.maxDeflection[row] = D[N_R - 1];
    if (a.row_status) a.row_status[row] = term ? kRayFail : kOk;
  }
  if (any_bad && threadIdx.x == 0) {
    // rays.pyx:322-371, sequential NaN repair by linear interpolation
    int term = 0;
    int icount = 0, iidx = 0;
    for (int j = 1; j < N_R; j++) {
      double rp = D[j], lp = L[j];
      if (j == N_R - 1 && (isnan(rp) || rp <= D[j - 1])) {
        term = 1;
        break;
      } else if (icount > 0 && !isnan(rp) && 0.0 <= rp && rp < 100.0 * kPi && rp > D[iidx]) {
        double delta = (double)icount + 1.0;
        for (int k = 1; k <= icount; k++) {
          double v = rp * (double)k;
          v += D[iidx] * (delta - (double)k);
          D[iidx + k] = v / delta;
          double w = lp * (double)k;
          w += L[iidx] * (delta - (double)k);
          L[iidx + k] = w / delta;
        }
        icount = 0;
      } else if (isnan(rp) || rp < 0.0 || rp > 100.0 * kPi) {
        if (icount == 0) iidx = j - 1;
        icount++;
      }
    }
    a.maxDeflection[row] = D[N_R - 1];
    if (a.row_status) a.row_status[row] = term ? kRayFail : kOk;
  }
  if (a.lag_C != nullptr) {
    // HotRegion.py:880-901 calibration fused into the same pass
    __syncthreads();
    const double C = a.lag_C[row], sc = a.lag_scale[row];
    for (int j = threadIdx.x; j < N_R; j += blockDim.x) L[j] = (L[j] - C) * sc;
  }
}

void launch_rays(const RaysArgs &a, cudaStream_t st) {
  if (a.n_rows <= 0) return;
  rays_kernel<<<a.n_rows, 128, 0, st>>>(a);
}

}  // namespace xg
