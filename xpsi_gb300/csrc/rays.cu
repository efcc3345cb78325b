// rays.cu -- K1: Schwarzschild ray tables (deflection, cos alpha, lag) per
// mesh parallel.  Replaces xpsi/cellmesh/rays.pyx:249-390 (compute_rays) and
// its per-ray quadrature rayIntegrator (:90-247).
//
// Work decomposition: one CTA per mesh row ("parallel"), one thread per ray;
// each thread runs its 2 or 4 QUADPACK-QAG / Gauss-Kronrod-61 integrals to
// epsrel 1e-12, the reference's quadrature problem, with the deflection and
// lag integrals over the same interval taken as a pair (their integrands
// share the square root, so each node is evaluated once for both):
// interval bookkeeping and error control in FP64, every panel's integrand
// evaluations and weighted sums in double-float arithmetic (FP32 pipes,
// ~1e-14 relative).  The row's NaN repair (:333-369) is a sequential walk
// done by one thread, for the rows that need one.  Optionally the lag is
// calibrated in the same pass (HotRegion.py:880-901: lag -= C(r), lag *=
// 2 pi f_mode).
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

// The deflection and lag integrands of a ray share their square root (Out*)
// or their inner value (In*): a pair evaluates both at each node once.
struct OutPair {
  OutDef d;
  __device__ void operator()(DF x, DF &fd, DF &fl) const {
    const DF f = d.root(x);
    fd = df_div(x, f);
    fl = df_div(x, df_fma(f, f, f));
  }
};
struct InPair {
  InDef d;
  __device__ void operator()(DF x, DF &fd, DF &fl) const {
    const DF X = d.value(x);
    fd = X;
    fl = df_div(df_mul(X, X), df_add(x, X));
  }
};

// gk_panel_df for the two integrands of a pair at once (the same nodes,
// weights and error estimate per integrand)
template <typename P>
__device__ __forceinline__ void gk61_pair_panel(const P &pf, double a, double b, double res[2],
                                                double err[2], double rabs[2], double rasc[2]) {
  constexpr int NH = XG_K61_HALF - 1;
  const double cd = 0.5 * (a + b), hd = 0.5 * (b - a);
  const DF c = df_split(cd), h = df_split(hd);
  float fv1[2][NH], fv2[2][NH];
  DF fc[2];
  pf(c, fc[0], fc[1]);
  DF rk[2], rg[2];
  float ra[2];
  const DF wkc{XG_K61_WK2[2 * NH], XG_K61_WK2[2 * NH + 1]};
  const DF wgc{XG_K61_WG2[2 * NH], XG_K61_WG2[2 * NH + 1]};
#pragma unroll
  for (int q = 0; q < 2; q++) {
    rk[q] = df_mul(wkc, fc[q]);
    rg[q] = df_mul(wgc, fc[q]);
    ra[q] = fabsf(rk[q].h);
  }
#pragma unroll 1
  for (int j = 0; j < NH; j++) {
    const DF dx = df_mul(h, DF{XG_K61_X2[2 * j], XG_K61_X2[2 * j + 1]});
    DF f1[2], f2[2];
    pf(df_sub(c, dx), f1[0], f1[1]);
    pf(df_add(c, dx), f2[0], f2[1]);
    const DF wk{XG_K61_WK2[2 * j], XG_K61_WK2[2 * j + 1]};
    const DF wg{XG_K61_WG2[2 * j], XG_K61_WG2[2 * j + 1]};
#pragma unroll
    for (int q = 0; q < 2; q++) {
      fv1[q][j] = f1[q].h;
      fv2[q][j] = f2[q].h;
      const DF s2 = df_add(f1[q], f2[q]);
      rk[q] = df_fma(wk, s2, rk[q]);
      if (wg.h != 0.0f) rg[q] = df_fma(wg, s2, rg[q]);
      ra[q] += wk.h * (fabsf(f1[q].h) + fabsf(f2[q].h));
    }
  }
  const double ah = fabs(hd);
  const double eps = 2.220446049250313e-16, dmin = 2.2250738585072014e-308;
#pragma unroll
  for (int q = 0; q < 2; q++) {
    const float mean = 0.5f * rk[q].h;
    float rc = wkc.h * fabsf(fc[q].h - mean);
#pragma unroll 1
    for (int j = 0; j < NH; j++)
      rc += XG_K61_WK2[2 * j] * (fabsf(fv1[q][j] - mean) + fabsf(fv2[q][j] - mean));
    res[q] = df_value(rk[q]) * hd;
    const double rad = (double)ra[q] * ah, rcd = (double)rc * ah;
    // QUADPACK's err = rasc min(1, (200 |K - G| / rasc)^1.5): the ratio is
    // free of the half-width (it cancels), so it is formed in float from the
    // double-float and float sums; only the product with rasc is FP64
    const DF dk = df_sub(rk[q], rg[q]);
    double e;
    if (rc != 0.0f && dk.h != 0.0f) {
      const float x = 200.0f * fabsf(dk.h) / rc, sc = x * sqrtf(x);
      e = sc < 1.0f ? rcd * (double)sc : rcd;
    } else {
      e = fabs(df_value(dk) * hd);
    }
    if (rad > dmin / (50.0 * eps)) {
      const double fl = 50.0 * eps * rad;
      if (fl > e) e = fl;
    }
    err[q] = e;
    rabs[q] = rad;
    rasc[q] = rcd;
  }
}

// QUADPACK QAG at relative 1e-12, limit 100 (rays.pyx:140-236) for the two
// integrals of a pair over the same interval: the first panel's tests are
// QUADPACK's for each integral, and while either error is above its
// tolerance the interval whose larger error relative to its own tolerance
// is largest is bisected (both integrals refined there).  Each integral is
// thus at least as accurate as its own QAG run would leave it.  Statuses:
// 0, 11 (limit), 18 (round-off), 21 (bad integrand), as qag_panels.
template <typename P>
__device__ int q61_pair(const P &pf, double a, double b, double &r1, double &r2) {
  constexpr int LIMIT = 100;
  const double eps = 2.220446049250313e-16, dmin = 2.2250738585072014e-308;
  const double epsrel = 1.0e-12;
  double al[LIMIT], bl[LIMIT], rl[2][LIMIT], el[2][LIMIT];
  double r0[2], e0[2], ra0[2], rc0[2];
  gk61_pair_panel(pf, a, b, r0, e0, ra0, rc0);
  bool done[2];
  int st0[2];
#pragma unroll
  for (int q = 0; q < 2; q++) {
    const double tol = epsrel * fabs(r0[q]);
    st0[q] = -1;
    if (e0[q] <= 50.0 * eps * ra0[q] && e0[q] > tol) st0[q] = 18;
    else if ((e0[q] <= tol && e0[q] != rc0[q]) || e0[q] == 0.0) st0[q] = 0;
    done[q] = st0[q] >= 0;
  }
  if (done[0] && done[1]) {
    r1 = r0[0];
    r2 = r0[1];
    return st0[0] > st0[1] ? st0[0] : st0[1];
  }
  int size = 1;
  al[0] = a; bl[0] = b;
  rl[0][0] = r0[0]; el[0][0] = e0[0];
  rl[1][0] = r0[1]; el[1][0] = e0[1];
  double area[2] = {r0[0], r0[1]}, errsum[2] = {e0[0], e0[1]};
  int rnd1 = 0, rnd2 = 0, fail = 0, iter = 1, k = 0;
  auto tol_of = [&](int q) { return epsrel * fabs(area[q]); };
  // an interval's priority: the larger of its two errors over their
  // tolerances (the reciprocals taken once per bisection step)
  auto prio = [&](int i, double i0, double i1) { return fmax(el[0][i] * i0, el[1][i] * i1); };
  do {
    const double ai = al[k], bi = bl[k];
    const double a1 = ai, b1 = 0.5 * (ai + bi), a2 = b1, b2 = bi;
    double R1[2], E1[2], RA1[2], RC1[2], R2[2], E2[2], RA2[2], RC2[2];
    gk61_pair_panel(pf, a1, b1, R1, E1, RA1, RC1);
    gk61_pair_panel(pf, a2, b2, R2, E2, RA2, RC2);
#pragma unroll
    for (int q = 0; q < 2; q++) {
      const double ri = rl[q][k], ei = el[q][k];
      const double r12 = R1[q] + R2[q], e12 = E1[q] + E2[q];
      errsum[q] += e12 - ei;
      area[q] += r12 - ri;
      if (RC1[q] != E1[q] && RC2[q] != E2[q]) {
        if (fabs(ri - r12) <= 1.0e-5 * fabs(r12) && e12 >= 0.99 * ei) rnd1++;
        if (iter >= 10 && e12 > ei) rnd2++;
      }
    }
    const bool above = errsum[0] > tol_of(0) || errsum[1] > tol_of(1);
    if (above) {
      if (rnd1 >= 12 || rnd2 >= 40) fail = 2;
      const double edge = (1.0 + 100.0 * eps) * (fabs(a2) + 1000.0 * dmin);
      if (fabs(a1) <= edge && fabs(b2) <= edge) fail = 3;
    }
    const int nw = size++;
    al[k] = a1; bl[k] = b1;
    al[nw] = a2; bl[nw] = b2;
#pragma unroll
    for (int q = 0; q < 2; q++) {
      rl[q][k] = R1[q]; el[q][k] = E1[q];
      rl[q][nw] = R2[q]; el[q][nw] = E2[q];
    }
    k = 0;
    const double i0 = 1.0 / fmax(tol_of(0), dmin), i1 = 1.0 / fmax(tol_of(1), dmin);
    double pk = prio(0, i0, i1);
    for (int i = 1; i < size; i++) {
      const double pi = prio(i, i0, i1);
      if (pi > pk) { pk = pi; k = i; }
    }
    iter++;
    if (!(iter < LIMIT && !fail && above)) break;
  } while (true);
  double s0 = 0.0, s1 = 0.0;
  for (int i = 0; i < size; i++) {
    s0 += rl[0][i];
    s1 += rl[1][i];
  }
  r1 = s0;
  r2 = s1;
  if (!(errsum[0] > tol_of(0) || errsum[1] > tol_of(1))) return 0;
  if (fail == 2) return 18;
  if (fail == 3) return 21;
  if (iter == LIMIT) return 11;
  return 5;
}


// rays.pyx:90-247; returns deflection in d, lag in seconds in l
// the turning radius r_c / r_s of a ray of impact parameter b / r_s
// (rays.pyx:156, :194): 2 b cos((atan(sqrt(4 b^2 / 27 - 1)) - pi) / 3) / sqrt 3,
// the divisions by the constants 27, 3 and sqrt 3 taken as products with
// their reciprocals (an ulp apart)
__device__ __forceinline__ double turning_radius(double b) {
  constexpr double i27 = 1.0 / 27.0, i3 = 1.0 / 3.0;
  const double isq3 = 0.57735026918962576451;  // 1 / sqrt(3)
  return 2.0 * b * cos((atan(sqrt(4.0 * b * b * i27 - 1.0)) - kPi) * i3) * isq3;
}

// u_sq1u = u sqrt(1 - u), formed once per row (rays.pyx forms it per ray)
__device__ void ray_integrate(double cos_alpha, double r_s, double u, double u_sq1u, double &d,
                              double &l) {
  const int EFAILED = 5;
  int status = 0;
  double sas = 1.0 - cos_alpha * cos_alpha;
  double sa = sqrt(sas);
  // alpha = acos(cos_alpha) enters only through alpha <= pi/2 and alpha >
  // pi/2, which are cos_alpha >= 0 and cos_alpha < 0 except where acos
  // rounds to pi/2 from a cosine a few ulps below zero: there it is formed
  double alpha = cos_alpha >= 0.0 ? 0.0 : kPi;
  if (fabs(cos_alpha) < 1.0e-15) alpha = acos(cos_alpha);
  double b = sa / u_sq1u;
  d = 0.0;
  l = 0.0;
  if (b <= kBPhotonSphere) {
    const OutDef fd{df_split(1.0 - sas), df_split(sas), df_split(1.0 / (1.0 / u - 1.0))};
    status = q61_pair(OutPair{fd}, 0.0, 1.0, d, l);
    if (status == EFAILED) d = nan("");
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
      rc = turning_radius(b);
      wR = sqrt(1.0 - rc * u);
    }
    if (isnan(wR)) wR = 0.0;
    const InDef fd{df_split(1.0 / (rc - 1.0))};
    status = q61_pair(InPair{fd}, wR, 1.0, d, l);
    if (status == EFAILED) d = nan("");
    if (status != EFAILED) {
      const double irc = 1.0 / rc;
      d *= 2.0 * b * irc;
      l *= 2.0 * b * b * r_s * irc;
    }
  } else if (alpha > kPi / 2.0) {
    double rc = turning_radius(b);
    double wR = sqrt(1.0 - rc * u);
    if (isnan(wR)) wR = 0.0;
    const InDef fd{df_split(1.0 / (rc - 1.0))};
    double d1, d0, l1, l0;
    status = q61_pair(InPair{fd}, 0.0, 1.0, d1, l1);
    if (status == EFAILED) d = nan("");
    if (status != EFAILED) {
      status = q61_pair(InPair{fd}, wR, 1.0, d0, l0);
      if (status == EFAILED) d = nan("");
    }
    if (status != EFAILED) {
      const double irc = 1.0 / rc;
      d = 2.0 * b * (2.0 * d1 - d0) * irc;
      l = 2.0 * b * b * r_s * (2.0 * l1 - l0) * irc;
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
  const double u_sq1u = u * sqrt(1.0 - u);
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
    ray_integrate(ca, r_s, u, u_sq1u, d, l);
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
