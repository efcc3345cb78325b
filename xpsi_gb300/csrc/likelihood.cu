// likelihood.cu -- K6: expected counts per phase bin and the background-
// marginalised Poisson log-likelihood, replacing
//   xpsi/tools/compute_expected_counts.pyx:66-197 and
//   xpsi/likelihoods/default_background_marginalisation.pyx:38-734.
//
// One warp per (likelihood evaluation, channel).  Lanes integrate the
// Akima-periodic phase interpolant of each component over their phase bins
// and hold one phase bin each for the channel sums (Newton steps, Gaussian
// width, the normalisation A), which are reduced with xor-butterfly shuffles
// so every lane holds the same bits and control flow stays warp-uniform;
// the marginal integral is a QUADPACK-style adaptive Gauss-Kronrod-21 quadrature run to
// relative 1e-13 whose 21 node evaluations per panel are spread over the
// lanes.  The reference's CQUAD call (:416-419) asks for relative 1e-8 on
// this smooth integrand, so both converge to the same integral.  The channel
// terms are summed per evaluation in channel order by a second kernel, which
// also applies the reference's early exits (slim cut :677-684, vanished
// integral :423-429).
#include <climits>

#include "common.cuh"
#include "kernels.h"
#include "log_table.h"

namespace xg {
namespace {

// Natural logarithm of a positive, normal double-float m with a table:
// m = 2^e f, f in [0.75, 1.5) (as df_log), then f = c (f / c) with c the
// nearest node 0.75 + i / 128 (|f / c - 1| <= 1 / 192) and
//   ln f = ln c + 2 atanh(s),  s = (f - c) / (f + c),  |s| <= 1 / 385,
// the series 2 s (1 + s^2 / 3 + s^4 / 5) truncated below 1e-17 relative
// (the s^4 / 5 term in float, its rounding ~1e-19); ln c from the table
// (gen_log_table.py, float pairs).  About half the work of df_log's
// 11-term series.  tab: the table in shared memory.
__device__ __forceinline__ DF df_log_t(DF m, const DF *tab) {
  const DF ln2{0.6931471824645996f, -1.9046542121259336e-09f};
  const DF third{0.3333333432674408f, -9.934107758624577e-09f};
  const int bits = __float_as_int(m.h);
  int e = ((bits >> 23) & 0xff) - 127;
  if ((bits & 0x7fffff) >= 0x400000) e += 1;
  const float sc = __int_as_float((127 - e) << 23);
  const DF f{__fmul_rn(m.h, sc), __fmul_rn(m.l, sc)};
  int i = __float2int_rn((f.h - 0.75f) * 128.0f);
  i = min(max(i, 0), XG_LOGT_N - 1);
  const float c = 0.75f + (float)i * 0.0078125f;
  const DF s = df_div(df_add(f, DF{-c, 0.0f}), df_add(f, DF{c, 0.0f}));
  const DF s2 = df_mul(s, s);
  const float s4_5 = __fmul_rn(__fmul_rn(s2.h, s2.h), 0.2f);
  const DF p = df_add(DF{1.0f, 0.0f}, df_add(df_mul(s2, third), DF{s4_5, 0.0f}));
  return df_add(df_fma(DF{(float)e, 0.0f}, ln2, tab[i]), df_mul(df_add(s, s), p));
}

// exp(x) of a double-float x, returned as a double: x = k ln 2 + r with
// |r| <= ln 2 / 2 (ln 2 in parts, gen_log_table.py: k times the first two
// exact for |k| < 2^11), exp(r) by its Taylor series through r^13 / 13! in
// double-float (truncation below 4e-18 relative), then 2^k in FP64; 0 below
// the double range, the FP64 exp beyond ln 2^1000.
__device__ __forceinline__ double df_exp_d(DF x) {
  if (x.h != x.h) return (double)x.h;
  if (x.h < -760.0f) return 0.0;
  if (x.h > 690.0f) return exp((double)x.h + (double)x.l);
  const float kf = rintf(x.h * 1.44269504088896341f);
  const int k = (int)kf;
  DF r = df_add(x, DF{-kf * XG_LN2_1, 0.0f});
  r = df_add(r, DF{-kf * XG_LN2_2, 0.0f});
  r = df_fma(DF{-kf, 0.0f}, DF{XG_LN2_3, XG_LN2_4}, r);
  DF p{XG_EXPT[XG_EXPT_N - 1][0], XG_EXPT[XG_EXPT_N - 1][1]};
#pragma unroll
  for (int n = XG_EXPT_N - 2; n >= 0; n--) p = df_fma(p, r, DF{XG_EXPT[n][0], XG_EXPT[n][1]});
  // 2^k from the bit pattern, split in two factors to stay normal
  const int k1 = k / 2, k2 = k - k1;
  const double f1 = __hiloint2double((k1 + 1023) << 20, 0);
  const double f2 = __hiloint2double((k2 + 1023) << 20, 0);
  return df_value(p) * f1 * f2;
}

constexpr int kWarps = 4;
constexpr int kMaxB = 64;      // phase bins per channel held in shared memory
constexpr int kQagLimit = 256; // interval list of the marginal quadrature
constexpr int kMaxPiecesPerLane = 8;  // pulse knots per lane in the warp's Akima build

struct WarpSmem {
  double star[kMaxB];
  double data[kMaxB];
  DF q[kMaxB];        // SCALE / c_j(Bi): the relative form of the integrand
  float dataf[kMaxB];  // counts (exact in float below 2^24)
  double al[kQagLimit], bl[kQagLimit], rl[kQagLimit], el[kQagLimit];
};

struct Marg {
  int n;
  double SCALE, T, A;
  const double *data, *star;
  // relative form (set when every c_j(Bi) > 0, so A = x(Bi))
  int rel;
  double Bi;
  const DF *q;
  const float *dataf;
  const DF *logt;  // df_log_t's table (shared memory)
  DF nS;           // n SCALE as a pair (relative form)
};

// :84-138, as the reference writes it
__device__ __forceinline__ double marginal_integrand_direct(const Marg &m, double B) {
  double x = 0.0;
  for (int j = 0; j < m.n; j++) {
    double c = m.SCALE * (m.star[j] + B);
    if (c > 0.0) x += m.data[j] * log(c) - c;
    else if (are_equal(c, 0.0) && are_equal(m.data[j], 0.0)) {}
    else return 0.0;
  }
  return exp(x - m.A);
}

// The same integrand in relative form.  With c_j(B) = SCALE (s_j + B) and
// A = x(Bi),
//   x(B) - A = sum_j d_j log(c_j(B) / c_j(Bi)) - n SCALE (B - Bi),
// whose terms are O(d_j |B - Bi| / c_j) instead of O(d_j log c_j): no
// cancellation against A.  The ratio 1 + (B - Bi) SCALE / c_j(Bi), its
// logarithm, the sum and its exponential are taken in double-float
// arithmetic (FP32 pipes); a node where
// some ratio is not positive (c_j(B) <= 0) takes the direct form, which
// holds the reference's tests for that case.
__device__ __forceinline__ double marginal_integrand(const Marg &m, double B) {
  if (!m.rel) return marginal_integrand_direct(m, B);
  const double dBd = B - m.Bi;
  const DF dB = df_split(dBd);
  const DF one{1.0f, 0.0f};
  DF acc{0.0f, 0.0f};
  for (int j = 0; j < m.n; j++) {
    const DF r = df_fma(dB, m.q[j], one);
    if (!(r.h > 0.0f)) return marginal_integrand_direct(m, B);
    if (m.dataf[j] != 0.0f) acc = df_fma(DF{m.dataf[j], 0.0f}, df_log_t(r, m.logt), acc);
  }
  return df_exp_d(df_sub(acc, df_mul(m.nS, dB)));
}

// sum over the warp; the butterfly adds the same pairs in every lane, so all
// lanes return identical bits
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// The Akima-periodic pieces of one component's pulse through (x[i], y[i]),
// i < n, built once per warp in double-float arithmetic: the pulse scaled
// by 2^-e (e the binary exponent of its largest value, exact) into yd[],
// the chord slopes into ch[], each interval's (k1, k2, k3) into k1[], k2[],
// k3[] (akima_piece_df, with the grid's 1/h and 1/h^2 from ih[], ih2[]), then
// yd[] over ch[] -- the
// pieces akima_periodic_integral forms again for every bin that reaches
// them, here once, on the FP32 pipes (~2^-48 relative).  Returns e; ends
// with __syncwarp.
__device__ __forceinline__ int akima_pieces_warp_df(const double *x, const double *y, int n,
                                                    const DF *ih, const DF *ih2, DF *ch, DF *k1,
                                                    DF *k2, DF *k3, int lane) {
  int e = INT_MIN;
  bool inf = false;
  for (int q = lane; q < n; q += 32) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(y[q]);
    const int f = (int)((b >> 52) & 0x7ff);
    if (f == 0x7ff) inf = true;
    else if (f != 0) e = max(e, f - 1022);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    e = max(e, __shfl_xor_sync(0xffffffffu, e, o));
    inf = __shfl_xor_sync(0xffffffffu, (int)inf, o) != 0 || inf;
  }
  if (inf || e == INT_MIN) e = 0;
  // yd (in k3[] for now) and the chords
  for (int q = lane; q < n; q += 32) k3[q] = df_split(ldexp(y[q], -e));
  __syncwarp();
  for (int q = lane; q < n - 1; q += 32)
    ch[q] = df_mul(df_sub(k3[q + 1], k3[q]), ih[q]);
  __syncwarp();
  DF yq[kMaxPiecesPerLane];
  int c = 0;
  for (int q = lane; q < n; q += 32) yq[c++] = k3[q];
  __syncwarp();
  for (int i = lane; i < n - 1; i += 32) {
    DF a1, a2, a3;
    akima_piece_df(ch[periodic_chord(i - 2, n)], ch[periodic_chord(i - 1, n)], ch[i],
                   ch[periodic_chord(i + 1, n)], ch[periodic_chord(i + 2, n)], ih[i], ih2[i],
                   a1, a2, a3);
    k1[i] = a1;
    k2[i] = a2;
    k3[i] = a3;
  }
  __syncwarp();
  c = 0;
  for (int q = lane; q < n; q += 32) ch[q] = yq[c++];
  __syncwarp();
  return e;
}
// akima_periodic_integral over [lo, hi] from the pieces of
// akima_pieces_warp_df (yd in yd[]), in units of 2^e
__device__ __forceinline__ DF akima_integral_df(const double *x, const DF *yd, int n,
                                                const DF *k1, const DF *k2, const DF *k3,
                                                double lo, double hi) {
  const DF third{0.3333333432674408f, -9.934107758624577e-09f};
  const int ia = locate(x, n, lo), ib = locate(x, n, hi);
  DF acc{0.0f, 0.0f};
  for (int i = ia; i <= ib; i++) {
    const double u = (i == ia) ? lo - x[i] : 0.0;
    const double w = (i == ib) ? hi - x[i] : x[i + 1] - x[i];
    // F(t) = t (y + t (k1 / 2 + t (k2 / 3 + t k3 / 4))) at w and u
    const DF c1{0.5f * k1[i].h, 0.5f * k1[i].l}, c3{0.25f * k3[i].h, 0.25f * k3[i].l};
    const DF c2 = df_mul(k2[i], third);
    DF F[2];
    const double ts[2] = {w, u};
#pragma unroll
    for (int z = 0; z < 2; z++) {
      const DF t = df_split(ts[z]);
      F[z] = df_mul(t, df_fma(t, df_fma(t, df_fma(t, c3, c2), c1), yd[i]));
    }
    acc = df_add(acc, df_sub(F[0], F[1]));
  }
  return acc;
}

// :140-173 (returns the step; writes the Gaussian width); lane-parallel over
// the phase bins.  pow(s, 2.0) of the reference is s * s, as its C compiler
// emits it.
__device__ __forceinline__ double newton_delta(const Marg &m, double B, int lane, double &std) {
  double x = 0.0, y = 0.0;
  for (int j = lane; j < m.n; j += 32) {
    // d / s and d / s^2 from one reciprocal (an ulp from the two divisions)
    const double is = 1.0 / (m.star[j] + B);
    const double t = m.data[j] * is;
    y += t;
    x += t * is;
  }
  y = warp_sum(y);
  x = warp_sum(x);
  y = 2.0 * m.T - 2.0 * y;
  x *= 2.0;
  std = sqrt(2.0 / x);
  return -1.0 * y / x;
}

// The 21-point Gauss-Kronrod panels of the marginal quadrature, evaluated by
// the warp: lane l holds node l and node l + 32 of up to two panels (nodes
// 0..20 the first, 21..41 the second; within a panel, nodes 0..9 at
// c - h X[j], 10 at c, 11..20 at c + h X[j]).  The weighted sums of the
// rule are lane-parallel xor-butterfly reductions (identical bits in every
// lane); the error estimate follows QUADPACK (the (200 e / rc)^1.5 scaling,
// the 50 eps round-off floor).
struct Panel {
  double res, err, rabs, rasc;
};

__device__ __forceinline__ int gk21_slot(int n) { return n < 10 ? n : (n == 10 ? 10 : n - 11); }

__device__ __forceinline__ double gk21_node(double a, double b, int n) {
  const int NH = XG_K21_HALF - 1;
  double c = 0.5 * (a + b), h = 0.5 * (b - a);
  if (n < NH) return c - h * XG_K21_X[n];
  if (n == NH) return c;
  return c + h * XG_K21_X[n - NH - 1];
}

__device__ __forceinline__ Panel gk21_finish(double rk, double rg, double ra, double rc, double a,
                                             double b) {
  const double h = 0.5 * (b - a), ah = fabs(h);
  Panel P;
  P.res = rk * h;
  ra *= ah;
  rc *= ah;
  double e = fabs((rk - rg) * h);
  if (rc != 0.0 && e != 0.0) {
    const double x = 200.0 * e / rc, sc = x * sqrt(x);  // x^1.5
    e = sc < 1.0 ? rc * sc : rc;
  }
  const double eps = 2.220446049250313e-16, dmin = 2.2250738585072014e-308;
  if (ra > dmin / (50.0 * eps)) {
    const double fl = 50.0 * eps * ra;
    if (fl > e) e = fl;
  }
  P.err = e;
  P.rabs = ra;
  P.rasc = rc;
  return P;
}

// one panel [a1, b1] (two: also [a2, b2]); returns the panels' sums
__device__ void warp_panels(const Marg &m, int lane, double a1, double b1, double a2, double b2,
                            bool two, Panel &P1, Panel &P2) {
  const int total = two ? 42 : 21;
  double f0 = 0.0, f1 = 0.0;
  if (lane < total) f0 = marginal_integrand(m, lane < 21 ? gk21_node(a1, b1, lane)
                                                         : gk21_node(a2, b2, lane - 21));
  if (lane + 32 < total) f1 = marginal_integrand(m, gk21_node(a2, b2, lane + 32 - 21));
  double rk1 = 0.0, rg1 = 0.0, ra1 = 0.0, rk2 = 0.0, rg2 = 0.0, ra2 = 0.0;
  if (lane < total) {
    if (lane < 21) {
      const int s = gk21_slot(lane);
      rk1 = XG_K21_WK[s] * f0; rg1 = XG_K21_WG[s] * f0; ra1 = XG_K21_WK[s] * fabs(f0);
    } else {
      const int s = gk21_slot(lane - 21);
      rk2 = XG_K21_WK[s] * f0; rg2 = XG_K21_WG[s] * f0; ra2 = XG_K21_WK[s] * fabs(f0);
    }
  }
  if (lane + 32 < total) {
    const int s = gk21_slot(lane + 32 - 21);
    rk2 += XG_K21_WK[s] * f1; rg2 += XG_K21_WG[s] * f1; ra2 += XG_K21_WK[s] * fabs(f1);
  }
  rk1 = warp_sum(rk1); rg1 = warp_sum(rg1); ra1 = warp_sum(ra1);
  if (two) { rk2 = warp_sum(rk2); rg2 = warp_sum(rg2); ra2 = warp_sum(ra2); }
  const double mean1 = 0.5 * rk1, mean2 = 0.5 * rk2;
  double rc1 = 0.0, rc2 = 0.0;
  if (lane < total) {
    if (lane < 21) rc1 = XG_K21_WK[gk21_slot(lane)] * fabs(f0 - mean1);
    else rc2 = XG_K21_WK[gk21_slot(lane - 21)] * fabs(f0 - mean2);
  }
  if (lane + 32 < total) rc2 += XG_K21_WK[gk21_slot(lane + 32 - 21)] * fabs(f1 - mean2);
  rc1 = warp_sum(rc1);
  P1 = gk21_finish(rk1, rg1, ra1, rc1, a1, b1);
  if (two) {
    rc2 = warp_sum(rc2);
    P2 = gk21_finish(rk2, rg2, ra2, rc2, a2, b2);
  }
}

// index of the first largest error among el[0..size) (QUADPACK's choice of
// the interval to bisect), by a warp arg-max with ties to the lower index;
// identical in every lane (a NaN error counts as -inf)
__device__ __forceinline__ int warp_worst(const double *el, int size, int lane) {
  double v = -INFINITY;
  int k = 0x7fffffff;
  for (int i = lane; i < size; i += 32) {
    const double e = isnan(el[i]) ? -INFINITY : el[i];
    if (k == 0x7fffffff || e > v) {
      v = e;
      k = i;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double v2 = __shfl_xor_sync(0xffffffffu, v, o);
    const int k2 = __shfl_xor_sync(0xffffffffu, k, o);
    if (v2 > v || (v2 == v && k2 < k)) {
      v = v2;
      k = k2;
    }
  }
  return k;
}

// adaptive GK21 (same scheme as the rays' QAG), warp-cooperative; a < b
__device__ double warp_qag21_core(const Marg &m, WarpSmem &w, int lane, double a, double b,
                                  double epsabs, double er) {
  const double eps = 2.220446049250313e-16, dmin = 2.2250738585072014e-308;
  Panel P0, Pu;
  warp_panels(m, lane, a, b, 0.0, 0.0, false, P0, Pu);
  const double r0 = P0.res, e0 = P0.err, ra0 = P0.rabs, rc0 = P0.rasc;
  double tol = fmax(epsabs, er * fabs(r0));
  double rfloor = 50.0 * eps * ra0;
  if ((e0 <= rfloor && e0 > tol) || (e0 <= tol && e0 != rc0) || e0 == 0.0) return r0;
  if (lane == 0) { w.al[0] = a; w.bl[0] = b; w.rl[0] = r0; w.el[0] = e0; }
  __syncwarp();
  int size = 1, iter = 1, k = 0, rnd1 = 0, rnd2 = 0, fail = 0;
  double area = r0, errsum = e0;
  do {
    double ai = w.al[k], bi = w.bl[k], ri = w.rl[k], ei = w.el[k];
    double a1 = ai, b1 = 0.5 * (ai + bi), a2 = b1, b2 = bi;
    Panel P1, P2;
    warp_panels(m, lane, a1, b1, a2, b2, true, P1, P2);
    const double r1 = P1.res, e1 = P1.err, rc1 = P1.rasc;
    const double r2 = P2.res, e2 = P2.err, rc2 = P2.rasc;
    double r12 = r1 + r2, e12 = e1 + e2;
    errsum += e12 - ei;
    area += r12 - ri;
    if (rc1 != e1 && rc2 != e2) {
      double delta = ri - r12;
      if (fabs(delta) <= 1.0e-5 * fabs(r12) && e12 >= 0.99 * ei) rnd1++;
      if (iter >= 10 && e12 > ei) rnd2++;
    }
    tol = fmax(epsabs, er * fabs(area));
    if (errsum > tol) {
      if (rnd1 >= 6 || rnd2 >= 20) fail = 2;
      double edge = (1.0 + 100.0 * eps) * (fabs(a2) + 1000.0 * dmin);
      if (fabs(a1) <= edge && fabs(b2) <= edge) fail = 3;
    }
    int nw = size++;
    __syncwarp();
    if (lane == 0) {
      if (e2 > e1) {
        w.al[k] = a2; w.bl[k] = b2; w.rl[k] = r2; w.el[k] = e2;
        w.al[nw] = a1; w.bl[nw] = b1; w.rl[nw] = r1; w.el[nw] = e1;
      } else {
        w.al[k] = a1; w.bl[k] = b1; w.rl[k] = r1; w.el[k] = e1;
        w.al[nw] = a2; w.bl[nw] = b2; w.rl[nw] = r2; w.el[nw] = e2;
      }
    }
    __syncwarp();
    k = warp_worst(w.el, size, lane);
    iter++;
  } while (iter < kQagLimit && !fail && errsum > tol);
  double sum = 0.0;
  for (int i = lane; i < size; i += 32) sum += w.rl[i];
  sum = warp_sum(sum);
  __syncwarp();
  return sum;
}

// dyadic pieces toward an endpoint holding all the mass (see warp_marginal)
__device__ double warp_dyadic(const Marg &m, WarpSmem &w, int lane, double lo, double hi,
                              bool toward_lo, double er) {
  const double L = hi - lo;
  double sum = 0.0;
  int seen = 0, quiet_after = 0;
  for (int k = 0; k < 2100; k++) {
    double s1 = ldexp(L, -(k + 1)), s0 = ldexp(L, -k);
    double p0 = toward_lo ? lo + s1 : hi - s0;
    double p1 = toward_lo ? lo + s0 : hi - s1;
    if (!(p0 < p1) || (toward_lo ? p0 <= lo : p1 >= hi)) break;
    double r = warp_qag21_core(m, w, lane, p0, p1, 0.0, er);
    sum += r;
    if (r != 0.0) seen = 1;
    if (seen && fabs(r) <= 1.0e-17 * fabs(sum)) {
      if (++quiet_after >= 4) break;
    } else {
      quiet_after = 0;
    }
  }
  return sum;
}

// the marginal integral over [a, b]: adaptive GK21 at relative
// min(epsrel, 1e-13); when every interior node sees zero but an endpoint
// does not (a channel without counts has a window ~1e91 wide whose integrand
// decays on the scale 1 / exposure), the window is cut into dyadic pieces
// toward that endpoint, as a Clenshaw-Curtis rule with endpoint nodes would
// resolve it.
__device__ double warp_marginal(const Marg &m, WarpSmem &w, int lane, double a, double b,
                                double epsabs, double epsrel) {
  const double eps = 2.220446049250313e-16;
  double sign = 1.0;
  if (b < a) { double t = a; a = b; b = t; sign = -1.0; }
  if (a == b) return 0.0;
  double er = epsrel < 1.0e-13 ? epsrel : 1.0e-13;
  if (epsabs <= 0.0 && er < 50.0 * eps) er = 50.0 * eps;
  double r = warp_qag21_core(m, w, lane, a, b, epsabs, er);
  if (r == 0.0) {
    double fa = marginal_integrand(m, a);
    double fb = marginal_integrand(m, b);
    if (fa != 0.0 || fb != 0.0) {
      double mid = 0.5 * (a + b);
      double rl = (fa != 0.0) ? warp_dyadic(m, w, lane, a, mid, true, er)
                              : warp_qag21_core(m, w, lane, a, mid, 0.0, er);
      double rr = (fb != 0.0) ? warp_dyadic(m, w, lane, mid, b, false, er)
                              : warp_qag21_core(m, w, lane, mid, b, 0.0, er);
      r = rl + rr;
    }
  }
  return sign * r;
}

__global__ void __launch_bounds__(32 * kWarps) like_channel_kernel(LikeArgs a) {
  __shared__ WarpSmem ws[kWarps];
  __shared__ DF s_logt[XG_LOGT_N];
  // the phase grid's 1 / h and 1 / h^2 as pairs, shared by the warps' Akima builds
  __shared__ DF s_ih[kQagLimit], s_ih2[kQagLimit];
  for (int t = threadIdx.x; t < XG_LOGT_N; t += blockDim.x) s_logt[t] = DF{XG_LOGT[t][0], XG_LOGT[t][1]};
  for (int t = threadIdx.x; t < a.N_P - 1 && t < kQagLimit; t += blockDim.x) {
    const double h = a.comp_phases[t + 1] - a.comp_phases[t];
    s_ih[t] = df_split(1.0 / h);
    s_ih2[t] = df_split(1.0 / (h * h));
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const long gw = (long)blockIdx.x * kWarps + wid;
  if (gw >= (long)a.n_vec * a.K) return;
  const int v = (int)(gw / a.K), ch = (int)(gw % a.K);
  WarpSmem &w = ws[wid];
  const int B = a.B, N_P = a.N_P;
  const double n = (double)B;
  const double SCALE = a.exposure / n;
  const double T = a.exposure;
  // expected star count rate per phase bin (compute_expected_counts.pyx:66-197).
  // Each component's Akima pieces are built once by the warp (in the
  // quadrature's interval lists, free until the marginal integral) and
  // integrated over every bin; pulses longer than those lists take the
  // per-bin form.
  const bool warp_pieces = N_P > 1 && N_P <= kQagLimit && N_P <= 32 * kMaxPiecesPerLane;
  for (int j = lane; j < B; j += 32) w.star[j] = 0.0;
  if (warp_pieces) {
    DF *yd = reinterpret_cast<DF *>(w.el), *k1 = reinterpret_cast<DF *>(w.al);
    DF *k2 = reinterpret_cast<DF *>(w.bl), *k3 = reinterpret_cast<DF *>(w.rl);
    const double *xs = a.comp_phases;
    for (int h = 0; h < a.H; h++) {
      const double *pulse = a.signals + (((size_t)v * a.H + h) * a.K + ch) * N_P;
      const double sh = a.shifts[(size_t)v * a.H + h];
      const bool neg = a.allow_negative[h] == 1;
      const int ex = akima_pieces_warp_df(xs, pulse, N_P, s_ih, s_ih2, yd, k1, k2, k3, lane);
      for (int j = lane; j < B; j += 32) {
        double st = w.star[j];
        double pa = a.phase_edges[j] + sh, pb = a.phase_edges[j + 1] + sh;
        if (are_equal(pb - pa, 1.0)) { pa = 0.0; pb = 1.0; }
        else { pa -= floor(pa); pb -= floor(pb); }
        // the reference's argument checks (akima_periodic_integral)
        auto piece = [&](double lo, double hi) -> double {
          if (lo > hi || lo < xs[0] || hi > xs[N_P - 1]) return nan("");
          if (lo == hi) return 0.0;
          return ldexp(df_value(akima_integral_df(xs, yd, N_P, k1, k2, k3, lo, hi)), ex);
        };
        double val;
        if (pa < pb) {
          val = piece(pa, pb);
          if (val > 0.0 || neg) st += val;
        } else {
          val = piece(pa, 1.0);
          if (val > 0.0 || neg) st += val;
          val = piece(0.0, pb);
          if (val > 0.0 || neg) st += val;
        }
        w.star[j] = st;
      }
      __syncwarp();
    }
  }
  for (int j = lane; j < B; j += 32) {
    double st = w.star[j];
    for (int h = 0; h < a.H && !warp_pieces; h++) {
      const double *pulse = a.signals + (((size_t)v * a.H + h) * a.K + ch) * N_P;
      const double sh = a.shifts[(size_t)v * a.H + h];
      const bool neg = a.allow_negative[h] == 1;
      if (N_P > 1) {
        double pa = a.phase_edges[j] + sh, pb = a.phase_edges[j + 1] + sh;
        if (are_equal(pb - pa, 1.0)) { pa = 0.0; pb = 1.0; }
        else { pa -= floor(pa); pb -= floor(pb); }
        double val;
        if (pa < pb) {
          val = akima_periodic_integral(a.comp_phases, pulse, N_P, pa, pb);
          if (val > 0.0 || neg) st += val;
        } else {
          val = akima_periodic_integral(a.comp_phases, pulse, N_P, pa, 1.0);
          if (val > 0.0 || neg) st += val;
          val = akima_periodic_integral(a.comp_phases, pulse, N_P, 0.0, pb);
          if (val > 0.0 || neg) st += val;
        }
      } else if (j == 0) {
        st = pulse[0];
      }
    }
    if (st < 0.0) st = 0.0;
    if (a.background) st += a.background[(size_t)ch * B + j];
    st *= n;
    w.star[j] = st;
    w.data[j] = a.counts[(size_t)ch * B + j];
  }
  __syncwarp();
  double av_STAR = 0.0, av_DATA = 0.0;
  for (int j = lane; j < B; j += 32) {
    av_STAR += w.star[j];
    av_DATA += w.data[j];
  }
  av_STAR = warp_sum(av_STAR);
  av_DATA = warp_sum(av_DATA);
  const size_t o = (size_t)v * a.K + ch;
  int flag = 0;
  double term = 0.0, Bout = 0.0;
  if (a.slim >= 0.0) {
    double limit = av_STAR * SCALE - a.slim * sqrt(av_STAR * SCALE) - av_DATA;
    if (limit > 0.0) flag = 1;
  }
  const double *support = a.support + 2 * (size_t)ch;
  Marg m{B, SCALE, T, 0.0, w.data, w.star, 0, 0.0, w.q, w.dataf, s_logt};
  double Bfinal = 0.0;
  if (!flag) {
    av_STAR /= n;
    av_DATA /= T;
    double Bv;
    if (are_equal(av_DATA, 0.0) && are_equal(av_STAR, 0.0)) {
      double lower = 0.0;
      if (lower < support[0]) lower = support[0];
      double upper = 10.0 / T;
      if (upper > support[1] && support[1] > 0.0) upper = support[1];
      Bv = 0.0;
      term = log((exp(-1.0 * lower * T) - exp(-1.0 * upper * T)) / T);
    } else {
      double B_min = 0.0;
      Bv = av_DATA - av_STAR;
      if (Bv <= B_min) {
        double min_counts = -1.0;
        for (int j = 0; j < B; j++)
          if (are_equal(w.star[j], 0.0)) { min_counts = -2.0; break; }
        if (are_equal(min_counts, -2.0)) {
          for (int j = 0; j < B; j++)
            if ((are_equal(min_counts, -2.0) && w.data[j] > 0.0) ||
                (0.0 < w.data[j] && w.data[j] < min_counts))
              min_counts = w.data[j];
        }
        if (!are_equal(min_counts, -1.0)) {
          if (are_equal(min_counts, -2.0)) { Bv = 0.0; B_min = 0.0; }
          else { Bv = 0.01 * min_counts / SCALE; B_min = 0.1 * Bv; }
        } else {
          Bv = B_min;
        }
      }
      double stdv;
      double dB = newton_delta(m, Bv, lane, stdv);
      int counter = 0, steps = 0;
      // the reference's Newton loop (:336-352) has no step limit; 10000 steps
      // bound it here (convergence takes a handful)
      while (fabs(dB) > a.epsilon * stdv && counter < 2 && steps++ < 10000) {
        Bv += dB;
        if (Bv < B_min) {
          if (B_min > 0.0) counter += 1;
          else counter = 2;
          Bv = B_min;
        }
        dB = newton_delta(m, Bv, lane, stdv);
      }
      double std_est = 0.0;
      for (int j = lane; j < B; j += 32) {
        const double sb = w.star[j] + Bv;
        std_est += w.data[j] / (sb * sb);
      }
      std_est = warp_sum(std_est);
      if (std_est > 0.0) std_est = sqrt(1.0 / std_est);
      else std_est = 1e90;
      double lower = Bv - a.sigmas * std_est, upper = Bv + a.sigmas * std_est;
      if (lower < B_min) lower = B_min;
      double Bi = Bv;
      if (lower < support[0]) {
        lower = support[0];
        if (upper < support[0] && support[1] > 0.0) { upper = support[1]; Bi = support[0]; }
        else if (upper < support[0]) { upper = support[0] + a.sigmas * std_est; Bi = support[0]; }
      }
      if (upper > support[1] && support[1] > 0.0) {
        upper = support[1];
        if (lower > support[1]) { lower = support[0]; Bi = support[1]; }
      }
      if (Bi < lower) Bi = lower;
      else if (Bi > upper) Bi = upper;
      double A = 0.0, dsum = 0.0;
      for (int j = lane; j < B; j += 32) {
        double c = SCALE * (w.star[j] + Bi);
        if (c > 0.0) A += w.data[j] * log(c) - c;
        else if (are_equal(c, 0.0) && are_equal(w.data[j], 0.0)) {}
        else A += a.llzero;
        dsum += w.data[j];
      }
      A = warp_sum(A);
      dsum = warp_sum(dsum);
      m.A = A;
      // relative form of the integrand when every c_j(Bi) > 0
      bool pos = true;
      for (int j = lane; j < B; j += 32) {
        const double c = SCALE * (w.star[j] + Bi);
        pos = pos && c > 0.0;
        w.q[j] = c > 0.0 ? df_split(SCALE / c) : DF{0.0f, 0.0f};
        w.dataf[j] = (float)w.data[j];
      }
      __syncwarp();
      if (__all_sync(0xffffffffu, pos)) {
        m.rel = 1;
        m.Bi = Bi;
        m.nS = df_split((double)m.n * m.SCALE);
      }
      double result;
      if (dsum == 0.0) {
        // no counts in the channel: every term is -c_j, so the integrand is
        // exp(-T (B - Bi)) exactly and its integral over the window is closed
        // form (the reference's quadrature converges to this value)
        result = exp(-T * (lower - Bi)) * (-expm1(-T * (upper - lower))) / T;
      } else {
        result = warp_marginal(m, w, lane, lower, upper, a.epsabs, a.epsrel);
      }
      if (result > 0.0) term = log(result) + A + a.precomp[ch];
      else flag = 2;
    }
    Bfinal = Bv;
    Bout = Bv;
  }
  if (lane == 0) {
    a.chan_ll[o] = term;
    a.chan_flag[o] = flag;
    if (a.mcl_bg && flag == 0) {
      a.mcl_bg[o] = Bout * T;
      double Bs = Bout;
      if (Bs < support[0]) Bs = support[0];
      else if (Bs > support[1] && support[1] > 0.0) Bs = support[1];
      a.mcl_bg_s[o] = Bs * T;
    }
  }
  if (a.star) {
    for (int j = lane; j < B; j += 32) {
      double s = w.star[j];
      if (flag == 0) s = SCALE * (s + Bfinal);
      a.star[o * B + j] = s;
    }
  }
}

// (s, c) += x with Neumaier's compensation: s + c carries the sum to about
// twice the working precision whatever the order of magnitudes
__device__ __forceinline__ void comp_add(double &s, double &c, double x) {
  const double t = s + x;
  c += (fabs(s) >= fabs(x)) ? (s - t) + x : (x - t) + s;
  s = t;
}

// per-evaluation sum over channels and the reference's early exits: one
// warp per evaluation; the first flagged channel (lowest index) decides the
// early exit (:677-684, :423-429), otherwise the channel terms are summed
// with compensation (each lane over its channels, then the lanes' sums and
// corrections by a fixed butterfly: bitwise reproducible)
__global__ void like_finalize_kernel(LikeArgs a) {
  const int lane = threadIdx.x & 31;
  const int v = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (v >= a.n_vec) return;
  double LL = 0.0, LLc = 0.0;
  int first = 0x7fffffff;
  for (int ch = lane; ch < a.K; ch += 32) {
    const size_t o = (size_t)v * a.K + ch;
    if (a.chan_flag[o] != 0) {
      if (ch < first) first = ch;
    } else {
      comp_add(LL, LLc, a.chan_ll[o]);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    first = min(first, __shfl_xor_sync(0xffffffffu, first, o));
    const double s2 = __shfl_xor_sync(0xffffffffu, LL, o);
    const double c2 = __shfl_xor_sync(0xffffffffu, LLc, o);
    // both lanes of a pair form the same (s, c): add the lower lane's pair
    // to the higher's in a fixed order
    double s = (lane & o) ? s2 : LL, c = (lane & o) ? c2 : LLc;
    comp_add(s, c, (lane & o) ? LL : s2);
    c += (lane & o) ? LLc : c2;
    LL = s;
    LLc = c;
  }
  LL = LL + LLc;
  int st = kOk;
  if (first != 0x7fffffff) {
    const int f = a.chan_flag[(size_t)v * a.K + first];
    // llzero * (0.1 + 0.9 U): U from a hash of (evaluation, channel)
    uint32_t hsh = (uint32_t)v * 2654435761u ^ (uint32_t)first * 40503u ^ 0x9e3779b9u;
    hsh ^= hsh >> 16; hsh *= 0x7feb352du; hsh ^= hsh >> 15; hsh *= 0x846ca68bu; hsh ^= hsh >> 16;
    const double U = (double)(hsh >> 8) / 16777215.0;
    LL = a.llzero * (0.1 + 0.9 * U);
    st = (f == 1) ? kSlimCut : kQuadFail;
  }
  if (lane == 0) {
    a.loglike[v] = LL;
    a.status[v] = st;
  }
}

}  // namespace

void launch_likelihood(const LikeArgs &a, cudaStream_t st) {
  long warps = (long)a.n_vec * a.K;
  if (warps <= 0) return;
  unsigned blocks = (unsigned)((warps + kWarps - 1) / kWarps);
  like_channel_kernel<<<blocks, 32 * kWarps, 0, st>>>(a);
  like_finalize_kernel<<<(a.n_vec + 3) / 4, 128, 0, st>>>(a);
}

}  // namespace xg

namespace xg {
namespace {
// default_background_marginalisation.pyx:38-68: -sum_j ln(d_ij!)
__global__ void precomp_kernel(int K, int B, const int32_t *counts, double *out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= K) return;
  double s = 0.0;
  for (int j = 0; j < B; j++) s += lgamma((double)(uint32_t)counts[(size_t)i * B + j] + 1.0);
  out[i] = -s;
}
}  // namespace

void launch_precomputation(int K, int B, const int32_t *counts, double *out, cudaStream_t st) {
  if (K <= 0) return;
  precomp_kernel<<<(K + 127) / 128, 128, 0, st>>>(K, B, counts, out);
}
}  // namespace xg

// ---------------------------------------------------------------------------
// Allocation-free variant of the batched likelihood entry point.
//
// Some callers cannot allocate device memory when they call the likelihood:
// a sampler or serving host whose framework owns all device memory through
// its own pool (allocations from outside the pool fail or fragment it), and
// code that must run in a fixed memory budget known in advance.  For them
// xgpu_likelihood_batch_static takes device inputs and outputs from the
// caller, as xgpu_likelihood_batch does, and keeps the per-(evaluation,
// channel) scratch -- the channel's log-likelihood term and its early-exit
// flag -- in the fixed array below, which every GPU that loads this library
// holds until the process exits.
// ---------------------------------------------------------------------------
#include <mutex>

#include "../../include/xpsi_gb300.h"

namespace {

// 4 MiB: 12 bytes per (evaluation, channel) -> at most 349525 of them
constexpr size_t kLikeScratchBytes = size_t(4) << 20;
constexpr size_t kLikeScratchPerChannel = sizeof(double) + sizeof(int32_t);
static __device__ __align__(256) unsigned char g_like_scratch[kLikeScratchBytes];

// device address of g_like_scratch per device, looked up with that device
// current (the host-side name of the array is not a device address) and
// kept with the unique id of the context it belongs to: a context created
// anew (after cudaDeviceReset) has a new id, and the address is looked up
// again instead of reusing one from the destroyed context
std::mutex g_like_scratch_mu;
void *g_like_scratch_addr[64] = {};
unsigned long long g_like_scratch_ctx[64] = {};

using CtxGetCurrent = int (*)(void **);
using CtxGetId = int (*)(void *, unsigned long long *);

// the current context's unique id, through the driver entry points the
// runtime hands out (no link-time dependency on the driver library); 0 if
// they are unavailable
unsigned long long current_context_id() {
  static CtxGetCurrent get_cur = nullptr;
  static CtxGetId get_id = nullptr;
  static bool looked = false;
  if (!looked) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_cur = reinterpret_cast<CtxGetCurrent>(p);
    p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<CtxGetId>(p);
    looked = true;
  }
  void *ctx = nullptr;
  unsigned long long id = 0;
  if (get_cur && get_id && get_cur(&ctx) == 0 && ctx && get_id(ctx, &id) == 0) return id;
  return 0;
}

int like_scratch_address(void **out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return -4;
  std::lock_guard<std::mutex> lk(g_like_scratch_mu);
  const unsigned long long ctx = current_context_id();
  if (!g_like_scratch_addr[dev] || ctx == 0 || ctx != g_like_scratch_ctx[dev]) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_like_scratch) != cudaSuccess || p == nullptr) return -4;
    g_like_scratch_addr[dev] = p;
    g_like_scratch_ctx[dev] = ctx;
  }
  *out = g_like_scratch_addr[dev];
  return 0;
}

}  // namespace

extern "C" int xgpu_likelihood_batch_static(const xgpu_likelihood_batch_data *d,
                                            void *stream) {
  if (d == nullptr || d->n_vec < 0 || d->K <= 0) return -2;
  if (d->B > 64 || d->N_P < 5) return -2;
  const size_t n = (size_t)d->n_vec * (size_t)d->K;
  if (n > kLikeScratchBytes / kLikeScratchPerChannel) return -3;
  void *base = nullptr;
  int rc = like_scratch_address(&base);
  if (rc) return rc;
  if (n == 0) return 0;
  xg::LikeArgs a{};
  a.n_vec = d->n_vec; a.K = d->K; a.B = d->B; a.H = d->H; a.N_P = d->N_P;
  a.exposure = d->exposure; a.epsabs = d->epsabs; a.epsrel = d->epsrel;
  a.epsilon = d->epsilon; a.sigmas = d->sigmas; a.llzero = d->llzero; a.slim = d->slim;
  a.phase_edges = d->phase_edges; a.comp_phases = d->comp_phases; a.counts = d->counts;
  a.precomp = d->precomp; a.support = d->support; a.background = d->background;
  a.signals = d->signals; a.shifts = d->shifts; a.allow_negative = d->allow_negative;
  // every (evaluation, channel) term and flag is written by the channel
  // kernel before the finalize kernel reads it, so nothing needs clearing
  a.chan_ll = static_cast<double *>(base);
  a.chan_flag = reinterpret_cast<int32_t *>(static_cast<unsigned char *>(base) + n * sizeof(double));
  a.star = d->star; a.mcl_bg = d->mcl_bg; a.mcl_bg_s = d->mcl_bg_support;
  a.loglike = d->loglike; a.status = d->status;
  xg::launch_likelihood(a, static_cast<cudaStream_t>(stream));
  return cudaGetLastError() == cudaSuccess ? 0 : -5;
}
