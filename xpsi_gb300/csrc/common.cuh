// common.cuh -- device-side building blocks shared by the pulse-likelihood
// kernels: physical constants, status codes, spline pieces (Steffen, Akima
// with periodic ends) and a QUADPACK-style adaptive Gauss-Kronrod integrator.
//
// The numerical semantics follow the X-PSI reference path (cited per item);
// the spline and quadrature algorithms are the published ones the reference
// reaches through GSL (Steffen 1990; Akima 1970 with periodic end chords;
// QUADPACK QAG, Piessens et al. 1983).
#pragma once

#include <climits>
#include <cuda_runtime.h>
#include <stdint.h>

#include "gk_nodes.h"

namespace xg {

// xpsi/global_imports.py constants
constexpr double kPi = 3.14159265358979323846;
constexpr double kHalfPi = kPi / 2.0;
constexpr double kTwoPi = 2.0 * kPi;
constexpr double kC = 2.99792458e8;
constexpr double kKeV = 1.60217662e-16;
constexpr double kKB = 1.38064852e-23;
constexpr double kHKeV = 4.135667662e-18;
constexpr double kErg = 1.0e-7;                  // hot_BB.pyx:23
constexpr double kPlanck = 5.040366110812353e22; // hot_BB.pyx:24
constexpr double kBPhotonSphere = 2.598076211353316;  // 3 sqrt(3)/2, rays.pyx:59

// status words shared by every batched entry point
enum Status : int32_t {
  kOk = 0,
  kRayFail = 1,     // rays.pyx:331-339 -> HotRegion.RayError
  kPulseFail = 2,   // integrator terminate -> HotRegion.PulseError
  kAtmosBounds = 3, // Photosphere.py:486-507
  kQuadFail = 4,    // marginal integral vanished -> random llzero
  kSlimCut = 5,     // slim early exit (default_background_marginalisation.pyx:677-684)
  kBadInput = 6,
};

// tools/core.pyx:118-122
__host__ __device__ __forceinline__ bool are_equal(double x, double y) {
  return fabs(x - y) < 1.0e-12;
}

// rays.pyx:53-57
__device__ __forceinline__ double image_deflection(int order, double psi) {
  double s = (order % 2 == 0) ? 1.0 : -1.0;
  return (order % 2 != 0) ? (double)(order + 1) * kPi + s * psi
                          : (double)order * kPi + s * psi;
}

// largest i in [0, n-2] with x[i] <= v (v inside [x[0], x[n-1]])
template <typename T>
__device__ __forceinline__ int locate(const T *x, int n, T v) {
  int lo = 0, hi = n - 1;
  while (hi > lo + 1) {
    int mid = (lo + hi) >> 1;
    if (x[mid] > v) hi = mid; else lo = mid;
  }
  return lo;
}

// ---------------------------------------------------------------------
// Steffen (1990) monotone cubic, evaluated without a coefficient table: the
// node slopes of interval i need only y[i-1..i+2].  End slopes are the end
// chords (Steffen sect. 2.2, the choice GSL's steffen type makes).
// ---------------------------------------------------------------------
template <typename XF, typename YF>
__device__ __forceinline__ double steffen_slope(const XF &x, const YF &y, int n, int i) {
  if (i == 0) return (y(1) - y(0)) / (x(1) - x(0));
  if (i == n - 1) return (y(n - 1) - y(n - 2)) / (x(n - 1) - x(n - 2));
  double hl = x(i) - x(i - 1), hr = x(i + 1) - x(i);
  double sl = (y(i) - y(i - 1)) / hl, sr = (y(i + 1) - y(i)) / hr;
  double p = (sl * hr + sr * hl) / (hl + hr);
  double mag = fmin(fabs(sl), fmin(fabs(sr), 0.5 * fabs(p)));
  return (copysign(1.0, sl) + copysign(1.0, sr)) * mag;
}

struct Cubic {
  double y0, k1, k2, k3, x0;
};

template <typename XF, typename YF>
__device__ __forceinline__ Cubic steffen_piece(const XF &x, const YF &y, int n, int i) {
  double h = x(i + 1) - x(i);
  double s = (y(i + 1) - y(i)) / h;
  double d0 = steffen_slope(x, y, n, i), d1 = steffen_slope(x, y, n, i + 1);
  Cubic c;
  c.x0 = x(i);
  c.y0 = y(i);
  c.k1 = d0;
  c.k2 = (3.0 * s - 2.0 * d0 - d1) / h;
  c.k3 = (d0 + d1 - 2.0 * s) / (h * h);
  return c;
}

__device__ __forceinline__ double cubic_eval(const Cubic &c, double v) {
  double t = v - c.x0;
  return c.y0 + t * (c.k1 + t * (c.k2 + t * c.k3));
}

__device__ __forceinline__ double cubic_deriv(const Cubic &c, double v) {
  double t = v - c.x0;
  return c.k1 + t * (2.0 * c.k2 + 3.0 * c.k3 * t);
}

// Views of one parallel's ray tables for the Steffen evaluations of the
// integrators: the main table (deflection -> cos alpha or lag) and the
// reversed table on cos(deflection) over the rays up to the first deflection
// above pi/2 (integrator_for_azimuthal_invariance.pyx:209-227,
// integrator_for_time_invariance.pyx:151-164,206-213).
struct MainX { const double *D; __device__ double operator()(int j) const { return D[j]; } };
struct ArrY { const double *Y; __device__ double operator()(int j) const { return Y[j]; } };
struct AltX {
  const double *D; int jalt;
  __device__ double operator()(int t) const { return cos(D[jalt - t]); }
};
struct AltY {
  const double *Y; int jalt;
  __device__ double operator()(int t) const { return Y[jalt - t]; }
};

template <typename XF>
__device__ __forceinline__ int locate_f(const XF &x, int n, double v) {
  int lo = 0, hi = n - 1;
  while (hi > lo + 1) {
    int mid = (lo + hi) >> 1;
    if (x(mid) > v) hi = mid; else lo = mid;
  }
  return lo;
}

template <typename XF, typename YF>
__device__ __forceinline__ void steffen_eval(const XF &x, const YF &y, int n, double v,
                                             double *val, double *der) {
  int i = locate_f(x, n, v);
  Cubic c = steffen_piece(x, y, n, i);
  if (val) *val = cubic_eval(c, v);
  if (der) *der = cubic_deriv(c, v);
}

// hot_BB.pyx:54-82 with kT = k_B 10^logT / keV formed once by the caller
__device__ __forceinline__ double eval_bb(double E, double kT) {
  return E * E * E / (exp(E / kT) - 1.0);
}

// 4-point Lagrange stencils of the Num4D atmosphere (hot_Num4D.pyx:248-439):
// the base node for a query inside the grid (the node the reference's cached
// walk lands on) and the stencil weights in the reference's operation order.
__device__ __forceinline__ int stencil_base(const double *g, int n, double v) {
  // base node of the 4-point stencil around the interval holding v
  int lo = 0, hi = n - 1;
  while (hi > lo + 1) {
    int mid = (lo + hi) >> 1;
    if (g[mid] > v) hi = mid; else lo = mid;
  }
  int b = lo - 1;
  if (b < 0) b = 0;
  if (b > n - 4) b = n - 4;
  return b;
}

__device__ __forceinline__ void lagrange4(const double *P, int b, double x, double w[4]) {
  double d0 = (x - P[b + 1]) * (x - P[b + 2]) * (x - P[b + 3]);
  double d1 = (x - P[b]) * (x - P[b + 2]) * (x - P[b + 3]);
  double d2 = (x - P[b]) * (x - P[b + 1]) * (x - P[b + 3]);
  double d3 = (x - P[b]) * (x - P[b + 1]) * (x - P[b + 2]);
  double s0 = 1.0 / (P[b] - P[b + 1]); s0 /= P[b] - P[b + 2]; s0 /= P[b] - P[b + 3];
  double s1 = 1.0 / (P[b + 1] - P[b]); s1 /= P[b + 1] - P[b + 2]; s1 /= P[b + 1] - P[b + 3];
  double s2 = 1.0 / (P[b + 2] - P[b]); s2 /= P[b + 2] - P[b + 1]; s2 /= P[b + 2] - P[b + 3];
  double s3 = 1.0 / (P[b + 3] - P[b]); s3 /= P[b + 3] - P[b + 1]; s3 /= P[b + 3] - P[b + 2];
  w[0] = d0 * s0; w[1] = d1 * s1; w[2] = d2 * s2; w[3] = d3 * s3;
}

// exact integral of a cubic piece over [x0 + u, x0 + w]
__host__ __device__ __forceinline__ double piece_integral(double y0, double k1, double k2,
                                                          double k3, double u, double w) {
  double Fw = w * (y0 + w * (0.5 * k1 + w * (k2 / 3.0 + 0.25 * k3 * w)));
  double Fu = u * (y0 + u * (0.5 * k1 + u * (k2 / 3.0 + 0.25 * k3 * u)));
  return Fw - Fu;
}

// ---------------------------------------------------------------------
// Akima (1970) piece coefficients for interval i from the chord slopes
// m[i-2..i+2]; a segment whose two weights vanish is the chord.
// ---------------------------------------------------------------------
template <typename Real>
__device__ __forceinline__ void akima_piece(Real mm2, Real mm1, Real m0, Real mp1, Real mp2,
                                            Real h, Real &k1, Real &k2, Real &k3) {
  Real wl = fabs(mp1 - m0) + fabs(mm1 - mm2);
  if (wl == Real(0)) {
    k1 = m0; k2 = Real(0); k3 = Real(0);
    return;
  }
  Real wr = fabs(mp2 - mp1) + fabs(m0 - mm1);
  Real f = fabs(mm1 - mm2) / wl;
  Real tl = (Real(1) - f) * mm1 + f * m0;
  Real tr;
  if (wr == Real(0)) {
    tr = m0;
  } else {
    Real g = fabs(m0 - mm1) / wr;
    tr = (Real(1) - g) * m0 + g * mp1;
  }
  k1 = tl;
  k2 = (Real(3) * m0 - Real(2) * tl - tr) / h;
  k3 = (tl + tr - Real(2) * m0) / (h * h);
}

// periodic chord index: chords 0..n-2, ghosts -2,-1 -> n-3,n-2; n-1,n -> 0,1
__device__ __forceinline__ int periodic_chord(int j, int n) {
  if (j < 0) return j + (n - 1);
  if (j > n - 2) return j - (n - 1);
  return j;
}


// integral of the Akima-periodic interpolant through (x[i], y[i]) over [lo, hi]
__device__ inline double akima_periodic_integral(const double *x, const double *y, int n, double lo,
                                          double hi) {
  if (lo > hi || lo < x[0] || hi > x[n - 1]) return nan("");
  if (lo == hi) return 0.0;
  auto chord = [&](int j) -> double {
    int q = periodic_chord(j, n);
    return (y[q + 1] - y[q]) / (x[q + 1] - x[q]);
  };
  int ia = locate(x, n, lo), ib = locate(x, n, hi);
  double acc = 0.0;
  for (int i = ia; i <= ib; i++) {
    double h = x[i + 1] - x[i];
    double k1, k2, k3;
    akima_piece(chord(i - 2), chord(i - 1), chord(i), chord(i + 1), chord(i + 2), h, k1, k2, k3);
    double u = (i == ia) ? lo - x[i] : 0.0;
    double w = (i == ib) ? hi - x[i] : h;
    acc += piece_integral(y[i], k1, k2, k3, u, w);
  }
  return acc;
}


// ---------------------------------------------------------------------
// Double-float numbers: an unevaluated sum h + l of two floats, about 48
// significant bits (~4e-15 relative per operation).  On this GPU an FP32
// instruction issues at 64x the FP64 rate, and a double-float operation is
// 7-30 FP32 instructions, so FP64-path work whose values stay inside the
// float exponent range runs in this form at FP64-class accuracy for a
// fraction of the FP64 pipe's time.  Methods: Knuth's two-sum, Dekker's
// fast two-sum and product (the product error taken with an FMA), one
// correction step of long division for the quotient and of Newton's method
// for the square root.  The _rn intrinsics keep the compiler from
// contracting or reassociating the error-free transformations.
// ---------------------------------------------------------------------
struct DF {
  float h, l;
};

// Knuth: s + e == a + b exactly
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
// Dekker: s + e == a + b when |a| >= |b|
__device__ __forceinline__ DF fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return DF{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ DF df_split(double v) {
  const float h = (float)v;
  return DF{h, (float)(v - (double)h)};
}
__device__ __forceinline__ double df_value(DF a) { return (double)a.h + (double)a.l; }
__device__ __forceinline__ DF df_neg(DF a) { return DF{-a.h, -a.l}; }
__device__ __forceinline__ DF df_add(DF a, DF b) {
  float s, e;
  two_sum(a.h, b.h, s, e);
  e = __fadd_rn(e, __fadd_rn(a.l, b.l));
  return fast_two_sum(s, e);
}
__device__ __forceinline__ DF df_sub(DF a, DF b) { return df_add(a, df_neg(b)); }
// a * b (the a.l * b.l term, ~2^-48 relative, is dropped)
__device__ __forceinline__ DF df_mul(DF a, DF b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return fast_two_sum(p, e);
}
// a * b + c
__device__ __forceinline__ DF df_fma(DF a, DF b, DF c) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  float s, f;
  two_sum(p, c.h, s, f);
  f = __fadd_rn(f, __fadd_rn(e, c.l));
  return fast_two_sum(s, f);
}
// a / b: float quotient of the high parts, corrected by the remainder
// a - q b (formed exactly through the FMA product error).  The quotients
// may be the fast approximate ones (2 ulp): the correction absorbs the first
// one's error and the second's is ~2^-23 of a ~2^-23 term.
__device__ __forceinline__ DF df_div(DF a, DF b) {
  const float q1 = __fdividef(a.h, b.h);
  const float p = __fmul_rn(q1, b.h);
  const float pe = __fmaf_rn(q1, b.h, -p);
  float r = __fsub_rn(a.h, p);
  r = __fsub_rn(r, pe);
  r = __fadd_rn(r, a.l);
  r = __fmaf_rn(-q1, b.l, r);
  const float q2 = __fdividef(r, b.h);
  return fast_two_sum(q1, q2);
}
// sqrt(a): an approximate float root s = a rsqrt(a) plus one Newton
// correction (a - s^2) / (2 s) with the residual formed exactly; 0 for
// a == 0, NaN for a < 0 (as sqrt)
__device__ __forceinline__ DF df_sqrt(DF a) {
  if (!(a.h > 0.0f)) return DF{__fsqrt_rn(a.h), 0.0f};
  const float rs = rsqrtf(a.h);
  const float s = __fmul_rn(a.h, rs);
  const float p = __fmul_rn(s, s);
  const float pe = __fmaf_rn(s, s, -p);
  float r = __fsub_rn(a.h, p);
  r = __fsub_rn(r, pe);
  r = __fadd_rn(r, a.l);
  const float c = __fmul_rn(r, __fmul_rn(0.5f, rs));
  return fast_two_sum(s, c);
}

// Natural logarithm of a positive, normal double-float m.  With m = 2^e f,
// f in [0.75, 1.5): log m = e ln 2 + 2 atanh(s), s = (f - 1) / (f + 1),
// |s| <= 0.2, by the series atanh s = s (1 + s^2/3 + s^4/5 + ...) through
// s^20/21 (truncation below 1e-17 relative).  The coefficients are 1/(2k+1)
// and ln 2 as float pairs.
__device__ __forceinline__ DF df_log(DF m) {
  constexpr float kC[11][2] = {
      {1.0f, 0.0f},
      {0.3333333432674408f, -9.934107758624577e-09f},
      {0.20000000298023224f, -2.9802322831784522e-09f},
      {0.1428571492433548f, -6.38621200366174e-09f},
      {0.1111111119389534f, -8.278422947149977e-10f},
      {0.09090909361839294f, -2.709302115988521e-09f},
      {0.07692307978868484f, -2.8656079731348427e-09f},
      {0.06666667014360428f, -3.47693762670076e-09f},
      {0.05882352963089943f, -2.1913472425527658e-10f},
      {0.05263157933950424f, -3.9213582381236733e-10f},
      {0.0476190485060215f, -8.869738832295582e-10f}};
  const DF ln2{0.6931471824645996f, -1.9046542121259336e-09f};
  // exponent e with m.h 2^-e in [0.75, 1.5), from the float's bits
  const int bits = __float_as_int(m.h);
  int e = ((bits >> 23) & 0xff) - 127;  // m.h = 1.x 2^e
  if ((bits & 0x7fffff) >= 0x400000) e += 1;  // 1.x >= 1.5: use 0.75 2^(e+1)
  const float sc = __int_as_float((127 - e) << 23);  // 2^-e, exact
  const DF f{__fmul_rn(m.h, sc), __fmul_rn(m.l, sc)};
  const DF one{1.0f, 0.0f};
  const DF s = df_div(df_sub(f, one), df_add(f, one));
  const DF s2 = df_mul(s, s);
  DF p{kC[10][0], kC[10][1]};
#pragma unroll
  for (int k = 9; k >= 0; k--) p = df_fma(p, s2, DF{kC[k][0], kC[k][1]});
  return df_fma(DF{(float)e, 0.0f}, ln2, df_mul(df_add(s, s), p));
}

// acc + a b in double-float, the sum held unnormalised in (s, c): s gathers
// the rounded products through error-free sums, c the product and sum
// errors; the caller renormalises once (two_sum of s and c)
__device__ __forceinline__ void df_acc_mul(DF a, DF b, float &s, float &c) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  float q;
  two_sum(s, p, s, q);
  c = __fadd_rn(c, __fadd_rn(q, e));
}
__device__ __forceinline__ DF df_norm(float s, float c) {
  DF r;
  two_sum(s, c, r.h, r.l);
  return r;
}

// binary exponent x of |v| = f 2^x, f in [0.5, 1), from the bit pattern
// (integer work); kZeroExp for zero and subnormal values
constexpr int kZeroExp = -2100;
__device__ __forceinline__ int binary_exponent(double v) {
  const int e = (__double2hiint(v) >> 20) & 0x7ff;
  return e == 0 ? kZeroExp : e - 1022;
}
// 2^x as a double from the bit pattern (0 below the normal range, the
// largest power of two above it)
__device__ __forceinline__ double pow2_double(int x) {
  const int b = x + 1023;
  if (b <= 0) return 0.0;
  return __hiloint2double(min(b, 2046) << 20, 0);
}
// v 2^e, as ldexp(v, e) (one rounding at most), by a product with the
// power of two where that is a normal double
__device__ __forceinline__ double scale_pow2(double v, int e) {
  return (e >= -1022 && e <= 1023) ? v * pow2_double(e) : ldexp(v, e);
}
// the largest frexp exponent of |v| over a lane's values, from the bit
// patterns (integer work): fold() each value, exponent() at the end gives
// what frexp(max |v|) gives, 0 when the largest is 0, infinite or NaN
// throughout (NaNs are skipped as fmax skips them; an infinity gives 0)
struct MaxExponent {
  int e = INT_MIN;
  bool inf = false;
  __device__ __forceinline__ void fold(double v) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const int f = (int)((b >> 52) & 0x7ff);
    const unsigned long long m = b & 0xfffffffffffffull;
    if (f == 0x7ff) {
      inf = inf || m == 0ull;
    } else if (f != 0) {
      e = max(e, f - 1022);
    } else if (m != 0ull) {
      e = max(e, -1010 - __clzll((long long)m));
    }
  }
  __device__ __forceinline__ void merge_warp() {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      e = max(e, __shfl_xor_sync(0xffffffffu, e, o));
      inf = __shfl_xor_sync(0xffffffffu, (int)inf, o) != 0 || inf;
    }
  }
  __device__ __forceinline__ int exponent() const { return (inf || e == INT_MIN) ? 0 : e; }
};

// Akima piece (akima_piece above) in double-float arithmetic, with the
// divisions by h and h^2 taken as products with their reciprocals
__device__ __forceinline__ DF df_abs(DF a) { return a.h < 0.0f ? df_neg(a) : a; }
__device__ __forceinline__ void akima_piece_df(DF mm2, DF mm1, DF m0, DF mp1, DF mp2, DF ih,
                                               DF ih2, DF &k1, DF &k2, DF &k3) {
  const DF one{1.0f, 0.0f};
  const DF wl = df_add(df_abs(df_sub(mp1, m0)), df_abs(df_sub(mm1, mm2)));
  if (wl.h == 0.0f) {
    k1 = m0;
    k2 = k3 = DF{0.0f, 0.0f};
    return;
  }
  const DF wr = df_add(df_abs(df_sub(mp2, mp1)), df_abs(df_sub(m0, mm1)));
  const DF f = df_div(df_abs(df_sub(mm1, mm2)), wl);
  const DF tl = df_fma(df_sub(one, f), mm1, df_mul(f, m0));
  DF tr;
  if (wr.h == 0.0f) {
    tr = m0;
  } else {
    const DF gg = df_div(df_abs(df_sub(m0, mm1)), wr);
    tr = df_fma(df_sub(one, gg), m0, df_mul(gg, mp1));
  }
  k1 = tl;
  const DF m3 = df_add(df_add(m0, m0), m0);
  k2 = df_mul(df_sub(df_sub(m3, df_add(tl, tl)), tr), ih);
  k3 = df_mul(df_sub(df_add(tl, tr), df_add(m0, m0)), ih2);
}

// ---------------------------------------------------------------------
// QUADPACK QAG with a Gauss-Kronrod rule, one thread per integral.  The
// interval list lives in the caller-provided arrays (local memory).
// Returns a GSL-compatible status: 0 ok, 5 failed, 11 max iterations,
// 18 round-off, 21 singularity.  Result semantics match the reference's
// GSL call (best estimate returned on every status).
// ---------------------------------------------------------------------
// the adaptive bisection, with panel(lo, hi, result, error, |f| integral,
// |f - mean| integral) evaluating one Gauss-Kronrod panel
template <int LIMIT, typename Panel>
__device__ int qag_panels(const Panel &panel, double a, double b, double epsabs, double epsrel,
                          double &result, double &abserr) {
  const double eps = 2.220446049250313e-16, dmin = 2.2250738585072014e-308;
  double al[LIMIT], bl[LIMIT], rl[LIMIT], el[LIMIT];
  double r0, e0, ra0, rc0;
  panel(a, b, r0, e0, ra0, rc0);
  int size = 1;
  al[0] = a; bl[0] = b; rl[0] = r0; el[0] = e0;
  double tol = fmax(epsabs, epsrel * fabs(r0));
  double rfloor = 50.0 * eps * ra0;
  if (e0 <= rfloor && e0 > tol) { result = r0; abserr = e0; return 18; }
  if ((e0 <= tol && e0 != rc0) || e0 == 0.0) { result = r0; abserr = e0; return 0; }
  if (LIMIT == 1) { result = r0; abserr = e0; return 11; }
  double area = r0, errsum = e0;
  int rnd1 = 0, rnd2 = 0, fail = 0, iter = 1, k = 0;
  do {
    double ai = al[k], bi = bl[k], ri = rl[k], ei = el[k];
    double a1 = ai, b1 = 0.5 * (ai + bi), a2 = b1, b2 = bi;
    double r1, e1, ra1, rc1, r2, e2, ra2, rc2;
    panel(a1, b1, r1, e1, ra1, rc1);
    panel(a2, b2, r2, e2, ra2, rc2);
    double r12 = r1 + r2, e12 = e1 + e2;
    errsum += e12 - ei;
    area += r12 - ri;
    if (rc1 != e1 && rc2 != e2) {
      double delta = ri - r12;
      if (fabs(delta) <= 1.0e-5 * fabs(r12) && e12 >= 0.99 * ei) rnd1++;
      if (iter >= 10 && e12 > ei) rnd2++;
    }
    tol = fmax(epsabs, epsrel * fabs(area));
    if (errsum > tol) {
      if (rnd1 >= 6 || rnd2 >= 20) fail = 2;
      double edge = (1.0 + 100.0 * eps) * (fabs(a2) + 1000.0 * dmin);
      if (fabs(a1) <= edge && fabs(b2) <= edge) fail = 3;
    }
    int nw = size++;
    if (e2 > e1) {
      al[k] = a2; bl[k] = b2; rl[k] = r2; el[k] = e2;
      al[nw] = a1; bl[nw] = b1; rl[nw] = r1; el[nw] = e1;
    } else {
      al[k] = a1; bl[k] = b1; rl[k] = r1; el[k] = e1;
      al[nw] = a2; bl[nw] = b2; rl[nw] = r2; el[nw] = e2;
    }
    k = 0;
    for (int i = 1; i < size; i++)
      if (el[i] > el[k]) k = i;
    iter++;
  } while (iter < LIMIT && !fail && errsum > tol);
  double sum = 0.0;
  for (int i = 0; i < size; i++) sum += rl[i];
  result = sum;
  abserr = errsum;
  if (errsum <= tol) return 0;
  if (fail == 2) return 18;
  if (fail == 3) return 21;
  if (iter == LIMIT) return 11;
  return 5;
}


// One Gauss-Kronrod panel with the integrand evaluated and the Kronrod and
// Gauss sums accumulated in double-float arithmetic (X2, WK2, WG2: the
// rule's nodes and weights as float pairs); the |f| and |f - mean| sums,
// which only scale the error estimate, in FP32; the panel's result and
// error estimate in FP64 with QUADPACK's formulas (the (200 e / rc)^1.5
// scaling and the 50 eps round-off floor).
template <int HALF, typename F>
__device__ __forceinline__ void gk_panel_df(const F &f, const float *X2, const float *WK2,
                                            const float *WG2, double a, double b, double &res,
                                            double &err, double &rabs, double &rasc) {
  constexpr int NH = HALF - 1;
  const double cd = 0.5 * (a + b), hd = 0.5 * (b - a);
  const DF c = df_split(cd), h = df_split(hd);
  float fv1[NH], fv2[NH];
  const DF fc = f(c);
  DF rk = df_mul(DF{WK2[2 * NH], WK2[2 * NH + 1]}, fc);
  DF rg = df_mul(DF{WG2[2 * NH], WG2[2 * NH + 1]}, fc);
  float ra = fabsf(rk.h);
  // not unrolled: one inlined copy of the integrand, fv in local memory
#pragma unroll 1
  for (int j = 0; j < NH; j++) {
    const DF dx = df_mul(h, DF{X2[2 * j], X2[2 * j + 1]});
    const DF f1 = f(df_sub(c, dx)), f2 = f(df_add(c, dx));
    fv1[j] = f1.h;
    fv2[j] = f2.h;
    const DF s2 = df_add(f1, f2);
    rk = df_fma(DF{WK2[2 * j], WK2[2 * j + 1]}, s2, rk);
    if (WG2[2 * j] != 0.0f) rg = df_fma(DF{WG2[2 * j], WG2[2 * j + 1]}, s2, rg);
    ra += WK2[2 * j] * (fabsf(f1.h) + fabsf(f2.h));
  }
  const float mean = 0.5f * rk.h;
  float rc = WK2[2 * NH] * fabsf(fc.h - mean);
#pragma unroll 1
  for (int j = 0; j < NH; j++) rc += WK2[2 * j] * (fabsf(fv1[j] - mean) + fabsf(fv2[j] - mean));
  res = df_value(rk) * hd;
  const double ah = fabs(hd);
  const double rad = (double)ra * ah, rcd = (double)rc * ah;
  double e = fabs(df_value(df_sub(rk, rg)) * hd);
  if (rcd != 0.0 && e != 0.0) {
    const double x = 200.0 * e / rcd, sc = x * sqrt(x);  // x^1.5
    e = sc < 1.0 ? rcd * sc : rcd;
  }
  const double eps = 2.220446049250313e-16, dmin = 2.2250738585072014e-308;
  if (rad > dmin / (50.0 * eps)) {
    const double fl = 50.0 * eps * rad;
    if (fl > e) e = fl;
  }
  err = e;
  rabs = rad;
  rasc = rcd;
}

// the polarisation angle in the oblate Schwarzschild approximation (Loktev
// et al. 2020), cellmesh/common_functions.pyx:7-66
__device__ inline double pol_angle(double leaf, double sin_psi, double cos_psi, double sin_alpha,
                            double cos_alpha, double sin_th, double cos_th, double sin_i,
                            double cos_i, double sin_gamma, double cos_gamma, double Grav_z,
                            double mu, double eta, double beta, double Lorentz, double cos_xi) {
  const double chi_0 = atan2(-sin_th * sin(leaf), sin_i * cos_th - sin_th * cos_i * cos(leaf));
  const double sa_over_sp = !are_equal(sin_psi, 0.0) ? sin_alpha / sin_psi : Grav_z;
  const double chi_1 = atan2(sin_gamma * sin_i * sin(leaf) * sa_over_sp,
                             cos_gamma - cos_alpha * mu);
  const double sin_lambda = sin_th * cos_gamma - sin_gamma * cos_th;
  const double cos_lambda = cos_th * cos_gamma + sin_th * sin_gamma;
  const double cos_eps = sa_over_sp * (cos_i * sin_lambda - sin_i * cos_lambda * cos(leaf) +
                                       cos_psi * sin_gamma) - cos_alpha * sin_gamma;
  const double chi_p = atan2(cos_eps * eta * mu * beta / Lorentz,
                             (1. - mu * mu / (1. + beta * cos_xi)));
  return chi_0 + chi_1 + chi_p;
}

}  // namespace xg
