// mesh_math.h -- the mathematics of the hot-region cell meshes, shared by
// the host builder (mesh.cpp, g++) and the GPU builder (mesh_gpu.cu, nvcc):
// the area quadratures of xpsi/cellmesh/mesh_tools.pyx:18-890, the AGM_14
// effective gravity (surface_radiation_field/effective_gravity_universal.pyx:
// 10-71) and the per-parallel and per-cell steps of the spot / polar-cap
// meshes (xpsi/cellmesh/mesh.pyx:23-417, polar_mesh.pyx:23-430).
//
// The reference integrates areas with GSL's CQUAD at relative 1e-8.  Here the
// areas use an adaptive Gauss-Kronrod-21 bisection (QUADPACK QAG) at relative
// 1e-13, the same scheme the oracle's GSL-API subset serves CQUAD with, so
// the reference build used for the golden fixtures and this builder give the
// same meshes.  Every step is written as a function of its own indices
// (accumulations the reference does in a loop are replayed), so a thread per
// table entry, parallel or cell computes what the sequential loop computes.
#pragma once
#include <math.h>
#include <stddef.h>

#include "gk_nodes.h"

// XG_HD: host and device; XG_QD: the quadrature-based steps, device-only
// under nvcc (the Gauss-Kronrod tables are __constant__ there) and host
// functions under the host compiler
#ifdef __CUDACC__
#define XG_HD __host__ __device__
#define XG_QD __device__
#else
#define XG_HD
#define XG_QD
#endif

namespace xgm {

constexpr double PI = 3.14159265358979323846;
constexpr double PI_2 = PI / 2.0;
constexpr double TWO_PI = 2.0 * PI;
constexpr double C_LIGHT = 2.99792458e8;

XG_HD inline bool are_equal(double x, double y) { return fabs(x - y) < 1.0e-12; }

// ---------------------------------------------------------------- quadrature
template <typename F>
XG_QD void gk21(const F &f, double a, double b, double &res, double &err, double &rabs, double &rasc) {
  const int NH = XG_K21_HALF - 1;
  double c = 0.5 * (a + b), h = 0.5 * (b - a), ah = fabs(h);
  double fv1[NH], fv2[NH];
  double fc = f(c);
  double rk = XG_K21_WK[NH] * fc, rg = XG_K21_WG[NH] * fc, ra = fabs(rk);
  for (int j = 0; j < NH; j++) {
    double dx = h * XG_K21_X[j];
    double f1 = f(c - dx), f2 = f(c + dx);
    fv1[j] = f1;
    fv2[j] = f2;
    rk += XG_K21_WK[j] * (f1 + f2);
    rg += XG_K21_WG[j] * (f1 + f2);
    ra += XG_K21_WK[j] * (fabs(f1) + fabs(f2));
  }
  double mean = 0.5 * rk;
  double rc = XG_K21_WK[NH] * fabs(fc - mean);
  for (int j = 0; j < NH; j++)
    rc += XG_K21_WK[j] * (fabs(fv1[j] - mean) + fabs(fv2[j] - mean));
  res = rk * h;
  ra *= ah;
  rc *= ah;
  double e = fabs((rk - rg) * h);
  if (rc != 0.0 && e != 0.0) {
    const double x = 200.0 * e / rc, sc = x * sqrt(x);  // x^1.5 without pow
    e = sc < 1.0 ? rc * sc : rc;
  }
  const double eps = 2.220446049250313e-16, dmin = 2.2250738585072014e-308;
  if (ra > dmin / (50.0 * eps)) e = (e < 50.0 * eps * ra) ? 50.0 * eps * ra : e;
  err = e;
  rabs = ra;
  rasc = rc;
}

// interval list of the adaptive quadrature (LIMIT intervals)
template <int LIMIT>
struct WorkT {
  static constexpr int kLimit = LIMIT;
  double al[LIMIT], bl[LIMIT], rl[LIMIT], el[LIMIT];
};

template <typename F, typename W>
XG_QD double qag21(const F &f, double a, double b, double epsabs, double er, W &w) {
  constexpr int LIMIT = W::kLimit;
  const double eps = 2.220446049250313e-16, dmin = 2.2250738585072014e-308;
  double r0, e0, ra0, rc0;
  gk21(f, a, b, r0, e0, ra0, rc0);
  double tol = (epsabs < er * fabs(r0)) ? er * fabs(r0) : epsabs;
  if ((e0 <= 50.0 * eps * ra0 && e0 > tol) || (e0 <= tol && e0 != rc0) || e0 == 0.0) return r0;
  int size = 1, iter = 1, k = 0, rnd1 = 0, rnd2 = 0, fail = 0;
  w.al[0] = a; w.bl[0] = b; w.rl[0] = r0; w.el[0] = e0;
  double area = r0, errsum = e0;
  do {
    double ai = w.al[k], bi = w.bl[k], ri = w.rl[k], ei = w.el[k];
    double a1 = ai, b1 = 0.5 * (ai + bi), a2 = b1, b2 = bi;
    double r1, e1, ra1, rc1, r2, e2, ra2, rc2;
    gk21(f, a1, b1, r1, e1, ra1, rc1);
    gk21(f, a2, b2, r2, e2, ra2, rc2);
    double r12 = r1 + r2, e12 = e1 + e2;
    errsum += e12 - ei;
    area += r12 - ri;
    if (rc1 != e1 && rc2 != e2) {
      if (fabs(ri - r12) <= 1.0e-5 * fabs(r12) && e12 >= 0.99 * ei) rnd1++;
      if (iter >= 10 && e12 > ei) rnd2++;
    }
    tol = (epsabs < er * fabs(area)) ? er * fabs(area) : epsabs;
    if (errsum > tol) {
      if (rnd1 >= 6 || rnd2 >= 20) fail = 2;
      double edge = (1.0 + 100.0 * eps) * (fabs(a2) + 1000.0 * dmin);
      if (fabs(a1) <= edge && fabs(b2) <= edge) fail = 3;
    }
    int nw = size++;
    if (e2 > e1) {
      w.al[k] = a2; w.bl[k] = b2; w.rl[k] = r2; w.el[k] = e2;
      w.al[nw] = a1; w.bl[nw] = b1; w.rl[nw] = r1; w.el[nw] = e1;
    } else {
      w.al[k] = a1; w.bl[k] = b1; w.rl[k] = r1; w.el[k] = e1;
      w.al[nw] = a2; w.bl[nw] = b2; w.rl[nw] = r2; w.el[nw] = e2;
    }
    k = 0;
    for (int i = 1; i < size; i++)
      if (w.el[i] > w.el[k]) k = i;
    iter++;
  } while (iter < LIMIT && !fail && errsum > tol);
  double sum = 0.0;
  for (int i = 0; i < size; i++) sum += w.rl[i];
  return sum;
}

template <typename F, typename W>
XG_QD double dyadic(const F &f, double lo, double hi, bool toward_lo, double er, W &w) {
  const double L = hi - lo;
  double sum = 0.0;
  int seen = 0, quiet = 0;
  for (int k = 0; k < 2100; k++) {
    double s1 = ldexp(L, -(k + 1)), s0 = ldexp(L, -k);
    double p0 = toward_lo ? lo + s1 : hi - s0;
    double p1 = toward_lo ? lo + s0 : hi - s1;
    if (!(p0 < p1) || (toward_lo ? p0 <= lo : p1 >= hi)) break;
    double r = qag21(f, p0, p1, 0.0, er, w);
    sum += r;
    if (r != 0.0) seen = 1;
    if (seen && fabs(r) <= 1.0e-17 * fabs(sum)) {
      if (++quiet >= 4) break;
    } else {
      quiet = 0;
    }
  }
  return sum;
}

// the quadrature standing where the reference calls CQUAD(epsabs, epsrel)
template <typename F, typename W>
XG_QD double integrate(const F &f, double a, double b, double epsabs, double epsrel, W &w) {
  double sign = 1.0;
  if (b < a) { const double t = a; a = b; b = t; sign = -1.0; }
  if (a == b) return 0.0;
  double er = (1.0e-13 < epsrel) ? 1.0e-13 : epsrel;
  if (epsabs <= 0.0 && er < 50.0 * 2.220446049250313e-16) er = 50.0 * 2.220446049250313e-16;
  double r = qag21(f, a, b, epsabs, er, w);
  if (r == 0.0) {
    double fa = f(a), fb = f(b);
    if (fa != 0.0 || fb != 0.0) {
      double m = 0.5 * (a + b);
      double rl = fa != 0.0 ? dyadic(f, a, m, true, er, w) : qag21(f, a, m, 0.0, er, w);
      double rr = fb != 0.0 ? dyadic(f, m, b, false, er, w) : qag21(f, m, b, 0.0, er, w);
      r = rl + rr;
    }
  }
  return sign * r;
}

// ---------------------------------------------------------------- geometry
// mesh_tools.pyx:18-56
XG_HD inline double radiusNormalised(double mu, double epsilon, double zeta, int shape) {
  if (shape == 0) return 1.0 + epsilon * (-0.788 + 1.030 * zeta) * mu * mu;
  return 1.0;
}
// mesh_tools.pyx:58-97
XG_HD inline double f_theta(double mu, double radius, double epsilon, double zeta, int shape) {
  double d = -2.0 * epsilon * (-0.788 + 1.030 * zeta) * mu * sqrt(1.0 - mu * mu);
  if (shape == 0) return d / (radius * sqrt(1.0 - 2.0 * zeta / radius));
  return 0.0;
}
// f_theta^2 for the surface element sqrt(1 + f^2) of the area integrands:
// (2 eps c mu sin theta)^2 / (r (r - 2 zeta)), the same quantity without
// f_theta's two square roots and two divisions; sin_theta is sqrt(1 - mu^2)
// for theta in [0, pi], and accurate near the poles where 1 - mu^2 cancels
XG_HD inline double f_theta_sq(double mu, double sin_theta, double radius, double epsilon,
                               double zeta, int shape) {
  if (shape != 0) return 0.0;
  const double d = 2.0 * epsilon * (-0.788 + 1.030 * zeta) * mu * sin_theta;
  return d * d / (radius * (radius - 2.0 * zeta));
}
// effective_gravity_universal.pyx:10-71
XG_HD inline double effectiveGravity(double mu, double R_eq, double x, double epsilon, int shape) {
  double g_0 = x * C_LIGHT * C_LIGHT / (R_eq * sqrt(1.0 - 2.0 * x));
  double esq = epsilon, esqsq = epsilon * epsilon;
  double c_e = -0.791 + 0.776 * x, c_p = 1.138 - 1.431 * x;
  double d_e = (-1.315 + 2.431 * x) * esq * x, d_p = (0.653 - 2.864 * x) * esq * x;
  double d_60 = (13.47 - 27.13 * x) * esq * x;
  double f_e = -1.172 * x * esqsq, f_p = 0.975 * x * esqsq;
  double g = 1.0;
  g += (c_e + d_e + f_e) * esq * (1.0 - mu * mu);
  g += (c_p + d_p + f_p - d_60) * esq * mu * mu;
  g += d_60 * esq * fabs(mu);
  if (shape == 0) return log10(g * g_0) + 2.0;
  return log10(g_0) + 2.0;
}

struct Star {
  double R_eq, epsilon, zeta, Omega;
  int shape;
};

// mesh_tools.pyx:99-154
template <typename W>
XG_QD double integrateArea(double lo, double hi, const Star &s, int av, W &w) {
  auto f = [&](double theta) -> double {
    if (are_equal(theta, 0.0)) return 0.0;
    double mu = cos(theta);
    double radius = radiusNormalised(mu, s.epsilon, s.zeta, s.shape);
    double ft = f_theta(mu, radius, s.epsilon, s.zeta, s.shape);
    double v = radius * radius * sqrt(1.0 + ft * ft) * sin(theta);
    return av == 0 ? v : theta * v;
  };
  return s.R_eq * s.R_eq * integrate(f, lo, hi, 0.0, 1.0e-8, w);
}

// mesh_tools.pyx:156-161
XG_HD inline double eval_psi(double theta, double phi, double THETA) {
  return acos(cos(THETA) * cos(theta) + sin(THETA) * sin(theta) * cos(phi));
}
// mesh_tools.pyx:264-273
XG_HD inline double eval_phi(double theta, double THETA, double psi) {
  double cos_phi = cos(psi) - cos(THETA) * cos(theta);
  cos_phi /= sin(THETA) * sin(theta);
  if (!(-1.0 <= cos_phi && cos_phi <= 1.0)) return -1.0;
  return acos(cos_phi);
}
// mesh_tools.pyx:275-300
XG_HD inline double get_interval(double a, double b, double LB, double UB) {
  int ac = (LB <= a && a <= UB), bc = (LB <= b && b <= UB);
  if (ac == 0) ac = 2 * (int)(a > UB);
  if (bc == 0) bc = 2 * (int)(b > UB);
  if (ac == bc) return ac == 1 ? b - a : 0.0;
  if (bc == 1 && ac == 0) return b - LB;
  if (bc == 2 && ac == 1) return UB - a;
  if (bc == 2 && ac == 0) return UB - LB;
  return 0.0;
}

struct Region {
  double colat, cedeRadius, superRadius, superAzi, superColat;
  // cosines and sines of the region's angles, formed once (the ring extent
  // at every quadrature node needs them)
  double cos_colat, sin_colat, cos_cede, cos_sc, sin_sc, cos_sr;
};
XG_HD inline Region make_region(double colat, double cedeRadius, double superRadius,
                                double superAzi, double superColat) {
  Region g;
  g.colat = colat;
  g.cedeRadius = cedeRadius;
  g.superRadius = superRadius;
  g.superAzi = superAzi;
  g.superColat = superColat;
  g.cos_colat = cos(colat);
  g.sin_colat = sin(colat);
  g.cos_cede = cos(cedeRadius);
  g.cos_sc = cos(superColat);
  g.sin_sc = sin(superColat);
  g.cos_sr = cos(superRadius);
  return g;
}
// eval_phi with the trigonometric values given (the same operations)
XG_HD inline double eval_phi_cs(double cos_theta, double sin_theta, double cos_THETA,
                                double sin_THETA, double cos_psi) {
  double cos_phi = cos_psi - cos_THETA * cos_theta;
  cos_phi /= sin_THETA * sin_theta;
  if (!(-1.0 <= cos_phi && cos_phi <= 1.0)) return -1.0;
  return acos(cos_phi);
}

// azimuthal extent of the ceding annulus at colatitude theta restricted to
// [phi_a, phi_b] (cell) or unrestricted (spot): mesh_tools.pyx:302-370, 775-830
XG_HD inline double ring_extent(double theta, double cos_theta, double sin_theta, const Region &g,
                                bool cell, double phi_a, double phi_b, bool &zero) {
  zero = false;
  double aLB, aUB, cLB, cUB;
  aUB = eval_phi_cs(cos_theta, sin_theta, g.cos_colat, g.sin_colat, g.cos_cede);
  if (are_equal(aUB, -1.0)) {
    if (theta + g.colat < g.cedeRadius) {
      aUB = PI;
      aLB = -PI;
    } else {
      zero = true;
      return 0.0;
    }
  } else {
    aLB = -aUB;
  }
  if (fabs(theta - g.superColat) > g.superRadius) {
    cLB = cUB = 0.0;
  } else {
    cUB = eval_phi_cs(cos_theta, sin_theta, g.cos_sc, g.sin_sc, g.cos_sr);
    if (are_equal(cUB, -1.0)) {
      zero = true;
      return 0.0;
    }
    cLB = -cUB;
    cUB += g.superAzi;
    cLB += g.superAzi;
    if (cUB > PI) cUB -= TWO_PI;
    if (cLB < -PI) cLB += TWO_PI;
  }
  auto I = [&](double lo, double hi) -> double {
    return cell ? get_interval(phi_a, phi_b, lo, hi) : (-lo + hi);
  };
  double dphi = 0.0;
  if (cUB >= cLB) {
    if (cLB >= aUB || cUB <= aLB) dphi = I(aLB, aUB);
    else if (cLB >= aLB && cUB <= aUB) dphi = I(aLB, cLB) + I(cUB, aUB);
    else if (cLB < aLB && aLB < cUB && cUB <= aUB) dphi = I(cUB, aUB);
    else if (aLB <= cLB && cLB < aUB && aUB < cUB) dphi = I(aLB, cLB);
    else if (cLB < aLB && cUB > aUB) { zero = true; return 0.0; }
  } else {
    if (cUB >= aUB || cLB <= aLB) { zero = true; return 0.0; }
    else if (cUB >= aLB && cLB <= aUB) dphi = I(cUB, cLB);
    else if (cUB < aLB && aLB < cLB && cLB <= aUB) dphi = I(aLB, cLB);
    else if (aLB <= cUB && cUB < aUB && aUB < cLB) dphi = I(cUB, aUB);
    else if (cUB < aLB && cLB > aUB) dphi = I(aLB, aUB);
  }
  return dphi;
}

// mesh_tools.pyx:373-410
XG_HD inline double theta_given_phi(double phi, double colat, double radius, const double interval[2]) {
  double x = sin(colat) * sin(phi) / sin(radius);
  if (x <= 1.0) {
    x = asin(x);
    double theta = tan(0.5 * (colat - radius)) / sin(0.5 * (x - phi));
    theta *= sin(0.5 * (x + phi));
    theta = atan(theta);
    theta *= theta < 0.0 ? -2.0 : 2.0;
    if (!(interval[0] <= theta && theta <= interval[1])) {
      x = PI - x;
      theta = tan(0.5 * (colat - radius)) / sin(0.5 * (x - phi));
      theta *= sin(0.5 * (x + phi));
      theta = atan(theta);
      theta *= theta < 0.0 ? -2.0 : 2.0;
      if (!(interval[0] <= theta && theta <= interval[1])) return -1.0;
    }
    return theta;
  }
  return -1.0;
}

XG_HD inline double phi_edge(double theta, double phi_a, double phi_b, const Region &g, bool super) {
  // top/bottom crossings of a cell edge (mesh_tools.pyx:520-640)
  double v;
  if (!super) {
    v = eval_phi(theta, g.colat, g.cedeRadius);
    if (v >= 0.0) {
      if (!(phi_a <= v && v <= phi_b)) {
        if (!(phi_a <= -1.0 * v && -1.0 * v <= phi_b)) v = -1.0;
        else if (v < 0.0) v *= -1.0;
      } else if (v < 0.0) {
        v *= -1.0;
      }
    }
    return v;
  }
  if (fabs(theta - g.superColat) > g.superRadius) return -1.0;
  v = eval_phi(theta, g.superColat, g.superRadius);
  if (v >= 0.0) {
    v += g.superAzi;
    if (v > PI) v -= TWO_PI;
    if (v < -PI) v += TWO_PI;
    if (!(phi_a <= v && v <= phi_b)) v = -1.0;
    else if (v < 0.0) v *= -1.0;
  }
  if (v < 0.0) {
    v = eval_phi(theta, g.superColat, g.superRadius);
    if (v > 0.0) {
      v *= -1.0;
      v += g.superAzi;
      if (v > PI) v -= TWO_PI;
      if (v < -PI) v += TWO_PI;
      if (!(phi_a <= v && v <= phi_b)) v = -1.0;
      else if (v < 0.0) v *= -1.0;
    }
  }
  return v;
}

// mesh_tools.pyx:412-772: the integrand of a cell's area over colatitude
// (the cell's share of the ring, times the surface element)
struct CellIntegrand {
  Star s;
  Region g;
  double pa, pb;
  XG_HD double operator()(double theta) const {
    if (are_equal(theta, 0.0)) return 0.0;
    double mu, st;
#ifdef __CUDA_ARCH__
    sincos(theta, &st, &mu);  // one argument reduction for both
#else
    mu = cos(theta);
    st = sin(theta);
#endif
    bool zero;
    const double dphi = ring_extent(theta, mu, st, g, true, pa, pb, zero);
    // outside the cell's share of the ring the integrand is 0 (a zero
    // extent times the finite surface factor): the factor is not formed
    if (zero || dphi == 0.0) return 0.0;
    const double radius = radiusNormalised(mu, s.epsilon, s.zeta, s.shape);
    const double ft2 = f_theta_sq(mu, st, radius, s.epsilon, s.zeta, s.shape);
    return dphi * radius * radius * sqrt(1.0 + ft2) * st;
  }
};

// when the integral over [ta, tb] vanishes, the reference integrates again
// between the region boundary's crossings of the cell's edges
XG_HD inline bool cell_fallback_interval(double ta, double tb, double pa, double pb,
                                         const Region &g, double &tmin, double &tmax) {
  const double interval[2] = {ta, tb};
  double tl[2] = {theta_given_phi(pa, g.colat, g.cedeRadius, interval),
                  theta_given_phi(pa - g.superAzi, g.superColat, g.superRadius, interval)};
  double tr[2] = {theta_given_phi(pb, g.colat, g.cedeRadius, interval),
                  theta_given_phi(pb - g.superAzi, g.superColat, g.superRadius, interval)};
  double top[2] = {phi_edge(ta, pa, pb, g, false), phi_edge(ta, pa, pb, g, true)};
  double bot[2] = {phi_edge(tb, pa, pb, g, false), phi_edge(tb, pa, pb, g, true)};
  double inter[2][2];
  for (int r = 0; r < 2; r++) {
    for (int q = 0; q < 2; q++) {
      if (tl[r] >= 0.0) { inter[r][q] = tl[r]; tl[r] = -1.0; }
      else if (tr[r] >= 0.0) { inter[r][q] = tr[r]; tr[r] = -1.0; }
      else if (top[r] >= 0.0) { inter[r][q] = ta; top[r] = -1.0; }
      else if (bot[r] >= 0.0) { inter[r][q] = tb; bot[r] = -1.0; }
      else inter[r][q] = -1.0;
    }
  }
  tmin = tb;
  tmax = ta;
  double th[4] = {inter[0][0], inter[0][1], inter[1][0], inter[1][1]};
  for (int i = 0; i < 4; i++) {
    if (th[i] >= 0.0) {
      if (th[i] < tmin) tmin = th[i];
      if (th[i] > tmax) tmax = th[i];
    }
  }
  return tmin < tmax;
}

template <typename W>
XG_QD double integrateCell(double ta, double tb, double pa, double pb, const Star &s,
                           const Region &g, W &w) {
  const CellIntegrand f{s, g, pa, pb};
  double integral = integrate(f, ta, tb, 0.0, 1.0e-8, w);
  if (are_equal(integral, 0.0)) {
    double tmin, tmax;
    if (cell_fallback_interval(ta, tb, pa, pb, g, tmin, tmax))
      integral = integrate(f, tmin, tmax, 0.0, 1.0e-8, w);
  }
  return s.R_eq * s.R_eq * integral;
}

// mesh_tools.pyx:775-870 (Lorentz factor off, as allocate_cells calls it)
template <typename W>
XG_QD double integrateSpot(double ta, double tb, const Star &s, const Region &g, W &w) {
  auto f = [&](double theta) -> double {
    if (are_equal(theta, 0.0)) return 0.0;
    double mu, st;
#ifdef __CUDA_ARCH__
    sincos(theta, &st, &mu);
#else
    mu = cos(theta);
    st = sin(theta);
#endif
    double radius = radiusNormalised(mu, s.epsilon, s.zeta, s.shape);
    double ft = f_theta(mu, radius, s.epsilon, s.zeta, s.shape);
    bool zero;
    double dphi = ring_extent(theta, mu, st, g, false, 0.0, 0.0, zero);
    if (zero) return 0.0;
    return dphi * radius * radius * sqrt(1.0 + ft * ft) * st;
  };
  return s.R_eq * s.R_eq * integrate(f, ta, tb, 0.0, 1.0e-8, w);
}

// Steffen interpolation at v on an ascending grid (for the 1000-point
// area-to-colatitude table, mesh.pyx:111-120)
XG_HD inline double steffen_at(const double *x, const double *y, int n, double v) {
  int lo = 0, hi = n - 1;
  while (hi > lo + 1) {
    int mid = (lo + hi) >> 1;
    if (x[mid] > v) hi = mid; else lo = mid;
  }
  auto slope = [&](int i) -> double {
    if (i == 0) return (y[1] - y[0]) / (x[1] - x[0]);
    if (i == n - 1) return (y[n - 1] - y[n - 2]) / (x[n - 1] - x[n - 2]);
    double hl = x[i] - x[i - 1], hr = x[i + 1] - x[i];
    double sl = (y[i] - y[i - 1]) / hl, sr = (y[i + 1] - y[i]) / hr;
    double p = (sl * hr + sr * hl) / (hl + hr);
    double mag = fabs(sr) < 0.5 * fabs(p) ? fabs(sr) : 0.5 * fabs(p);
    if (fabs(sl) < mag) mag = fabs(sl);
    return (copysign(1.0, sl) + copysign(1.0, sr)) * mag;
  };
  int i = lo;
  double h = x[i + 1] - x[i], s = (y[i + 1] - y[i]) / h;
  double d0 = slope(i), d1 = slope(i + 1);
  double k2 = (3.0 * s - 2.0 * d0 - d1) / h, k3 = (d0 + d1 - 2.0 * s) / (h * h);
  double t = v - x[i];
  return y[i] + t * (d0 + t * (k2 + t * k3));
}


// ---------------------------------------------------------------- mesh steps
// mesh.pyx:23-120 / polar_mesh.pyx:23-120: limits, cell widths, the
// superseding region's extreme points, and the mirror symmetry of the mesh
struct MeshPlan {
  int polar, invert, sym;
  size_t S, numCell, j_max;
  double lims[2], boundary_phi, delta_phi, area_factor;
  double cedeColat, cedeRadius, superRadius, superColat, superAzi;
  double sp1[2], sp2[2], sp3[2], sp4[2];
};

XG_HD inline void mesh_plan(bool polar, size_t numCell, size_t S, double cedeRadius,
                            double cedeColat, double superRadius, double superColat,
                            double superAzi, MeshPlan &pl) {
  pl.polar = polar;
  pl.invert = 0;
  pl.S = S;
  pl.numCell = numCell;
  pl.boundary_phi = PI;
  if (!polar) {
    pl.lims[0] = cedeColat - cedeRadius;
    pl.lims[1] = cedeColat + cedeRadius;
    pl.boundary_phi = asin(sin(cedeRadius) / sin(cedeColat));
    pl.area_factor = 2.0 * pl.boundary_phi;
    pl.delta_phi = 2.0 * pl.boundary_phi / (double)S;
  } else {
    pl.lims[0] = 0.0;
    if (cedeColat + cedeRadius > PI) {
      pl.invert = 1;
      pl.lims[1] = PI - cedeColat + cedeRadius;
      cedeColat = PI - cedeColat;
      superColat = PI - superColat;
    } else {
      pl.lims[1] = cedeColat + cedeRadius;
    }
    pl.area_factor = TWO_PI;
    pl.delta_phi = TWO_PI / (double)S;
  }
  pl.cedeColat = cedeColat;
  pl.cedeRadius = cedeRadius;
  pl.superRadius = superRadius;
  pl.superColat = superColat;
  pl.superAzi = superAzi;
  for (int k = 0; k < 2; k++) pl.sp1[k] = pl.sp2[k] = pl.sp3[k] = pl.sp4[k] = 0.0;
  if (superRadius > 0.0) {
    if (superColat - superRadius < 0.0) {
      pl.sp1[0] = superRadius - superColat;
      pl.sp1[1] = superAzi + PI;
      if (pl.sp1[1] > PI) pl.sp1[1] -= TWO_PI;
      pl.sp2[0] = superColat + superRadius;
      pl.sp2[1] = superAzi;
    } else if (superColat + superRadius > PI) {
      pl.sp1[0] = superColat - superRadius;
      pl.sp1[1] = superAzi;
      pl.sp2[0] = TWO_PI - superColat - superRadius;
      pl.sp2[1] = superAzi + PI;
      if (pl.sp2[1] > PI) pl.sp2[1] -= TWO_PI;
    } else {
      pl.sp1[0] = superColat - superRadius;
      pl.sp1[1] = superAzi;
      pl.sp2[0] = acos(cos(superColat) / cos(superRadius));
      pl.sp2[1] = superAzi + asin(sin(superRadius) / sin(superColat));
      if (pl.sp2[1] > PI) pl.sp2[1] -= TWO_PI;
      pl.sp3[0] = superColat + superRadius;
      pl.sp3[1] = superAzi;
      pl.sp4[0] = pl.sp2[0];
      pl.sp4[1] = superAzi - asin(sin(superRadius) / sin(superColat));
      if (pl.sp4[1] < -PI) pl.sp4[1] += TWO_PI;
    }
  }
  pl.sym = are_equal(superColat, cedeColat) && are_equal(superAzi, 0.0);
  pl.j_max = pl.sym ? S / 2 : S;
}

// np.linspace(-b + d/2, b - d/2, S): the cell-centre azimuths
XG_HD inline double mesh_phi(const MeshPlan &pl, size_t j) {
  const double a = pl.polar ? -PI + 0.5 * pl.delta_phi : -pl.boundary_phi + 0.5 * pl.delta_phi;
  const double b = pl.polar ? PI - 0.5 * pl.delta_phi : pl.boundary_phi - 0.5 * pl.delta_phi;
  if (j == pl.S - 1) return b;
  const double step = (b - a) / (double)(pl.S - 1);
  return a + (double)j * step;
}

// the colatitudes of the 1000-point table of area(colat..lims[1]), descending
constexpr int kAreaTab = 1000;
XG_HD inline double mesh_table_colat(const MeshPlan &pl, int i) {
  const double a = pl.lims[1], b = pl.lims[0];
  if (i == kAreaTab - 1) return b;
  const double step = (b - a) / (double)(kAreaTab - 1);
  return a + (double)i * step;
}

// the mesh's cell area and eta from the table's full-range entry (the
// table's last colatitude is lims[0], so the entry is the spot's area)
XG_HD inline void mesh_cell_area(const MeshPlan &pl, double area_full, double &cellArea,
                                 double &eta) {
  cellArea = pl.area_factor * area_full;
  cellArea /= (double)pl.numCell;
  eta = cellArea / pl.delta_phi;
}

// the S - 1 parallels dividing the mesh into rows of equal area
XG_HD inline void mesh_parallels(const MeshPlan &pl, const double *colat, const double *areaTab,
                                 double eta, double *parallels) {
  double i_eta = (double)pl.S * eta;
  for (size_t i = 0; i + 1 < pl.S; i++) {
    i_eta -= eta;
    parallels[i] = steffen_at(areaTab, colat, kAreaTab, i_eta);
  }
}

XG_HD inline void mesh_row_bounds(const MeshPlan &pl, const double *parallels, size_t i,
                                  double &lower, double &upper) {
  const size_t S = pl.S;
  if (i == S - 1) { lower = parallels[i - 1]; upper = pl.lims[1]; }
  else if (i == 0) { lower = pl.lims[0]; upper = parallels[i]; }
  else { lower = parallels[i - 1]; upper = parallels[i]; }
}

struct RowOut {
  double colat, r, effGrav, cos_gamma, maxAlpha;
};

// per-parallel quantities: the area-weighted centre colatitude, radius,
// effective gravity and surface tilt (mesh.pyx:140-170)
template <typename W>
XG_QD inline RowOut mesh_row(const Star &s, double lower, double upper, double eta, W &w) {
  RowOut o;
  o.colat = integrateArea(lower, upper, s, 1, w) / eta;
  const double mu = cos(o.colat);
  const double radius = radiusNormalised(mu, s.epsilon, s.zeta, s.shape);
  o.r = radius * s.R_eq;
  o.effGrav = effectiveGravity(mu, s.R_eq, s.zeta, s.epsilon, s.shape);
  const double ft = f_theta(mu, radius, s.epsilon, s.zeta, s.shape);
  o.cos_gamma = 1.0 / sqrt(1.0 + ft * ft);
  o.maxAlpha = PI_2 + acos(o.cos_gamma);
  return o;
}

// cell (i, j) (mesh.pyx:170-400): corner / centre membership tests against
// the ceding and superseding regions.  Returns 0 (area 0), 1 (the nominal
// cell area) or 2 (a cell cut by a boundary: integrate it), and the cell's
// azimuth edges, replayed as the reference's running sum of cell widths.
XG_HD inline int mesh_cell_kind(const MeshPlan &pl, size_t i, size_t j, double lower,
                                double upper, double colatC, double &leftmost,
                                double &rightmost) {
  const bool polar = pl.polar;
  const double cedeColat = pl.cedeColat, cedeRadius = pl.cedeRadius;
  const double superRadius = pl.superRadius, superColat = pl.superColat;
  const double superAzi = pl.superAzi, delta_phi = pl.delta_phi;
  int p1 = 0, p3 = 0;
  if (polar && i == 0) {
    p1 = p3 = (cedeColat <= cedeRadius);
    if (p1 == 1) { p1 = p1 * (superRadius <= superColat); p3 = p1; }
    else { p1 = p3 = 2; }
  }
  leftmost = polar ? -PI : -pl.boundary_phi;
  rightmost = leftmost + delta_phi;
  for (size_t k = 0; k < j; k++) {
    leftmost = rightmost;
    rightmost = leftmost + delta_phi;
  }
  if (!polar || i > 0) {
    p1 = (eval_psi(lower, leftmost, cedeColat) <= cedeRadius);
    p3 = (eval_psi(lower, rightmost, cedeColat) <= cedeRadius);
  }
  int p2 = (eval_psi(upper, leftmost, cedeColat) <= cedeRadius);
  int p4 = (eval_psi(upper, rightmost, cedeColat) <= cedeRadius);
  int p5 = (eval_psi(colatC, leftmost + 0.5 * delta_phi, cedeColat) <= cedeRadius);
  if (!polar || i > 0) {
    if (p1 == 1) p1 = p1 * (superRadius <= eval_psi(lower, leftmost - superAzi, superColat));
    else p1 = 2;
  }
  if (p2 == 1) p2 = p2 * (superRadius <= eval_psi(upper, leftmost - superAzi, superColat));
  else p2 = 2;
  if (!polar || i > 0) {
    if (p3 == 1) p3 = p3 * (superRadius <= eval_psi(lower, rightmost - superAzi, superColat));
    else p3 = 2;
  }
  if (p4 == 1) p4 = p4 * (superRadius <= eval_psi(upper, rightmost - superAzi, superColat));
  else p4 = 2;
  if (p5 == 1)
    p5 = p5 * (superRadius <= eval_psi(colatC, leftmost + 0.5 * delta_phi - superAzi, superColat));
  else
    p5 = 2;
  if (!(p1 == p2 && p2 == p3 && p3 == p4 && p4 == p5)) return 2;
  if (superRadius > 0.0) {
    const double l = leftmost, r = rightmost;
    auto in = [&](const double *q) { return lower <= q[0] && q[0] <= upper && l <= q[1] && q[1] <= r; };
    if (in(pl.sp1) || in(pl.sp2) || in(pl.sp3) || in(pl.sp4)) return 2;
  }
  return p5 == 1 ? 1 : 0;
}

XG_HD inline Region mesh_region(const MeshPlan &pl) {
  return make_region(pl.cedeColat, pl.cedeRadius, pl.superRadius, pl.superAzi, pl.superColat);
}

// area of cell (i, j)
template <typename W>
XG_QD inline double mesh_cell(const MeshPlan &pl, const Star &s, size_t i, size_t j,
                              double lower, double upper, double colatC, double cellArea,
                              W &w) {
  double leftmost, rightmost;
  const int kind = mesh_cell_kind(pl, i, j, lower, upper, colatC, leftmost, rightmost);
  if (kind == 2) return integrateCell(lower, upper, leftmost, rightmost, s, mesh_region(pl), w);
  return kind == 1 ? cellArea : 0.0;
}

}  // namespace xgm
