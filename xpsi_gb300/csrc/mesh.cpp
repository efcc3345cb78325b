// mesh.cpp -- host-side hot-region cell meshes for the batched path: the
// cell budget (xpsi/cellmesh/mesh_tools.pyx:892-1099, allocate_cells) and the
// spot / polar-cap meshes (xpsi/cellmesh/mesh.pyx:23-417,
// xpsi/cellmesh/polar_mesh.pyx:23-430) with their area quadratures
// (mesh_tools.pyx:18-890) and the AGM_14 effective gravity
// (surface_radiation_field/effective_gravity_universal.pyx:10-71).
//
// The reference integrates areas with GSL's CQUAD at relative 1e-8.  Here the
// areas use an adaptive Gauss-Kronrod-21 bisection (QUADPACK QAG) at relative
// 1e-13, the same scheme the oracle's GSL-API subset serves CQUAD with, so
// the reference build used for the golden fixtures and this builder give the
// same meshes.  Meshes of many parameter vectors are built concurrently on
// the host's cores (one std::thread per slice).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "../../include/xpsi_gb300.h"
#include "gk_nodes.h"

namespace {

constexpr double PI = 3.14159265358979323846;
constexpr double PI_2 = PI / 2.0;
constexpr double TWO_PI = 2.0 * PI;
constexpr double C_LIGHT = 2.99792458e8;

inline bool are_equal(double x, double y) { return std::fabs(x - y) < 1.0e-12; }

// ---------------------------------------------------------------- quadrature
template <typename F>
void gk21(const F &f, double a, double b, double &res, double &err, double &rabs, double &rasc) {
  const int NH = XG_K21_HALF - 1;
  double c = 0.5 * (a + b), h = 0.5 * (b - a), ah = std::fabs(h);
  double fv1[NH], fv2[NH];
  double fc = f(c);
  double rk = XG_K21_WK[NH] * fc, rg = XG_K21_WG[NH] * fc, ra = std::fabs(rk);
  for (int j = 0; j < NH; j++) {
    double dx = h * XG_K21_X[j];
    double f1 = f(c - dx), f2 = f(c + dx);
    fv1[j] = f1;
    fv2[j] = f2;
    rk += XG_K21_WK[j] * (f1 + f2);
    rg += XG_K21_WG[j] * (f1 + f2);
    ra += XG_K21_WK[j] * (std::fabs(f1) + std::fabs(f2));
  }
  double mean = 0.5 * rk;
  double rc = XG_K21_WK[NH] * std::fabs(fc - mean);
  for (int j = 0; j < NH; j++)
    rc += XG_K21_WK[j] * (std::fabs(fv1[j] - mean) + std::fabs(fv2[j] - mean));
  res = rk * h;
  ra *= ah;
  rc *= ah;
  double e = std::fabs((rk - rg) * h);
  if (rc != 0.0 && e != 0.0) {
    double sc = std::pow(200.0 * e / rc, 1.5);
    e = sc < 1.0 ? rc * sc : rc;
  }
  const double eps = 2.220446049250313e-16, dmin = 2.2250738585072014e-308;
  if (ra > dmin / (50.0 * eps)) e = std::max(e, 50.0 * eps * ra);
  err = e;
  rabs = ra;
  rasc = rc;
}

struct Work {
  std::vector<double> al, bl, rl, el;
  Work() : al(4000), bl(4000), rl(4000), el(4000) {}
};

template <typename F>
double qag21(const F &f, double a, double b, double epsabs, double er, Work &w) {
  const int LIMIT = 4000;
  const double eps = 2.220446049250313e-16, dmin = 2.2250738585072014e-308;
  double r0, e0, ra0, rc0;
  gk21(f, a, b, r0, e0, ra0, rc0);
  double tol = std::max(epsabs, er * std::fabs(r0));
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
      if (std::fabs(ri - r12) <= 1.0e-5 * std::fabs(r12) && e12 >= 0.99 * ei) rnd1++;
      if (iter >= 10 && e12 > ei) rnd2++;
    }
    tol = std::max(epsabs, er * std::fabs(area));
    if (errsum > tol) {
      if (rnd1 >= 6 || rnd2 >= 20) fail = 2;
      double edge = (1.0 + 100.0 * eps) * (std::fabs(a2) + 1000.0 * dmin);
      if (std::fabs(a1) <= edge && std::fabs(b2) <= edge) fail = 3;
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

template <typename F>
double dyadic(const F &f, double lo, double hi, bool toward_lo, double er, Work &w) {
  const double L = hi - lo;
  double sum = 0.0;
  int seen = 0, quiet = 0;
  for (int k = 0; k < 2100; k++) {
    double s1 = std::ldexp(L, -(k + 1)), s0 = std::ldexp(L, -k);
    double p0 = toward_lo ? lo + s1 : hi - s0;
    double p1 = toward_lo ? lo + s0 : hi - s1;
    if (!(p0 < p1) || (toward_lo ? p0 <= lo : p1 >= hi)) break;
    double r = qag21(f, p0, p1, 0.0, er, w);
    sum += r;
    if (r != 0.0) seen = 1;
    if (seen && std::fabs(r) <= 1.0e-17 * std::fabs(sum)) {
      if (++quiet >= 4) break;
    } else {
      quiet = 0;
    }
  }
  return sum;
}

// the quadrature standing where the reference calls CQUAD(epsabs, epsrel)
template <typename F>
double integrate(const F &f, double a, double b, double epsabs, double epsrel, Work &w) {
  double sign = 1.0;
  if (b < a) { std::swap(a, b); sign = -1.0; }
  if (a == b) return 0.0;
  double er = std::min(epsrel, 1.0e-13);
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
double radiusNormalised(double mu, double epsilon, double zeta, int shape) {
  if (shape == 0) return 1.0 + epsilon * (-0.788 + 1.030 * zeta) * mu * mu;
  return 1.0;
}
// mesh_tools.pyx:58-97
double f_theta(double mu, double radius, double epsilon, double zeta, int shape) {
  double d = -2.0 * epsilon * (-0.788 + 1.030 * zeta) * mu * std::sqrt(1.0 - mu * mu);
  if (shape == 0) return d / (radius * std::sqrt(1.0 - 2.0 * zeta / radius));
  return 0.0;
}
// effective_gravity_universal.pyx:10-71
double effectiveGravity(double mu, double R_eq, double x, double epsilon, int shape) {
  double g_0 = x * C_LIGHT * C_LIGHT / (R_eq * std::sqrt(1.0 - 2.0 * x));
  double esq = epsilon, esqsq = epsilon * epsilon;
  double c_e = -0.791 + 0.776 * x, c_p = 1.138 - 1.431 * x;
  double d_e = (-1.315 + 2.431 * x) * esq * x, d_p = (0.653 - 2.864 * x) * esq * x;
  double d_60 = (13.47 - 27.13 * x) * esq * x;
  double f_e = -1.172 * x * esqsq, f_p = 0.975 * x * esqsq;
  double g = 1.0;
  g += (c_e + d_e + f_e) * esq * (1.0 - mu * mu);
  g += (c_p + d_p + f_p - d_60) * esq * mu * mu;
  g += d_60 * esq * std::fabs(mu);
  if (shape == 0) return std::log10(g * g_0) + 2.0;
  return std::log10(g_0) + 2.0;
}

struct Star {
  double R_eq, epsilon, zeta, Omega;
  int shape;
};

// mesh_tools.pyx:99-154
double integrateArea(double lo, double hi, const Star &s, int av, Work &w) {
  auto f = [&](double theta) -> double {
    if (are_equal(theta, 0.0)) return 0.0;
    double mu = std::cos(theta);
    double radius = radiusNormalised(mu, s.epsilon, s.zeta, s.shape);
    double ft = f_theta(mu, radius, s.epsilon, s.zeta, s.shape);
    double v = radius * radius * std::sqrt(1.0 + ft * ft) * std::sin(theta);
    return av == 0 ? v : theta * v;
  };
  return s.R_eq * s.R_eq * integrate(f, lo, hi, 0.0, 1.0e-8, w);
}

// mesh_tools.pyx:156-161
double eval_psi(double theta, double phi, double THETA) {
  return std::acos(std::cos(THETA) * std::cos(theta) + std::sin(THETA) * std::sin(theta) * std::cos(phi));
}
// mesh_tools.pyx:264-273
double eval_phi(double theta, double THETA, double psi) {
  double cos_phi = std::cos(psi) - std::cos(THETA) * std::cos(theta);
  cos_phi /= std::sin(THETA) * std::sin(theta);
  if (!(-1.0 <= cos_phi && cos_phi <= 1.0)) return -1.0;
  return std::acos(cos_phi);
}
// mesh_tools.pyx:275-300
double get_interval(double a, double b, double LB, double UB) {
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
};

// azimuthal extent of the ceding annulus at colatitude theta restricted to
// [phi_a, phi_b] (cell) or unrestricted (spot): mesh_tools.pyx:302-370, 775-830
double ring_extent(double theta, const Region &g, bool cell, double phi_a, double phi_b,
                   bool &zero) {
  zero = false;
  double aLB, aUB, cLB, cUB;
  aUB = eval_phi(theta, g.colat, g.cedeRadius);
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
  if (std::fabs(theta - g.superColat) > g.superRadius) {
    cLB = cUB = 0.0;
  } else {
    cUB = eval_phi(theta, g.superColat, g.superRadius);
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
double theta_given_phi(double phi, double colat, double radius, const double interval[2]) {
  double x = std::sin(colat) * std::sin(phi) / std::sin(radius);
  if (x <= 1.0) {
    x = std::asin(x);
    double theta = std::tan(0.5 * (colat - radius)) / std::sin(0.5 * (x - phi));
    theta *= std::sin(0.5 * (x + phi));
    theta = std::atan(theta);
    theta *= theta < 0.0 ? -2.0 : 2.0;
    if (!(interval[0] <= theta && theta <= interval[1])) {
      x = PI - x;
      theta = std::tan(0.5 * (colat - radius)) / std::sin(0.5 * (x - phi));
      theta *= std::sin(0.5 * (x + phi));
      theta = std::atan(theta);
      theta *= theta < 0.0 ? -2.0 : 2.0;
      if (!(interval[0] <= theta && theta <= interval[1])) return -1.0;
    }
    return theta;
  }
  return -1.0;
}

double phi_edge(double theta, double phi_a, double phi_b, const Region &g, bool super) {
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
  if (std::fabs(theta - g.superColat) > g.superRadius) return -1.0;
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

// mesh_tools.pyx:412-772
double integrateCell(double ta, double tb, double pa, double pb, const Star &s, const Region &g,
                     Work &w) {
  auto f = [&](double theta) -> double {
    if (are_equal(theta, 0.0)) return 0.0;
    double mu = std::cos(theta);
    double radius = radiusNormalised(mu, s.epsilon, s.zeta, s.shape);
    double ft = f_theta(mu, radius, s.epsilon, s.zeta, s.shape);
    bool zero;
    double dphi = ring_extent(theta, g, true, pa, pb, zero);
    if (zero) return 0.0;
    return dphi * radius * radius * std::sqrt(1.0 + ft * ft) * std::sin(theta);
  };
  double integral = integrate(f, ta, tb, 0.0, 1.0e-8, w);
  if (are_equal(integral, 0.0)) {
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
    double tmin = tb, tmax = ta;
    double th[4] = {inter[0][0], inter[0][1], inter[1][0], inter[1][1]};
    for (int i = 0; i < 4; i++) {
      if (th[i] >= 0.0) {
        if (th[i] < tmin) tmin = th[i];
        if (th[i] > tmax) tmax = th[i];
      }
    }
    if (tmin < tmax) integral = integrate(f, tmin, tmax, 0.0, 1.0e-8, w);
  }
  return s.R_eq * s.R_eq * integral;
}

// mesh_tools.pyx:775-870 (Lorentz factor off, as allocate_cells calls it)
double integrateSpot(double ta, double tb, const Star &s, const Region &g, Work &w) {
  auto f = [&](double theta) -> double {
    if (are_equal(theta, 0.0)) return 0.0;
    double mu = std::cos(theta);
    double radius = radiusNormalised(mu, s.epsilon, s.zeta, s.shape);
    double ft = f_theta(mu, radius, s.epsilon, s.zeta, s.shape);
    bool zero;
    double dphi = ring_extent(theta, g, false, 0.0, 0.0, zero);
    if (zero) return 0.0;
    return dphi * radius * radius * std::sqrt(1.0 + ft * ft) * std::sin(theta);
  };
  return s.R_eq * s.R_eq * integrate(f, ta, tb, 0.0, 1.0e-8, w);
}

// Steffen interpolation at v on an ascending grid (for the 1000-point
// area-to-colatitude table, mesh.pyx:111-120)
double steffen_at(const double *x, const double *y, int n, double v) {
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
    double mag = std::min(std::fabs(sl), std::min(std::fabs(sr), 0.5 * std::fabs(p)));
    return (std::copysign(1.0, sl) + std::copysign(1.0, sr)) * mag;
  };
  int i = lo;
  double h = x[i + 1] - x[i], s = (y[i + 1] - y[i]) / h;
  double d0 = slope(i), d1 = slope(i + 1);
  double k2 = (3.0 * s - 2.0 * d0 - d1) / h, k3 = (d0 + d1 - 2.0 * s) / (h * h);
  double t = v - x[i];
  return y[i] + t * (d0 + t * (k2 + t * k3));
}

struct MeshOut {
  double *theta, *phi, *r, *area, *maxAlpha, *cos_gamma, *effGrav;
};

// mesh.pyx:23-417 (polar = false) and polar_mesh.pyx:23-430 (polar = true)
int build_mesh(bool polar, size_t numCell, size_t S, const Star &s, double cedeRadius,
               double cedeColat, double superRadius, double superColat, double superAzi,
               const MeshOut &o, Work &w) {
  if (S < 2) return -1;
  double lims[2];
  int invert = 0;
  double cellArea, delta_phi, boundary_phi = PI;
  std::vector<double> phi1(S);
  if (!polar) {
    lims[0] = cedeColat - cedeRadius;
    lims[1] = cedeColat + cedeRadius;
    boundary_phi = std::asin(std::sin(cedeRadius) / std::sin(cedeColat));
    cellArea = 2.0 * boundary_phi * integrateArea(lims[0], lims[1], s, 0, w);
    delta_phi = 2.0 * boundary_phi / (double)S;
  } else {
    lims[0] = 0.0;
    if (cedeColat + cedeRadius > PI) {
      invert = 1;
      lims[1] = PI - cedeColat + cedeRadius;
      cedeColat = PI - cedeColat;
      superColat = PI - superColat;
    } else {
      lims[1] = cedeColat + cedeRadius;
    }
    cellArea = TWO_PI * integrateArea(0.0, lims[1], s, 0, w);
    delta_phi = TWO_PI / (double)S;
  }
  // np.linspace(-b + d/2, b - d/2, S)
  {
    double a = polar ? -PI + 0.5 * delta_phi : -boundary_phi + 0.5 * delta_phi;
    double b = polar ? PI - 0.5 * delta_phi : boundary_phi - 0.5 * delta_phi;
    double step = (b - a) / (double)(S - 1);
    for (size_t j = 0; j < S; j++) phi1[j] = a + (double)j * step;
    phi1[S - 1] = b;
  }
  // 1000-point table of area(theta..lims[1]) against theta (descending theta)
  std::vector<double> colat(1000), areaTab(1000);
  {
    double a = lims[1], b = lims[0], step = (b - a) / 999.0;
    for (int i = 0; i < 1000; i++) colat[i] = a + (double)i * step;
    colat[999] = b;
  }
  cellArea /= (double)numCell;
  double eta = cellArea / delta_phi;
  for (int i = 0; i < 1000; i++) areaTab[i] = integrateArea(colat[i], lims[1], s, 0, w);
  std::vector<double> parallels(S - 1);
  double i_eta = (double)S * eta;
  for (size_t i = 0; i + 1 < S; i++) {
    i_eta -= eta;
    parallels[i] = steffen_at(areaTab.data(), colat.data(), 1000, i_eta);
  }
  double sp1[2] = {0, 0}, sp2[2] = {0, 0}, sp3[2] = {0, 0}, sp4[2] = {0, 0};
  if (superRadius > 0.0) {
    if (superColat - superRadius < 0.0) {
      sp1[0] = superRadius - superColat;
      sp1[1] = superAzi + PI;
      if (sp1[1] > PI) sp1[1] -= TWO_PI;
      sp2[0] = superColat + superRadius;
      sp2[1] = superAzi;
    } else if (superColat + superRadius > PI) {
      sp1[0] = superColat - superRadius;
      sp1[1] = superAzi;
      sp2[0] = TWO_PI - superColat - superRadius;
      sp2[1] = superAzi + PI;
      if (sp2[1] > PI) sp2[1] -= TWO_PI;
    } else {
      sp1[0] = superColat - superRadius;
      sp1[1] = superAzi;
      sp2[0] = std::acos(std::cos(superColat) / std::cos(superRadius));
      sp2[1] = superAzi + std::asin(std::sin(superRadius) / std::sin(superColat));
      if (sp2[1] > PI) sp2[1] -= TWO_PI;
      sp3[0] = superColat + superRadius;
      sp3[1] = superAzi;
      sp4[0] = sp2[0];
      sp4[1] = superAzi - std::asin(std::sin(superRadius) / std::sin(superColat));
      if (sp4[1] < -PI) sp4[1] += TWO_PI;
    }
  }
  const bool sym = are_equal(superColat, cedeColat) && are_equal(superAzi, 0.0);
  const size_t j_max = sym ? S / 2 : S;
  Region g{cedeColat, cedeRadius, superRadius, superAzi, superColat};
  std::vector<double> colatC(S);
  for (size_t j = 0; j < S * S; j++) o.area[j] = 0.0;
  for (size_t i = 0; i < S; i++) {
    double lower, upper;
    if (i == S - 1) { lower = parallels[i - 1]; upper = lims[1]; }
    else if (i == 0) { lower = lims[0]; upper = parallels[i]; }
    else { lower = parallels[i - 1]; upper = parallels[i]; }
    colatC[i] = integrateArea(lower, upper, s, 1, w) / eta;
    double mu = std::cos(colatC[i]);
    double radius = radiusNormalised(mu, s.epsilon, s.zeta, s.shape);
    o.r[i] = radius * s.R_eq;
    o.effGrav[i] = effectiveGravity(mu, s.R_eq, s.zeta, s.epsilon, s.shape);
    double ft = f_theta(mu, radius, s.epsilon, s.zeta, s.shape);
    o.cos_gamma[i] = 1.0 / std::sqrt(1.0 + ft * ft);
    o.maxAlpha[i] = PI_2 + std::acos(o.cos_gamma[i]);
    int p1 = 0, p3 = 0;
    if (polar && i == 0) {
      p1 = p3 = (cedeColat <= cedeRadius);
      if (p1 == 1) { p1 = p1 * (superRadius <= superColat); p3 = p1; }
      else { p1 = p3 = 2; }
    }
    double leftmost = polar ? -PI : -boundary_phi;
    for (size_t j = 0; j < j_max; j++) {
      double rightmost = leftmost + delta_phi;
      if (!polar || i > 0) {
        p1 = (eval_psi(lower, leftmost, cedeColat) <= cedeRadius);
        p3 = (eval_psi(lower, rightmost, cedeColat) <= cedeRadius);
      }
      int p2 = (eval_psi(upper, leftmost, cedeColat) <= cedeRadius);
      int p4 = (eval_psi(upper, rightmost, cedeColat) <= cedeRadius);
      int p5 = (eval_psi(colatC[i], leftmost + 0.5 * delta_phi, cedeColat) <= cedeRadius);
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
        p5 = p5 * (superRadius <= eval_psi(colatC[i], leftmost + 0.5 * delta_phi - superAzi, superColat));
      else
        p5 = 2;
      double &A = o.area[i * S + j];
      if (!(p1 == p2 && p2 == p3 && p3 == p4 && p4 == p5)) {
        A = integrateCell(lower, upper, leftmost, rightmost, s, g, w);
      } else if (superRadius > 0.0) {
        auto in = [&](const double *q) {
          return lower <= q[0] && q[0] <= upper && leftmost <= q[1] && q[1] <= rightmost;
        };
        if (in(sp1) || in(sp2) || in(sp3) || in(sp4))
          A = integrateCell(lower, upper, leftmost, rightmost, s, g, w);
        else if (p5 == 1)
          A = cellArea;
      } else if (p5 == 1) {
        A = cellArea;
      }
      if (sym) o.area[i * S + (S - 1 - j)] = A;
      leftmost = rightmost;
    }
  }
  for (size_t i = 0; i < S; i++)
    for (size_t j = 0; j < S; j++) {
      o.theta[i * S + j] = invert ? PI - colatC[i] : colatC[i];
      o.phi[i * S + j] = phi1[j];
    }
  return 0;
}

// mesh_tools.pyx:892-1099 (returns the superseding mesh side only; X-PSI's
// cede member is allocated by the same formula and is not used here)
void allocate(size_t num_cells, size_t mn, size_t mx, const Star &s, double superRadius,
              double cedeRadius, double superColat, double cedeColat, double superAzi,
              double holeColat, double holeRadius, double holeAzi, double out[4], Work &w) {
  double super_lims[2], super_cellArea, super_bphi, superColat_cpy = superColat;
  if (superColat - superRadius < 0.0 || superColat + superRadius > PI) {
    super_lims[0] = 0.0;
    if (superColat + superRadius > PI) {
      super_lims[1] = PI - superColat + superRadius;
      superColat = PI - superColat;
      holeColat = PI - holeColat;
    } else {
      super_lims[1] = superColat + superRadius;
    }
    super_bphi = PI;
    super_cellArea = TWO_PI;
  } else {
    super_lims[0] = superColat - superRadius;
    super_lims[1] = superColat + superRadius;
    super_bphi = std::asin(std::sin(superRadius) / std::sin(superColat));
    super_cellArea = 2.0 * super_bphi;
  }
  (void)super_bphi;
  super_cellArea *= integrateArea(super_lims[0], super_lims[1], s, 0, w);
  Region gs{superColat, superRadius, holeRadius, holeAzi, holeColat};
  double super_area = integrateSpot(super_lims[0], super_lims[1], s, gs, w);
  auto clamp_even = [&](double v) {
    if (v < (double)mn) v = (double)mn;
    else if (v > (double)mx) v = (double)mx;
    if ((size_t)v % 2 != 0) v += 1.0;
    return v;
  };
  if (are_equal(cedeRadius, 0.0)) {
    if (are_equal(super_area, 0.0)) super_area = super_cellArea / 1000.0;
    double sq = std::ceil(std::sqrt((double)num_cells * super_cellArea / super_area));
    sq = clamp_even(sq);
    out[0] = sq; out[1] = sq * sq; out[2] = 0.0; out[3] = 0.0;
    return;
  }
  double cede_lims[2], cede_cellArea;
  if (cedeColat - cedeRadius < 0.0 || cedeColat + cedeRadius > PI) {
    cede_lims[0] = 0.0;
    if (cedeColat + cedeRadius > PI) {
      cede_lims[1] = PI - cedeColat + cedeRadius;
      cedeColat = PI - cedeColat;
      superColat = PI - superColat_cpy;
    } else {
      cede_lims[1] = cedeColat + cedeRadius;
      superColat = superColat_cpy;
    }
    cede_cellArea = TWO_PI;
  } else {
    cede_lims[0] = cedeColat - cedeRadius;
    cede_lims[1] = cedeColat + cedeRadius;
    superColat = superColat_cpy;
    cede_cellArea = 2.0 * std::asin(std::sin(cedeRadius) / std::sin(cedeColat));
  }
  cede_cellArea *= integrateArea(cede_lims[0], cede_lims[1], s, 0, w);
  Region gc{cedeColat, cedeRadius, superRadius, superAzi, superColat};
  double cede_area = integrateSpot(cede_lims[0], cede_lims[1], s, gc, w);
  if (are_equal(super_area, 0.0)) super_area = super_cellArea / 1000.0;
  if (are_equal(cede_area, 0.0)) cede_area = cede_cellArea / 1000.0;
  double y = cede_area / super_area - 1.0, sn, cn;
  if (are_equal(y, 0.0)) { sn = 0.5 * num_cells; cn = 0.5 * num_cells; }
  else { sn = (double)num_cells * ((std::sqrt(1.0 + y) - 1.0) / y); cn = (double)num_cells - sn; }
  double ss = clamp_even(std::ceil(std::sqrt(sn * super_cellArea / super_area)));
  double cs = clamp_even(std::ceil(std::sqrt(cn * cede_cellArea / cede_area)));
  out[0] = ss; out[1] = ss * ss; out[2] = cs; out[3] = cs * cs;
}

}  // namespace

extern "C" {

int xgpu_allocate_cells(size_t num_cells, size_t min_sqrt, size_t max_sqrt, double R_eq,
                        double Omega, double zeta, double epsilon, int star_shape_ind,
                        double super_radius, double cede_radius, double super_colatitude,
                        double cede_colatitude, double super_azimuth, double hole_colatitude,
                        double hole_radius, double hole_azimuth, double *out4) {
  Star s{R_eq, epsilon, zeta, Omega, star_shape_ind};
  Work w;
  allocate(num_cells, min_sqrt, max_sqrt, s, super_radius, cede_radius, super_colatitude,
           cede_colatitude, super_azimuth, hole_colatitude, hole_radius, hole_azimuth, out4, w);
  return 0;
}

int xgpu_cell_mesh(int polar, size_t num_cells, size_t S, double R_eq, double zeta,
                   double epsilon, int star_shape_ind, double cede_radius,
                   double cede_colatitude, double super_radius, double super_colatitude,
                   double super_azimuth, double *theta, double *phi, double *r, double *area,
                   double *maxAlpha, double *cos_gamma, double *effGrav) {
  Star s{R_eq, epsilon, zeta, 0.0, star_shape_ind};
  Work w;
  MeshOut o{theta, phi, r, area, maxAlpha, cos_gamma, effGrav};
  return build_mesh(polar != 0, num_cells, S, s, cede_radius, cede_colatitude, super_radius,
                    super_colatitude, super_azimuth, o, w);
}

int xgpu_cell_mesh_many(int n, const xgpu_mesh_request *req, int n_threads) {
  if (n_threads <= 0) n_threads = (int)std::max(1u, std::thread::hardware_concurrency());
  std::vector<std::thread> pool;
  std::vector<int> rc(n, 0);
  auto work = [&](int t) {
    Work w;
    for (int i = t; i < n; i += n_threads) {
      const xgpu_mesh_request &q = req[i];
      Star s{q.R_eq, q.epsilon, q.zeta, 0.0, q.star_shape_ind};
      MeshOut o{q.theta, q.phi, q.r, q.area, q.maxAlpha, q.cos_gamma, q.effGrav};
      rc[i] = build_mesh(q.polar != 0, q.num_cells, q.S, s, q.cede_radius, q.cede_colatitude,
                         q.super_radius, q.super_colatitude, q.super_azimuth, o, w);
    }
  };
  for (int t = 0; t < n_threads; t++) pool.emplace_back(work, t);
  for (auto &th : pool) th.join();
  for (int i = 0; i < n; i++)
    if (rc[i]) return rc[i];
  return 0;
}

}  // extern "C"
