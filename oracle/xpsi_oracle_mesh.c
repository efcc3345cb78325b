/* xpsi_oracle_mesh.c -- the oracle's restatement of X-PSI's cell meshes.
 *
 * TEST INFRASTRUCTURE (the checker and the timed CPU baseline, never the
 * product).  Follows, step by step and in the same floating-point order:
 *
 *   xpsi/cellmesh/mesh_tools.pyx:18-97    radiusNormalised, f_theta
 *   xpsi/surface_radiation_field/effective_gravity_universal.pyx:10-71
 *   xpsi/cellmesh/mesh_tools.pyx:99-154   integrand, integrateArea
 *   xpsi/cellmesh/mesh_tools.pyx:156-158  eval_psi
 *   xpsi/cellmesh/mesh_tools.pyx:238-275  eval_phi, get_interval
 *   xpsi/cellmesh/mesh_tools.pyx:277-364  cell_integrand
 *   xpsi/cellmesh/mesh_tools.pyx:367-402  theta_given_phi
 *   xpsi/cellmesh/mesh_tools.pyx:405-720  integrateCell (with its retry over
 *                                          the element's intersection span)
 *   xpsi/cellmesh/mesh_tools.pyx:723-860  spot_integrand, integrateSpot
 *   xpsi/cellmesh/mesh_tools.pyx:892-1099 allocate_cells
 *   xpsi/cellmesh/mesh.pyx:23-417         construct_spot_cellMesh
 *   xpsi/cellmesh/polar_mesh.pyx:23-430   construct_polar_cellMesh
 *   xpsi/cellmesh/global_mesh.pyx:21-137  construct_closed_cellMesh
 *
 * The quadratures go through the GSL-API subset of gslsub (CQUAD at
 * epsabs 0, epsrel 1e-8, 100-interval workspaces; Steffen interpolation of
 * the 1000-point area table), the same routines the reference's own build
 * here links, so the meshes are bit-identical to that build's.  Where the
 * reference reads a local it never assigned (delta_phi in the fall-through
 * branches of cell_integrand and spot_integrand, get_interval's unreachable
 * pairs), this restatement uses 0.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "gslsub.h"

#define XO_2PI (2.0 * M_PI)
#define XO_HPI (0.5 * M_PI)
static const double xo_c = 2.99792458e8;

/* tools/core.pyx:118-122 */
static int are_equal(double x, double y) { return fabs(x - y) < 1.0e-12; }

/* mesh_tools.pyx:18-54 */
static double radius_normalised(double mu, double epsilon, double zeta, int shape) {
  if (shape == 0) return 1.0 + epsilon * (-0.788 + 1.030 * zeta) * mu * mu;
  return 1.0;
}

/* mesh_tools.pyx:56-97 */
static double f_theta(double mu, double radiusNormed, double epsilon, double zeta, int shape) {
  double d = -2.0 * epsilon * (-0.788 + 1.030 * zeta) * mu * sqrt(1.0 - mu * mu);
  if (shape == 0) return d / (radiusNormed * sqrt(1.0 - 2.0 * zeta / radiusNormed));
  return 0.0;
}

/* effective_gravity_universal.pyx:10-71 */
static double effective_gravity(double mu, double R_eq, double x, double epsilon, int shape) {
  double g_0 = x * xo_c * xo_c / (R_eq * sqrt(1.0 - 2.0 * x));
  double esq = epsilon;
  double esqsq = epsilon * epsilon;
  double c_e = -0.791 + 0.776 * x;
  double c_p = 1.138 - 1.431 * x;
  double d_e = (-1.315 + 2.431 * x) * esq * x;
  double d_p = (0.653 - 2.864 * x) * esq * x;
  double d_60 = (13.47 - 27.13 * x) * esq * x;
  double f_e = -1.172 * x * esqsq;
  double f_p = 0.975 * x * esqsq;
  double g = 1.0;
  g += (c_e + d_e + f_e) * esq * (1.0 - mu * mu);
  g += (c_p + d_p + f_p - d_60) * esq * mu * mu;
  g += d_60 * esq * fabs(mu);
  if (shape == 0) return log10(g * g_0) + 2.0;
  return log10(g_0) + 2.0;
}

/* mesh_tools.pyx:99-121 */
static double area_integrand(double theta, void *params) {
  if (are_equal(theta, 0.0)) return 0.0;
  const double *p = (const double *)params;
  double mu = cos(theta);
  double epsilon = p[0], zeta = p[1];
  int av = (int)p[2], shape = (int)p[3];
  double radius = radius_normalised(mu, epsilon, zeta, shape);
  double f = f_theta(mu, radius, epsilon, zeta, shape);
  if (av == 0) return radius * radius * sqrt(1.0 + f * f) * sin(theta);
  return theta * radius * radius * sqrt(1.0 + f * f) * sin(theta);
}

/* mesh_tools.pyx:123-154 */
static double integrate_area(double lo, double hi, double R_eq, double epsilon, double zeta,
                             int shape, int av, gsl_integration_cquad_workspace *w) {
  double params[4] = {epsilon, zeta, (double)av, (double)shape};
  double integral = 0.0, error = 0.0;
  size_t nevals = 0;
  gsl_function F;
  F.function = area_integrand;
  F.params = params;
  gsl_integration_cquad(&F, lo, hi, 0, 1.0e-8, w, &integral, &error, &nevals);
  return R_eq * R_eq * integral;
}

/* mesh_tools.pyx:156-160 */
static double eval_psi(double theta, double phi, double THETA) {
  return acos(cos(THETA) * cos(theta) + sin(THETA) * sin(theta) * cos(phi));
}

/* mesh_tools.pyx:238-247 */
static double eval_phi(double theta, double THETA, double psi) {
  double cos_phi = cos(psi) - cos(THETA) * cos(theta);
  cos_phi /= sin(THETA) * sin(theta);
  if (!(-1.0 <= cos_phi && cos_phi <= 1.0)) return -1.0;
  return acos(cos_phi);
}

/* mesh_tools.pyx:249-275 */
static double get_interval(double a, double b, double LB, double UB) {
  int ac = (LB <= a && a <= UB), bc = (LB <= b && b <= UB);
  if (ac == 0) ac = 2 * (int)(a > UB);
  if (bc == 0) bc = 2 * (int)(b > UB);
  if (ac == bc) return ac == 1 ? b - a : 0.0;
  if (bc == 1 && ac == 0) return b - LB;
  if (bc == 2 && ac == 1) return UB - a;
  if (bc == 2 && ac == 0) return UB - LB;
  return 0.0;
}

/* the ceding region's azimuthal bounds at theta and the superseding
 * region's (shared by cell_integrand and spot_integrand); returns 0 when the
 * integrand vanishes at theta */
static int region_bounds(double theta, double colat, double cedeRadius, double superRadius,
                         double superAzi, double superColat, double *aLB, double *aUB,
                         double *cLB, double *cUB) {
  *aUB = eval_phi(theta, colat, cedeRadius);
  if (are_equal(*aUB, -1.0)) {
    if (theta + colat < cedeRadius) {
      *aUB = M_PI;
      *aLB = -M_PI;
    } else {
      return 0;
    }
  } else {
    *aLB = -*aUB;
  }
  if (fabs(theta - superColat) > superRadius) {
    *cLB = *cUB = 0.0;
  } else {
    *cUB = eval_phi(theta, superColat, superRadius);
    if (are_equal(*cUB, -1.0)) return 0;
    *cLB = -*cUB;
    *cUB += superAzi;
    *cLB += superAzi;
    if (*cUB > M_PI) *cUB -= XO_2PI;
    if (*cLB < -M_PI) *cLB += XO_2PI;
  }
  return 1;
}

typedef struct {
  double epsilon, zeta, colat, cedeRadius, superRadius, superAzi, superColat, phi_a, phi_b;
  int shape;
} CellParams;

/* mesh_tools.pyx:277-364 */
static double cell_integrand(double theta, void *params) {
  if (are_equal(theta, 0.0)) return 0.0;
  const CellParams *p = (const CellParams *)params;
  double mu = cos(theta);
  double radius = radius_normalised(mu, p->epsilon, p->zeta, p->shape);
  double f = f_theta(mu, radius, p->epsilon, p->zeta, p->shape);
  double aLB, aUB, cLB, cUB, dphi = 0.0;
  if (!region_bounds(theta, p->colat, p->cedeRadius, p->superRadius, p->superAzi,
                     p->superColat, &aLB, &aUB, &cLB, &cUB))
    return 0.0;
  double a = p->phi_a, b = p->phi_b;
  if (cUB >= cLB) {
    if (cLB >= aUB || cUB <= aLB) {
      dphi = get_interval(a, b, aLB, aUB);
    } else if (cLB >= aLB && cUB <= aUB) {
      dphi = get_interval(a, b, aLB, cLB);
      dphi += get_interval(a, b, cUB, aUB);
    } else if (cLB < aLB && aLB < cUB && cUB <= aUB) {
      dphi = get_interval(a, b, cUB, aUB);
    } else if (aLB <= cLB && cLB < aUB && aUB < cUB) {
      dphi = get_interval(a, b, aLB, cLB);
    } else if (cLB < aLB && cUB > aUB) {
      return 0.0;
    }
  } else {
    if (cUB >= aUB || cLB <= aLB) {
      return 0.0;
    } else if (cUB >= aLB && cLB <= aUB) {
      dphi = get_interval(a, b, cUB, cLB);
    } else if (cUB < aLB && aLB < cLB && cLB <= aUB) {
      dphi = get_interval(a, b, aLB, cLB);
    } else if (aLB <= cUB && cUB < aUB && aUB < cLB) {
      dphi = get_interval(a, b, cUB, aUB);
    } else if (cUB < aLB && cLB > aUB) {
      dphi = get_interval(a, b, aLB, aUB);
    }
  }
  return dphi * radius * radius * sqrt(1.0 + f * f) * sin(theta);
}

/* mesh_tools.pyx:367-402 */
static double theta_given_phi(double phi, double colat, double radius, const double interval[2]) {
  double x = sin(colat) * sin(phi) / sin(radius);
  if (!(x <= 1.0)) return -1.0;
  x = asin(x);
  double theta = tan(0.5 * (colat - radius)) / sin(0.5 * (x - phi));
  theta *= sin(0.5 * (x + phi));
  theta = atan(theta);
  if (theta < 0.0) theta *= -2.0;
  else theta *= 2.0;
  if (!(interval[0] <= theta && theta <= interval[1])) {
    x = M_PI - x;
    theta = tan(0.5 * (colat - radius)) / sin(0.5 * (x - phi));
    theta *= sin(0.5 * (x + phi));
    theta = atan(theta);
    if (theta < 0.0) theta *= -2.0;
    else theta *= 2.0;
    if (!(interval[0] <= theta && theta <= interval[1])) return -1.0;
  }
  return theta;
}

/* the element's top or bottom crossing of the ceding region's boundary
 * (mesh_tools.pyx:524-533, 585-594) */
static double cede_edge_phi(double th, double colat, double cedeRadius, double phi_a,
                            double phi_b) {
  double v = eval_phi(th, colat, cedeRadius);
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

/* the same for the superseding region (mesh_tools.pyx:535-575, 596-636);
 * `strict` selects the reference's test on the mirrored branch, which is
 * `> 0` for the top edge and `>= 0` for the bottom edge */
static double super_edge_phi(double th, double superColat, double superRadius, double superAzi,
                             double phi_a, double phi_b, int strict) {
  if (fabs(th - superColat) > superRadius) return -1.0;
  double v = eval_phi(th, superColat, superRadius);
  if (v >= 0.0) {
    v += superAzi;
    if (v > M_PI) v -= XO_2PI;
    if (v < -M_PI) v += XO_2PI;
    if (!(phi_a <= v && v <= phi_b)) v = -1.0;
    else if (v < 0.0) v *= -1.0;
  }
  if (v < 0.0) {
    v = eval_phi(th, superColat, superRadius);
    if (strict ? (v > 0.0) : (v >= 0.0)) {
      v *= -1.0;
      v += superAzi;
      if (v > M_PI) v -= XO_2PI;
      if (v < -M_PI) v += XO_2PI;
      if (!(phi_a <= v && v <= phi_b)) v = -1.0;
      else if (v < 0.0) v *= -1.0;
    }
  }
  return v;
}

/* the first two non-negative candidates in the reference's order (left,
 * right, top, bottom), each consumed once (mesh_tools.pyx:638-692) */
static void take_two(double *left, double *right, double *top, double *bottom, double ta,
                     double tb, double out[2]) {
  for (int k = 0; k < 2; k++) {
    if (*left >= 0.0) {
      out[k] = *left;
      *left = -1.0;
    } else if (*right >= 0.0) {
      out[k] = *right;
      *right = -1.0;
    } else if (*top >= 0.0) {
      out[k] = ta;
      *top = -1.0;
    } else if (*bottom >= 0.0) {
      out[k] = tb;
      *bottom = -1.0;
    } else {
      out[k] = -1.0;
    }
  }
}

/* mesh_tools.pyx:405-720 */
static double integrate_cell(double theta_a, double theta_b, double phi_a, double phi_b,
                             double R_eq, double epsilon, double zeta, int shape, double colat,
                             double cedeRadius, double superRadius, double superAzi,
                             double superColat, gsl_integration_cquad_workspace *w) {
  CellParams p = {epsilon, zeta, colat, cedeRadius, superRadius, superAzi, superColat,
                  phi_a, phi_b, shape};
  double integral = 0.0, error = 0.0;
  size_t nevals = 0;
  gsl_function F;
  F.function = cell_integrand;
  F.params = &p;
  gsl_integration_cquad(&F, theta_a, theta_b, 0, 1.0e-8, w, &integral, &error, &nevals);
  if (are_equal(integral, 0.0)) {
    const double interval[2] = {theta_a, theta_b};
    double tl0 = theta_given_phi(phi_a, colat, cedeRadius, interval);
    double tl1 = theta_given_phi(phi_a - superAzi, superColat, superRadius, interval);
    double tr0 = theta_given_phi(phi_b, colat, cedeRadius, interval);
    double tr1 = theta_given_phi(phi_b - superAzi, superColat, superRadius, interval);
    double pt0 = cede_edge_phi(theta_a, colat, cedeRadius, phi_a, phi_b);
    double pt1 = super_edge_phi(theta_a, superColat, superRadius, superAzi, phi_a, phi_b, 1);
    double pb0 = cede_edge_phi(theta_b, colat, cedeRadius, phi_a, phi_b);
    double pb1 = super_edge_phi(theta_b, superColat, superRadius, superAzi, phi_a, phi_b, 0);
    double cede_t[2], super_t[2];
    take_two(&tl0, &tr0, &pt0, &pb0, theta_a, theta_b, cede_t);
    take_two(&tl1, &tr1, &pt1, &pb1, theta_a, theta_b, super_t);
    double theta_min = theta_b, theta_max = theta_a;
    const double th4[4] = {cede_t[0], cede_t[1], super_t[0], super_t[1]};
    for (int i = 0; i < 4; i++) {
      if (th4[i] >= 0.0) {
        if (th4[i] < theta_min) theta_min = th4[i];
        if (th4[i] > theta_max) theta_max = th4[i];
      }
    }
    if (theta_min < theta_max)
      gsl_integration_cquad(&F, theta_min, theta_max, 0, 1.0e-8, w, &integral, &error, &nevals);
  }
  return R_eq * R_eq * integral;
}

typedef struct {
  double epsilon, zeta, colat, cedeRadius, superRadius, superAzi, superColat, R_eq, Omega;
  int Lorentz, shape;
} SpotParams;

/* mesh_tools.pyx:723-809 */
static double spot_integrand(double theta, void *params) {
  if (are_equal(theta, 0.0)) return 0.0;
  const SpotParams *p = (const SpotParams *)params;
  double mu = cos(theta);
  double radius = radius_normalised(mu, p->epsilon, p->zeta, p->shape);
  double f = f_theta(mu, radius, p->epsilon, p->zeta, p->shape);
  double aLB, aUB, cLB, cUB, dphi = 0.0;
  if (!region_bounds(theta, p->colat, p->cedeRadius, p->superRadius, p->superAzi,
                     p->superColat, &aLB, &aUB, &cLB, &cUB))
    return 0.0;
  if (cUB >= cLB) {
    if (cLB >= aUB || cUB <= aLB) {
      dphi = -aLB + aUB;
    } else if (cLB >= aLB && cUB <= aUB) {
      dphi = -aLB + cLB;
      dphi += -cUB + aUB;
    } else if (cLB < aLB && aLB < cUB && cUB <= aUB) {
      dphi = -cUB + aUB;
    } else if (aLB <= cLB && cLB < aUB && aUB < cUB) {
      dphi = -aLB + cLB;
    } else if (cLB < aLB && cUB > aUB) {
      return 0.0;
    }
  } else {
    if (cUB >= aUB || cLB <= aLB) {
      return 0.0;
    } else if (cUB >= aLB && cLB <= aUB) {
      dphi = -cUB + cLB;
    } else if (cUB < aLB && aLB < cLB && cLB <= aUB) {
      dphi = -aLB + cLB;
    } else if (aLB <= cUB && cUB < aUB && aUB < cLB) {
      dphi = -cUB + aUB;
    } else if (cUB < aLB && cLB > aUB) {
      dphi = -aLB + aUB;
    }
  }
  double v;
  if (p->Lorentz == 1) {
    double rsr = 2.0 * p->zeta / radius;
    double beta = p->R_eq * radius * p->Omega * sin(theta) / (xo_c * sqrt(1.0 - rsr));
    v = 1.0 / sqrt(1.0 - beta * beta);
  } else {
    v = 1.0;
  }
  v *= dphi * radius * radius * sqrt(1.0 + f * f) * sin(theta);
  return v;
}

/* mesh_tools.pyx:812-860 */
static double integrate_spot(double ta, double tb, double R_eq, double epsilon, double zeta,
                             int shape, double colat, double cedeRadius, double superRadius,
                             double superColat, double superAzi, int Lorentz, double Omega,
                             gsl_integration_cquad_workspace *w) {
  SpotParams p = {epsilon, zeta, colat, cedeRadius, superRadius, superAzi, superColat,
                  R_eq, Omega, Lorentz, shape};
  double integral = 0.0, error = 0.0;
  size_t nevals = 0;
  gsl_function F;
  F.function = spot_integrand;
  F.params = &p;
  gsl_integration_cquad(&F, ta, tb, 0, 1.0e-8, w, &integral, &error, &nevals);
  return R_eq * R_eq * integral;
}

/* mesh_tools.pyx:892-1099: out = (super_sqrt, super_num, cede_sqrt, cede_num) */
void xo_allocate_cells(size_t num_cells, size_t min_sqrt, size_t max_sqrt, double R_eq,
                       double Omega, double zeta, double epsilon, int shape,
                       double superRadius, double cedeRadius, double superColat,
                       double cedeColat, double superAzi, double holeColat, double holeRadius,
                       double holeAzi, double out[4]) {
  double super_lims[2], cede_lims[2];
  double super_cellArea, cede_cellArea, super_area, cede_area;
  double superColat_cpy = superColat;
  gsl_integration_cquad_workspace *w = gsl_integration_cquad_workspace_alloc(100);
  if (superColat - superRadius < 0.0 || superColat + superRadius > M_PI) {
    super_lims[0] = 0.0;
    if (superColat + superRadius > M_PI) {
      super_lims[1] = M_PI - superColat + superRadius;
      superColat = M_PI - superColat;
      holeColat = M_PI - holeColat;
    } else {
      super_lims[1] = superColat + superRadius;
    }
    super_cellArea = XO_2PI;
  } else {
    super_lims[0] = superColat - superRadius;
    super_lims[1] = superColat + superRadius;
    super_cellArea = 2.0 * asin(sin(superRadius) / sin(superColat));
  }
  super_cellArea *= integrate_area(super_lims[0], super_lims[1], R_eq, epsilon, zeta, shape, 0, w);
  super_area = integrate_spot(super_lims[0], super_lims[1], R_eq, epsilon, zeta, shape,
                              superColat, superRadius, holeRadius, holeColat, holeAzi, 0, Omega,
                              w);
  if (are_equal(cedeRadius, 0.0)) {
    if (are_equal(super_area, 0.0)) super_area = super_cellArea / 1000.0;
    double s = ceil(sqrt((double)num_cells * super_cellArea / super_area));
    if (s < (double)min_sqrt) s = (double)min_sqrt;
    else if (s > (double)max_sqrt) s = (double)max_sqrt;
    if ((size_t)s % 2 != 0) s += 1.0;
    out[0] = s;
    out[1] = s * s;
    out[2] = 0.0;
    out[3] = 0.0;
    gsl_integration_cquad_workspace_free(w);
    return;
  }
  if (cedeColat - cedeRadius < 0.0 || cedeColat + cedeRadius > M_PI) {
    cede_lims[0] = 0.0;
    if (cedeColat + cedeRadius > M_PI) {
      cede_lims[1] = M_PI - cedeColat + cedeRadius;
      cedeColat = M_PI - cedeColat;
      superColat = M_PI - superColat_cpy;
    } else {
      cede_lims[1] = cedeColat + cedeRadius;
      superColat = superColat_cpy;
    }
    cede_cellArea = XO_2PI;
  } else {
    cede_lims[0] = cedeColat - cedeRadius;
    cede_lims[1] = cedeColat + cedeRadius;
    superColat = superColat_cpy;
    cede_cellArea = 2.0 * asin(sin(cedeRadius) / sin(cedeColat));
  }
  cede_cellArea *= integrate_area(cede_lims[0], cede_lims[1], R_eq, epsilon, zeta, shape, 0, w);
  cede_area = integrate_spot(cede_lims[0], cede_lims[1], R_eq, epsilon, zeta, shape, cedeColat,
                             cedeRadius, superRadius, superColat, superAzi, 0, Omega, w);
  if (are_equal(super_area, 0.0)) super_area = super_cellArea / 1000.0;
  if (are_equal(cede_area, 0.0)) cede_area = cede_cellArea / 1000.0;
  double y = (cede_area / super_area) - 1.0, super_num, cede_num;
  if (are_equal(y, 0.0)) {
    super_num = 0.5 * (double)num_cells;
    cede_num = 0.5 * (double)num_cells;
  } else {
    super_num = (double)num_cells * ((sqrt(1.0 + y) - 1.0) / y);
    cede_num = (double)num_cells - super_num;
  }
  double ss = ceil(sqrt(super_num * super_cellArea / super_area));
  double cs = ceil(sqrt(cede_num * cede_cellArea / cede_area));
  if (ss < (double)min_sqrt) ss = (double)min_sqrt;
  else if (ss > (double)max_sqrt) ss = (double)max_sqrt;
  if (cs < (double)min_sqrt) cs = (double)min_sqrt;
  else if (cs > (double)max_sqrt) cs = (double)max_sqrt;
  if ((size_t)ss % 2 != 0) ss += 1.0;
  if ((size_t)cs % 2 != 0) cs += 1.0;
  out[0] = ss;
  out[1] = ss * ss;
  out[2] = cs;
  out[3] = cs * cs;
  gsl_integration_cquad_workspace_free(w);
}

/* numpy.linspace(start, stop, n): start + i * step, the last point exactly stop */
static void linspace(double start, double stop, size_t n, double *out) {
  if (n == 0) return;
  if (n == 1) {
    out[0] = start;
    return;
  }
  double step = (stop - start) / (double)(n - 1);
  for (size_t i = 0; i < n; i++) out[i] = (double)i * step + start;
  out[n - 1] = stop;
}

/* the superseding region's points where its boundary is tangent to a
 * coordinate line (mesh.pyx:137-187, polar_mesh.pyx:133-183) */
static void super_points(double superRadius, double superColat, double superAzi,
                         double pts[4][2]) {
  memset(pts, 0, sizeof(double) * 8);
  if (!(superRadius > 0.0)) return;
  if (superColat - superRadius < 0.0) {
    pts[0][0] = superRadius - superColat;
    pts[0][1] = superAzi + M_PI;
    if (pts[0][1] > M_PI) pts[0][1] = pts[0][1] - XO_2PI;
    pts[1][0] = superColat + superRadius;
    pts[1][1] = superAzi;
  } else if (superColat + superRadius > M_PI) {
    pts[0][0] = superColat - superRadius;
    pts[0][1] = superAzi;
    pts[1][0] = XO_2PI - superColat - superRadius;
    pts[1][1] = superAzi + M_PI;
    if (pts[1][1] > M_PI) pts[1][1] = pts[1][1] - XO_2PI;
  } else {
    pts[0][0] = superColat - superRadius;
    pts[0][1] = superAzi;
    pts[1][0] = acos(cos(superColat) / cos(superRadius));
    pts[1][1] = superAzi + asin(sin(superRadius) / sin(superColat));
    if (pts[1][1] > M_PI) pts[1][1] = pts[1][1] - XO_2PI;
    pts[2][0] = superColat + superRadius;
    pts[2][1] = superAzi;
    pts[3][0] = pts[1][0];
    pts[3][1] = superAzi - asin(sin(superRadius) / sin(superColat));
    if (pts[3][1] < -M_PI) pts[3][1] = pts[3][1] + XO_2PI;
  }
}

/* flag of one corner or centre: 1 inside the ceding region and outside the
 * superseding one, 0 inside both, 2 outside the ceding region */
static int corner_flag(double th, double ph, double colat, double cedeRadius,
                       double superRadius, double superAzi, double superColat) {
  int p = (eval_psi(th, ph, colat) <= cedeRadius);
  if (p == 1) return p * (superRadius <= eval_psi(th, ph - superAzi, superColat));
  return 2;
}

/* mesh.pyx:23-417 (polar = 0) and polar_mesh.pyx:23-430 (polar = 1).
 * Outputs theta[S] (cell colatitude per parallel), phi[S] (cell azimuth per
 * column), r[S], area[S][S], maxAlpha[S], cos_gamma[S], effGrav[S].
 * Parallels are computed on n_threads OpenMP threads (each row's work is
 * independent, so the result does not depend on the thread count). */
int xo_cell_mesh(int polar, size_t numCell, size_t S, double R_eq, double zeta, double epsilon,
                 int shape, double cedeRadius, double cedeColat, double superRadius,
                 double superColat, double superAzi, int n_threads, double *theta,
                 double *phi_out, double *r, double *area, double *maxAlpha, double *cos_gamma,
                 double *effGrav) {
  if (S < 2) return -1;
  double lims[2], boundary_phi = M_PI, delta_phi;
  int invert = 0;
  gsl_integration_cquad_workspace *w0 = gsl_integration_cquad_workspace_alloc(100);
  double cellArea;
  if (polar) {
    lims[0] = 0.0;
    if (cedeColat + cedeRadius > M_PI) {
      invert = 1;
      lims[1] = M_PI - cedeColat + cedeRadius;
      cedeColat = M_PI - cedeColat;
      superColat = M_PI - superColat;
    } else {
      lims[1] = cedeColat + cedeRadius;
    }
    cellArea = XO_2PI * integrate_area(0.0, lims[1], R_eq, epsilon, zeta, shape, 0, w0);
    delta_phi = XO_2PI / (double)S;
    linspace(-M_PI + 0.5 * delta_phi, M_PI - 0.5 * delta_phi, S, phi_out);
  } else {
    lims[0] = cedeColat - cedeRadius;
    lims[1] = cedeColat + cedeRadius;
    boundary_phi = asin(sin(cedeRadius) / sin(cedeColat));
    cellArea = 2.0 * boundary_phi;
    cellArea *= integrate_area(lims[0], lims[1], R_eq, epsilon, zeta, shape, 0, w0);
    delta_phi = 2.0 * boundary_phi / (double)S;
    linspace(-boundary_phi + 0.5 * delta_phi, boundary_phi - 0.5 * delta_phi, S, phi_out);
  }
  double colatTab[1000], areaTab[1000];
  linspace(lims[1], lims[0], 1000, colatTab);
  cellArea /= (double)numCell;
  const double eta = cellArea / delta_phi;
  if (n_threads < 1) n_threads = 1;
#pragma omp parallel num_threads(n_threads)
  {
    gsl_integration_cquad_workspace *w = gsl_integration_cquad_workspace_alloc(100);
#pragma omp for schedule(static)
    for (int i = 0; i < 1000; i++)
      areaTab[i] = integrate_area(colatTab[i], lims[1], R_eq, epsilon, zeta, shape, 0, w);
    gsl_integration_cquad_workspace_free(w);
  }
  double *parallels = (double *)malloc(sizeof(double) * (S - 1));
  {
    gsl_interp *interp = gsl_interp_alloc(gsl_interp_steffen, 1000);
    gsl_interp_accel *acc = gsl_interp_accel_alloc();
    gsl_interp_init(interp, areaTab, colatTab, 1000);
    double i_eta = (double)S * eta;
    for (size_t i = 0; i + 1 < S; i++) {
      i_eta -= eta;
      parallels[i] = gsl_interp_eval(interp, areaTab, colatTab, i_eta, acc);
    }
    gsl_interp_free(interp);
    gsl_interp_accel_free(acc);
  }
  double pts[4][2];
  super_points(superRadius, superColat, superAzi, pts);
  const int sym = are_equal(superColat, cedeColat) && are_equal(superAzi, 0.0);
  const size_t j_max = sym ? S / 2 : S;
  memset(area, 0, sizeof(double) * S * S);
  const double left0 = polar ? -M_PI : -boundary_phi;
#pragma omp parallel num_threads(n_threads)
  {
    gsl_integration_cquad_workspace *w = gsl_integration_cquad_workspace_alloc(100);
#pragma omp for schedule(static, 1)
    for (long ii = 0; ii < (long)S; ii++) {
      const size_t i = (size_t)ii;
      double lower, upper;
      if (i == S - 1) {
        lower = parallels[i - 1];
        upper = lims[1];
      } else if (i == 0) {
        lower = lims[0];
        upper = parallels[i];
      } else {
        lower = parallels[i - 1];
        upper = parallels[i];
      }
      theta[i] = integrate_area(lower, upper, R_eq, epsilon, zeta, shape, 1, w) / eta;
      const double mu = cos(theta[i]);
      const double radius = radius_normalised(mu, epsilon, zeta, shape);
      r[i] = radius * R_eq;
      effGrav[i] = effective_gravity(mu, R_eq, zeta, epsilon, shape);
      const double f = f_theta(mu, radius, epsilon, zeta, shape);
      cos_gamma[i] = 1.0 / sqrt(1.0 + f * f);
      maxAlpha[i] = XO_HPI + acos(cos_gamma[i]);
      int p1 = 0, p3 = 0;
      if (polar && i == 0) {
        p1 = p3 = (cedeColat <= cedeRadius);
        if (p1 == 1) {
          p1 = p1 * (superRadius <= superColat);
          p3 = p1;
        } else {
          p1 = p3 = 2;
        }
      }
      double leftmost = left0;
      for (size_t j = 0; j < j_max; j++) {
        const double rightmost = leftmost + delta_phi;
        const double mid = leftmost + 0.5 * delta_phi;
        if (!polar || i > 0) {
          p1 = corner_flag(lower, leftmost, cedeColat, cedeRadius, superRadius, superAzi,
                           superColat);
          p3 = corner_flag(lower, rightmost, cedeColat, cedeRadius, superRadius, superAzi,
                           superColat);
        }
        const int p2 = corner_flag(upper, leftmost, cedeColat, cedeRadius, superRadius,
                                   superAzi, superColat);
        const int p4 = corner_flag(upper, rightmost, cedeColat, cedeRadius, superRadius,
                                   superAzi, superColat);
        const int p5 = corner_flag(theta[i], mid, cedeColat, cedeRadius, superRadius, superAzi,
                                   superColat);
        double A = 0.0;
        if (!(p1 == p2 && p2 == p3 && p3 == p4 && p4 == p5)) {
          A = integrate_cell(lower, upper, leftmost, rightmost, R_eq, epsilon, zeta, shape,
                             cedeColat, cedeRadius, superRadius, superAzi, superColat, w);
        } else if (superRadius > 0.0) {
          int hit = 0;
          for (int k = 0; k < 4; k++)
            if (lower <= pts[k][0] && pts[k][0] <= upper && leftmost <= pts[k][1] &&
                pts[k][1] <= rightmost)
              hit = 1;
          if (hit)
            A = integrate_cell(lower, upper, leftmost, rightmost, R_eq, epsilon, zeta, shape,
                               cedeColat, cedeRadius, superRadius, superAzi, superColat, w);
          else if (p5 == 1)
            A = cellArea;
        } else if (p5 == 1) {
          A = cellArea;
        }
        area[i * S + j] = A;
        if (sym) area[i * S + (S - 1 - j)] = A;
        leftmost = rightmost;
      }
    }
    gsl_integration_cquad_workspace_free(w);
  }
  if (invert)
    for (size_t i = 0; i < S; i++) theta[i] = M_PI - theta[i];
  free(parallels);
  gsl_integration_cquad_workspace_free(w0);
  return 0;
}

/* global_mesh.pyx:21-137: the closed mesh of the photosphere elsewhere.
 * Outputs theta[S], phi[S], r[S], maxAlpha[S], cos_gamma[S], effGrav[S] and
 * returns the (uniform) cell area through *cell_area. */
int xo_closed_cell_mesh(size_t S, size_t numCell, double R_eq, double zeta, double epsilon,
                        int shape, int n_threads, double *theta, double *phi_out, double *r,
                        double *cell_area, double *maxAlpha, double *cos_gamma,
                        double *effGrav) {
  const size_t nc = S / 2;
  if (nc < 2) return -1;
  gsl_integration_cquad_workspace *w0 = gsl_integration_cquad_workspace_alloc(100);
  double colatTab[1000], areaTab[1000];
  linspace(XO_HPI, 0.0, 1000, colatTab);
  double cellArea = XO_2PI * integrate_area(0.0, XO_HPI, R_eq, epsilon, zeta, shape, 0, w0) /
                    (double)numCell;
  cellArea *= 2.0;
  const double eta = cellArea * (double)S / XO_2PI;
  if (n_threads < 1) n_threads = 1;
#pragma omp parallel num_threads(n_threads)
  {
    gsl_integration_cquad_workspace *w = gsl_integration_cquad_workspace_alloc(100);
#pragma omp for schedule(static)
    for (int i = 0; i < 1000; i++)
      areaTab[i] = integrate_area(colatTab[i], XO_HPI, R_eq, epsilon, zeta, shape, 0, w);
    gsl_integration_cquad_workspace_free(w);
  }
  double *parallels = (double *)malloc(sizeof(double) * (nc - 1));
  {
    gsl_interp *interp = gsl_interp_alloc(gsl_interp_steffen, 1000);
    gsl_interp_accel *acc = gsl_interp_accel_alloc();
    gsl_interp_init(interp, areaTab, colatTab, 1000);
    double i_eta = (double)nc * eta;
    for (size_t i = 0; i + 1 < nc; i++) {
      i_eta -= eta;
      parallels[i] = gsl_interp_eval(interp, areaTab, colatTab, i_eta, acc);
    }
    gsl_interp_free(interp);
    gsl_interp_accel_free(acc);
  }
#pragma omp parallel num_threads(n_threads)
  {
    gsl_integration_cquad_workspace *w = gsl_integration_cquad_workspace_alloc(100);
#pragma omp for schedule(static, 1)
    for (long ii = 0; ii < (long)nc; ii++) {
      const size_t i = (size_t)ii;
      if (i == nc - 1)
        theta[i] = integrate_area(parallels[i - 1], XO_HPI, R_eq, epsilon, zeta, shape, 1, w) / eta;
      else if (i == 0)
        theta[i] = integrate_area(0.0, parallels[i], R_eq, epsilon, zeta, shape, 1, w) / eta;
      else
        theta[i] = integrate_area(parallels[i - 1], parallels[i], R_eq, epsilon, zeta, shape, 1,
                                  w) / eta;
      const double mu = cos(theta[i]);
      const double radius = radius_normalised(mu, epsilon, zeta, shape);
      r[i] = radius * R_eq;
      effGrav[i] = effective_gravity(mu, R_eq, zeta, epsilon, shape);
      const double f = f_theta(mu, radius, epsilon, zeta, shape);
      cos_gamma[i] = 1.0 / sqrt(1.0 + f * f);
      maxAlpha[i] = XO_HPI + acos(cos_gamma[i]);
    }
    gsl_integration_cquad_workspace_free(w);
  }
  const double delta_phi = XO_2PI / (double)S;
  linspace(-M_PI + 0.5 * delta_phi, M_PI - 0.5 * delta_phi, S, phi_out);
  for (size_t i = nc; i < S; i++) {
    theta[i] = M_PI - theta[S - i - 1];
    r[i] = r[S - i - 1];
    cos_gamma[i] = cos_gamma[S - i - 1];
    effGrav[i] = effGrav[S - i - 1];
    maxAlpha[i] = maxAlpha[S - i - 1];
  }
  *cell_area = cellArea;
  free(parallels);
  gsl_integration_cquad_workspace_free(w0);
  return 0;
}
