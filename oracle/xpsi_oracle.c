/*
 * xpsi_oracle.c -- CPU restatement of X-PSI's pulse-likelihood path (FP64).
 *
 * TEST INFRASTRUCTURE: this is the oracle.  Only tests/, the smoke check and
 * bench.py's CPU-baseline leg may load it, and only as the checker or the
 * timed CPU baseline -- never as the product path.  It follows the reference
 * Cython line by line (citations are file:line in the xpsi source tree) and
 * uses the oracle's GSL-API subset (gslsub) for splines and quadrature, as
 * the reference uses GSL.  Parity of this file with the reference modules
 * (built by build_ref.py) is checked in tests/test_oracle_vs_reference.py
 * and through the committed golden fixtures.
 *
 * Stages:
 *   xo_compute_rays          cellmesh/rays.pyx:249-390 (+ rayIntegrator :90-247)
 *   xo_integrate             cellmesh/integrator_for_azimuthal_invariance.pyx:70-665,
 *                            with Stokes Q and U as
 *                            cellmesh/integratorIQU_for_azimuthal_invariance.pyx:68-743
 *                            (atmospheres 1, 2, 3 = hot_BB_burst.pyx,
 *                            4 = hot_Num2D.pyx)
 *                            atmospheres: hot_BB.pyx:54-98, hot_Num4D.pyx:248-461
 *   xo_integrate_split       cellmesh/integrator_for_azimuthal_invariance_split.pyx
 *                            (hot_Num5D_split.pyx, hot_Num2D_split.pyx)
 *   xo_integrate_split_iqu   cellmesh/integratorIQU_for_azimuthal_invariance_split.pyx
 *   xo_integrate_general     cellmesh/integrator.pyx:48-667 (symmetry=False),
 *                            with Stokes Q and U as cellmesh/integratorIQU.pyx
 *   xo_integrate_time_invariant  cellmesh/integrator_for_time_invariance.pyx:59-338
 *   xo_energy_integrator     tools/energy_integrator.pyx:27-114
 *   xo_expected_counts       tools/compute_expected_counts.pyx:200-276
 *   xo_phase_integrator      tools/phase_integrator.pyx:23-121
 *   xo_phase_interpolator    tools/phase_interpolator.pyx:25-95
 *   xo_energy_interpolator   tools/energy_interpolator.pyx:27-113
 *   xo_precomputation        likelihoods/default_background_marginalisation.pyx:38-68
 *   xo_eval_marginal_likelihood   same file :176-734 and
 *                            tools/compute_expected_counts.pyx:66-197
 */
#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "gslsub.h"

#define XO_PI 3.14159265358979323846
static const double kPi = XO_PI;
static const double kHalfPi = XO_PI / 2.0;
static const double kTwoPi = 2.0 * XO_PI;
static const double kC = 2.99792458e8;            /* global_imports.py _c */
static const double kKeV = 1.60217662e-16;        /* global_imports.py _keV */
static const double kKB = 1.38064852e-23;         /* global_imports.py _k_B */
static const double kHKeV = 4.135667662e-18;      /* global_imports.py _h_keV */
static const double kErg = 1.0e-7;                /* hot_BB.pyx:23 */
static const double kPlanck = 5.040366110812353e22; /* hot_BB.pyx:24 */

/* tools/core.pyx:118-122 */
static int are_equal(double x, double y) { return fabs(x - y) < 1.0e-12; }

/* ================================================================== */
/* rays                                                               */
/* ================================================================== */
static const double kBPhotonSphere = 2.598076211353316; /* 3 sqrt(3) / 2, rays.pyx:59 */

/* rays.pyx:53-57 */
static double image_deflection(int order, double psi) {
  if (order % 2 != 0)
    return (double)(order + 1) * kPi + pow(-1.0, (double)order) * psi;
  return (double)order * kPi + pow(-1.0, (double)order) * psi;
}

/* rays.pyx:61-88 */
static double f_in_def(double x, void *p) {
  double rc = ((double *)p)[0];
  return 1.0 / sqrt(2.0 - x * x - (1.0 - x * x) * (1.0 - x * x) / (rc - 1.0));
}
static double f_in_lag(double x, void *p) {
  double rc = ((double *)p)[0];
  double X = 1.0 / sqrt(2.0 - x * x - (1.0 - x * x) * (1.0 - x * x) / (rc - 1.0));
  return X * X / (x + X);
}
static double f_out_def(double x, void *p) {
  double sas = ((double *)p)[0], Rr = ((double *)p)[1];
  return x / sqrt(1.0 - sas + x * x * sas * (2.0 - x * x - (1.0 - x * x) * (1.0 - x * x) / (Rr - 1.0)));
}
static double f_out_lag(double x, void *p) {
  double sas = ((double *)p)[0], Rr = ((double *)p)[1];
  double f = sqrt(1.0 - sas + x * x * sas * (2.0 - x * x - (1.0 - x * x) * (1.0 - x * x) / (Rr - 1.0)));
  return x / (f + f * f);
}

/* rays.pyx:90-247: out[0] = deflection, out[2] = lag (s) */
static void ray_integrator(gsl_integration_workspace *w, double cos_alpha,
                           double r_s, double u, double out[4]) {
  int status = GSL_SUCCESS;
  double outp[2], inp[1];
  gsl_function fd, fl;
  double sas = 1.0 - cos_alpha * cos_alpha;
  double sa = sqrt(sas);
  double alpha = acos(cos_alpha);
  double b = sa / (u * sqrt(1.0 - u));
  if (b <= kBPhotonSphere) {
    outp[0] = sas;
    outp[1] = 1.0 / u;
    fd.function = f_out_def; fd.params = outp;
    fl.function = f_out_lag; fl.params = outp;
    status = gsl_integration_qag(&fd, 0.0, 1.0, 0, 1.0e-12, 100, GSL_INTEG_GAUSS61, w, &out[0], &out[1]);
    if (status == GSL_EFAILED) out[0] = NAN;
    if (status != GSL_EFAILED) {
      status = gsl_integration_qag(&fl, 0.0, 1.0, 0, 1.0e-12, 100, GSL_INTEG_GAUSS61, w, &out[2], &out[3]);
      if (status == GSL_EFAILED) out[0] = NAN;
    }
    if (status != GSL_EFAILED) {
      out[0] *= 2.0 * b * u;
      out[2] *= 2.0 * b * b * u * r_s;
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
    inp[0] = rc;
    fd.function = f_in_def; fd.params = inp;
    fl.function = f_in_lag; fl.params = inp;
    if (isnan(wR)) wR = 0.0;
    status = gsl_integration_qag(&fd, wR, 1.0, 0, 1.0e-12, 100, GSL_INTEG_GAUSS61, w, &out[0], &out[1]);
    if (status == GSL_EFAILED) out[0] = NAN;
    if (status != GSL_EFAILED) {
      status = gsl_integration_qag(&fl, wR, 1.0, 0, 1.0e-12, 100, GSL_INTEG_GAUSS61, w, &out[2], &out[3]);
      if (status == GSL_EFAILED) out[0] = NAN;
    }
    if (status != GSL_EFAILED) {
      out[0] *= 2.0 * b / rc;
      out[2] *= 2.0 * b * b * r_s / rc;
    }
  } else if (alpha > kPi / 2.0) {
    double dd[2], dl[2], e;
    double rc = 2.0 * b * cos((atan(sqrt(4.0 * b * b / 27.0 - 1.0)) - kPi) / 3.0) / sqrt(3.0);
    inp[0] = rc;
    fd.function = f_in_def; fd.params = inp;
    fl.function = f_in_lag; fl.params = inp;
    double wR = sqrt(1.0 - rc * u);
    if (isnan(wR)) wR = 0.0;
    status = gsl_integration_qag(&fd, 0.0, 1.0, 0, 1.0e-12, 100, GSL_INTEG_GAUSS61, w, &dd[1], &e);
    if (status == GSL_EFAILED) out[0] = NAN;
    if (status != GSL_EFAILED) {
      status = gsl_integration_qag(&fd, wR, 1.0, 0, 1.0e-12, 100, GSL_INTEG_GAUSS61, w, &dd[0], &e);
      if (status == GSL_EFAILED) out[0] = NAN;
    }
    if (status != GSL_EFAILED) {
      status = gsl_integration_qag(&fl, 0.0, 1.0, 0, 1.0e-12, 100, GSL_INTEG_GAUSS61, w, &dl[1], &e);
      if (status == GSL_EFAILED) out[0] = NAN;
    }
    if (status != GSL_EFAILED) {
      status = gsl_integration_qag(&fl, wR, 1.0, 0, 1.0e-12, 100, GSL_INTEG_GAUSS61, w, &dl[0], &e);
      if (status == GSL_EFAILED) out[0] = NAN;
    }
    if (status != GSL_EFAILED) {
      out[0] = 2.0 * b * (2.0 * dd[1] - dd[0]) / rc;
      out[2] = 2.0 * b * b * r_s * (2.0 * dl[1] - dl[0]) / rc;
      double cor = 1.0 / u - rc + log((1.0 / u - 1.0) / (rc - 1.0));
      out[2] += 2.0 * r_s * cor;
    }
  }
  if (status != GSL_EFAILED) out[2] /= kC;
}

/* rays.pyx:249-390.  Rows are independent; the NaN-repair counter is kept
 * per row (the reference keeps it per OpenMP thread, which is equivalent
 * whenever a row finishes without a fatal flag). */
int xo_compute_rays(int n_threads, size_t N_u, double r_s,
                    const double *u_arr, double *maxAlpha, size_t N_R,
                    double *deflection, double *cos_alpha, double *lag,
                    double *maxDeflection) {
  int terminate = 0;
  gsl_error_handler_t *prev = gsl_set_error_handler_off();
  const double eps = 1.0e-8;
#pragma omp parallel num_threads(n_threads > 0 ? n_threads : 1) reduction(| : terminate)
  {
    gsl_integration_workspace *w = gsl_integration_workspace_alloc(100);
    int term = 0;
#pragma omp for schedule(static, 1)
    for (long ii = 0; ii < (long)N_u; ii++) {
      size_t i = (size_t)ii;
      double u = u_arr[i], extreme = 0.0;
      double *D = deflection + i * N_R, *CA = cos_alpha + i * N_R, *L = lag + i * N_R;
      size_t icount = 0, iidx = 0;
      if (u < 2.0 / 3.0)
        extreme = kPi - asin(sqrt(1.0 - u) * kBPhotonSphere * u);
      else if (are_equal(u, 2.0 / 3.0))
        extreme = kPi / 2.0;
      else if (2.0 / 3.0 < u && u < 1.0)
        extreme = asin(sqrt(1.0 - u) * kBPhotonSphere * u);
      if (maxAlpha[i] >= (1.0 - eps) * extreme) maxAlpha[i] = (1.0 - eps) * extreme;
      double inc = (1.0 - cos(maxAlpha[i])) / ((double)N_R - 1.0);
      for (size_t j = 0; j < N_R; j++) {
        CA[j] = 1.0 - (double)j * inc;
        if (j == 0) {
          CA[j] = 1.0;
          D[j] = 0.0;
          L[j] = 0.0;
          continue;
        }
        if (term) continue;
        double rp[4] = {0, 0, 0, 0};
        ray_integrator(w, CA[j], r_s, u, rp);
        if (j == N_R - 1 && (isnan(rp[0]) || rp[0] <= D[j - 1])) {
          term = 1;
        } else if (icount > 0 && !isnan(rp[0]) && 0.0 <= rp[0] && rp[0] < 100.0 * kPi &&
                   rp[0] > D[iidx]) {
          D[j] = rp[0];
          L[j] = rp[2];
          double delta = (double)icount + 1.0;
          for (size_t k = 1; k <= icount; k++) {
            D[iidx + k] = D[j] * (double)k;
            D[iidx + k] += D[iidx] * (delta - (double)k);
            D[iidx + k] /= delta;
            L[iidx + k] = L[j] * (double)k;
            L[iidx + k] += L[iidx] * (delta - (double)k);
            L[iidx + k] /= delta;
          }
          icount = 0;
        } else if (isnan(rp[0]) || rp[0] < 0.0 || rp[0] > 100.0 * kPi) {
          if (icount == 0) iidx = j - 1;
          icount++;
        } else {
          D[j] = rp[0];
          L[j] = rp[2];
        }
      }
      maxDeflection[i] = D[N_R - 1];
    }
    if (term) terminate = 1;
    gsl_integration_workspace_free(w);
  }
  gsl_set_error_handler(prev);
  return terminate;
}

/* ================================================================== */
/* atmospheres                                                        */
/* ================================================================== */
typedef struct {
  /* numerical 4-D table, dims (logT, logg, mu, log10(E/kT)), row major;
   * for the 2-D tables (atm_ext 4: Pol_Num2D, dims (mu, log10 E);
   * atm_ext 6: a split atmosphere reduced to (mu, E)) only mu, logE, I and,
   * for Stokes Q, the Q table on the same grids */
  const double *logT, *logg, *mu, *logE, *I;
  size_t nT, ng, nmu, nE;
  const double *Q;
} xo_atmos4d;

/* hot_BB.pyx:54-82 (times the norm :84-98 applied by the caller) */
static double eval_bb(double E, const double *vec) {
  double temp = (kKB / kKeV) * pow(10.0, vec[0]);
  return E * E * E / (exp(E / temp) - 1.0);
}

/* Per-thread state of the reference's Num4D evaluator
 * (hot_Num4D.pyx:66-199, ACCELERATE): the base node of each dimension's
 * 4-point stencil persists between calls.  The evaluator only moves a base
 * node when the query leaves the stencil's central interval, and it clamps an
 * out-of-table query only on the call that moves the node, so its output for
 * out-of-range arguments depends on the call history.  The oracle keeps that
 * state exactly as the reference does (one state per OpenMP thread, reset at
 * every integrator call). */
typedef struct {
  size_t BN[4];
  double node[8];
} num4d_state;

static void num4d_reset(num4d_state *st, const xo_atmos4d *A) {
  const double *g[4] = {A->logT, A->logg, A->mu, A->logE};
  for (int d = 0; d < 4; d++) {
    st->BN[d] = 0;
    st->node[2 * d] = g[d][1];
    st->node[2 * d + 1] = g[d][2];
  }
}

/* hot_Num4D.pyx:248-439 */
static double eval_num4d(const xo_atmos4d *A, num4d_state *st, double E,
                         double mu, const double *vec) {
  double v[4];
  double E_eff = (kKB / kKeV) * pow(10.0, vec[0]);
  v[0] = vec[0];
  v[1] = vec[1];
  v[2] = mu;
  v[3] = log10(E / E_eff);
  const double *g[4] = {A->logT, A->logg, A->mu, A->logE};
  size_t n[4] = {A->nT, A->ng, A->nmu, A->nE};
  size_t *BN = st->BN;
  double *node = st->node;
  for (int i = 0; i < 4; i++) {
    const double *P = g[i];
    if (v[i] < node[2 * i] && BN[i] != 0) {
      while (v[i] < P[BN[i] + 1]) {
        if (BN[i] > 0) BN[i] -= 1;
        else if (v[i] <= P[0]) { v[i] = P[0]; break; }
        else break;
      }
      node[2 * i] = P[BN[i] + 1];
      node[2 * i + 1] = P[BN[i] + 2];
    } else if (v[i] > node[2 * i + 1] && BN[i] != n[i] - 4) {
      while (v[i] > P[BN[i] + 2]) {
        if (BN[i] < n[i] - 4) BN[i] += 1;
        else if (v[i] >= P[n[i] - 1]) { v[i] = P[n[i] - 1]; break; }
        else break;
      }
      node[2 * i] = P[BN[i] + 1];
      node[2 * i + 1] = P[BN[i] + 2];
    }
  }
  double w[4][4];
  for (int d = 0; d < 4; d++) {
    const double *P = g[d];
    size_t b = BN[d];
    double x = v[d];
    double d0 = (x - P[b + 1]) * (x - P[b + 2]) * (x - P[b + 3]);
    double d1 = (x - P[b]) * (x - P[b + 2]) * (x - P[b + 3]);
    double d2 = (x - P[b]) * (x - P[b + 1]) * (x - P[b + 3]);
    double d3 = (x - P[b]) * (x - P[b + 1]) * (x - P[b + 2]);
    double s0 = 1.0 / (P[b] - P[b + 1]); s0 /= P[b] - P[b + 2]; s0 /= P[b] - P[b + 3];
    double s1 = 1.0 / (P[b + 1] - P[b]); s1 /= P[b + 1] - P[b + 2]; s1 /= P[b + 1] - P[b + 3];
    double s2 = 1.0 / (P[b + 2] - P[b]); s2 /= P[b + 2] - P[b + 1]; s2 /= P[b + 2] - P[b + 3];
    double s3 = 1.0 / (P[b + 3] - P[b]); s3 /= P[b + 3] - P[b + 1]; s3 /= P[b + 3] - P[b + 2];
    w[d][0] = d0 * s0; w[d][1] = d1 * s1; w[d][2] = d2 * s2; w[d][3] = d3 * s3;
  }
  size_t S0 = A->ng * A->nmu * A->nE, S1 = A->nmu * A->nE, S2 = A->nE;
  double I = 0.0;
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++)
      for (int k = 0; k < 4; k++)
        for (int l = 0; l < 4; l++) {
          double t = w[0][i] * w[1][j] * w[2][k] * w[3][l];
          I += t * A->I[(BN[0] + i) * S0 + (BN[1] + j) * S1 + (BN[2] + k) * S2 + BN[3] + l];
        }
  if (I < 0.0) return 0.0;
  return I * pow(10.0, 3.0 * v[0]);
}

/* cellmesh/common_functions.pyx:7-66: the polarisation angle in the oblate
 * Schwarzschild approximation (Loktev et al. 2020) */
static double pol_angle(double leaf, double sin_psi, double cos_psi, double sin_alpha,
                        double cos_alpha, double sin_th, double cos_th, double sin_i,
                        double cos_i, double sin_gamma, double cos_gamma, double Grav_z,
                        double mu, double eta, double beta, double Lorentz, double cos_xi) {
  double sin_chi_0 = -sin_th * sin(leaf);
  double cos_chi_0 = sin_i * cos_th - sin_th * cos_i * cos(leaf);
  double chi_0 = atan2(sin_chi_0, cos_chi_0);
  double sa_over_sp = !are_equal(sin_psi, 0.0) ? sin_alpha / sin_psi : Grav_z;
  double sin_chi_1 = sin_gamma * sin_i * sin(leaf) * sa_over_sp;
  double cos_chi_1 = cos_gamma - cos_alpha * mu;
  double chi_1 = atan2(sin_chi_1, cos_chi_1);
  double sin_lambda = sin_th * cos_gamma - sin_gamma * cos_th;
  double cos_lambda = cos_th * cos_gamma + sin_th * sin_gamma;
  double cos_eps = sa_over_sp * (cos_i * sin_lambda - sin_i * cos_lambda * cos(leaf) +
                                 cos_psi * sin_gamma) - cos_alpha * sin_gamma;
  double sin_chi_p = cos_eps * eta * mu * beta / Lorentz;
  double cos_chi_p = (1. - pow(mu, 2.0) / (1. + beta * cos_xi));
  double chi_p = atan2(sin_chi_p, cos_chi_p);
  return chi_0 + chi_1 + chi_p;
}

/* The reference's cached 4-point stencil walk in nd <= 5 dimensions, as
 * hot_Num5D_split.pyx:267-481 and hot_Num2D_split.pyx:200-347 run it: the
 * base node of a dimension moves only when the query leaves the central
 * interval, and a query beyond the grid is clamped only by the move that
 * reaches the grid end.  Weights are formed as the reference forms them
 * (products of the numerators, then of the inverse denominators). */
typedef struct {
  size_t BN[5];
  double node[10];
} walk_state;

static void walk_reset(walk_state *st, const double *const *g, int nd) {
  for (int d = 0; d < nd; d++) {
    st->BN[d] = 0;
    st->node[2 * d] = g[d][1];
    st->node[2 * d + 1] = g[d][2];
  }
}

static double walk_eval(const double *const *g, const size_t *n, int nd, const double *table,
                        walk_state *st, const double *vin) {
  double v[5], DIFF[5][4], SPACE[5][4];
  size_t *BN = st->BN;
  for (int i = 0; i < nd; i++) {
    const double *P = g[i];
    v[i] = vin[i];
    if (v[i] < st->node[2 * i] && BN[i] != 0) {
      while (v[i] < P[BN[i] + 1]) {
        if (BN[i] > 0) BN[i] -= 1;
        else if (v[i] <= P[0]) { v[i] = P[0]; break; }
        else break;
      }
      st->node[2 * i] = P[BN[i] + 1];
      st->node[2 * i + 1] = P[BN[i] + 2];
    } else if (v[i] > st->node[2 * i + 1] && BN[i] != n[i] - 4) {
      while (v[i] > P[BN[i] + 2]) {
        if (BN[i] < n[i] - 4) BN[i] += 1;
        else if (v[i] >= P[n[i] - 1]) { v[i] = P[n[i] - 1]; break; }
        else break;
      }
      st->node[2 * i] = P[BN[i] + 1];
      st->node[2 * i + 1] = P[BN[i] + 2];
    }
    const size_t b = BN[i];
    const double x = v[i];
    DIFF[i][0] = x - P[b + 1]; DIFF[i][0] *= x - P[b + 2]; DIFF[i][0] *= x - P[b + 3];
    DIFF[i][1] = x - P[b]; DIFF[i][1] *= x - P[b + 2]; DIFF[i][1] *= x - P[b + 3];
    DIFF[i][2] = x - P[b]; DIFF[i][2] *= x - P[b + 1]; DIFF[i][2] *= x - P[b + 3];
    DIFF[i][3] = x - P[b]; DIFF[i][3] *= x - P[b + 1]; DIFF[i][3] *= x - P[b + 2];
    SPACE[i][0] = 1.0 / (P[b] - P[b + 1]); SPACE[i][0] /= P[b] - P[b + 2]; SPACE[i][0] /= P[b] - P[b + 3];
    SPACE[i][1] = 1.0 / (P[b + 1] - P[b]); SPACE[i][1] /= P[b + 1] - P[b + 2]; SPACE[i][1] /= P[b + 1] - P[b + 3];
    SPACE[i][2] = 1.0 / (P[b + 2] - P[b]); SPACE[i][2] /= P[b + 2] - P[b + 1]; SPACE[i][2] /= P[b + 2] - P[b + 3];
    SPACE[i][3] = 1.0 / (P[b + 3] - P[b]); SPACE[i][3] /= P[b + 3] - P[b + 1]; SPACE[i][3] /= P[b + 3] - P[b + 2];
  }
  size_t stride[5];
  stride[nd - 1] = 1;
  for (int d = nd - 2; d >= 0; d--) stride[d] = stride[d + 1] * n[d + 1];
  double I = 0.0;
  const size_t total = (size_t)1 << (2 * nd);
  for (size_t c = 0; c < total; c++) {
    size_t idx[5], rem = c, off = 0;
    for (int d = nd - 1; d >= 0; d--) { idx[d] = rem & 3; rem >>= 2; }
    double dp = 1.0, sp = 1.0;
    for (int d = 0; d < nd; d++) {
      dp *= DIFF[d][idx[d]];
      sp *= SPACE[d][idx[d]];
      off += (BN[d] + idx[d]) * stride[d];
    }
    double temp = dp;
    temp *= sp;
    I += temp * table[off];
  }
  return I;
}

/* ================================================================== */
/* cell-mesh integrator, azimuthal invariance                         */
/* ================================================================== */
int xo_integrate(int n_threads, double R, double omega, double r_s,
                 double inclination, size_t S0, size_t S1,
                 const double *cellArea, const double *radius_arr,
                 const double *u_arr, const double *theta, const double *phi,
                 const double *srcCellParams, size_t n_params,
                 const int *radiates, const double *correction,
                 size_t n_correction, size_t N_R, const double *deflection,
                 const double *cos_alpha, const double *lag,
                 const double *maxDeflection, const double *cos_gammaArray,
                 size_t N_E, const double *energies, size_t N_L,
                 const double *leaves, size_t N_P, const double *phases,
                 int atm_ext, const xo_atmos4d *atmos, int image_order_limit,
                 double *flux, double *flux_Q, double *flux_U) {
  (void)R;
  /* the elsewhere correction (:257-261, :469-478): a blackbody elsewhere's
   * intensity at correction[i, J] is subtracted from every profile value and
   * every interpolated value is added, negative or not (:593-594) */
  const int perform_correction = correction != NULL;
  /* Stokes Q and U (integratorIQU_for_azimuthal_invariance.pyx:68-743) when
   * flux_Q and flux_U are given: profiles Q cos 2chi and Q sin 2chi beside I,
   * added wherever I is (:646-650) */
  const int ns = (flux_Q != NULL && flux_U != NULL) ? 3 : 1;
  const double sin_i = sin(inclination), cos_i = cos(inclination);
  const size_t leaf_lim = (N_L % 2 == 0) ? N_L / 2 : (N_L + 1) / 2;
  /* hot_Num4D.pyx:441-461, hot_Num2D.pyx:359-367 (atm_ext 4),
   * hot_Num5D_split.pyx:538-563 (atm_ext 6: the split atmosphere reduced to
   * (mu, E) by xo_integrate_split), hot_BB.pyx:84-98 */
  const double norm =
      (atm_ext == 2 || atm_ext == 4 || atm_ext == 6) ? kErg / kHKeV : kErg * kPlanck;
  int nt = n_threads > 0 ? n_threads : 1;
  int terminate_any = 0;
  double *priv = (double *)calloc((size_t)nt * ns * N_E * N_P, sizeof(double));
  /* integrator_for_azimuthal_invariance.pyx:213-226 */
  double *cos_defl = (double *)malloc(S0 * N_R * sizeof(double));
  double *ca_alt = (double *)malloc(S0 * N_R * sizeof(double));
  for (size_t i = 0; i < S0; i++)
    for (size_t j = 0; j < N_R; j++) {
      cos_defl[i * N_R + j] = cos(deflection[i * N_R + N_R - j - 1]);
      ca_alt[i * N_R + j] = cos_alpha[i * N_R + N_R - j - 1];
    }
  gsl_error_handler_t *prev = gsl_set_error_handler_off();

#pragma omp parallel num_threads(nt) reduction(| : terminate_any)
  {
    int T = 0;
#ifdef _OPENMP
    T = omp_get_thread_num();
#endif
    double *pflux = priv + (size_t)T * ns * N_E * N_P;
    gsl_interp_accel *acc_a = gsl_interp_accel_alloc(), *acc_alt = gsl_interp_accel_alloc();
    gsl_interp_accel *acc_l = gsl_interp_accel_alloc(), *acc_p = gsl_interp_accel_alloc();
    gsl_interp_accel *acc_q = gsl_interp_accel_alloc(), *acc_u = gsl_interp_accel_alloc();
    gsl_interp *ia = gsl_interp_alloc(gsl_interp_steffen, N_R);
    gsl_interp *il = gsl_interp_alloc(gsl_interp_steffen, N_R);
    gsl_interp *ip = gsl_interp_alloc(gsl_interp_akima_periodic, N_L);
    gsl_interp *iq = gsl_interp_alloc(gsl_interp_akima_periodic, N_L);
    gsl_interp *iu = gsl_interp_alloc(gsl_interp_akima_periodic, N_L);
    double *PHASE = (double *)malloc(N_L * sizeof(double));
    /* ns blocks of [N_E][N_L]: I, then Q and U */
    double *PROFILE = (double *)malloc((size_t)ns * N_E * N_L * sizeof(double));
    const size_t NR = (size_t)ns * N_E;
    num4d_state nst;
    if (atm_ext == 2) num4d_reset(&nst, atmos);
    /* the 2-D tables' evaluators, I and Q each with its own cached walk
     * (hot_Num2D.pyx:56-146, hot_Num2D_split.pyx; one per thread) */
    walk_state wst, wstq;
    const double *g2[2] = {atmos ? atmos->mu : NULL, atmos ? atmos->logE : NULL};
    const size_t n2[2] = {atmos ? atmos->nmu : 0, atmos ? atmos->nE : 0};
    if (atm_ext == 4 || atm_ext == 6) {
      walk_reset(&wst, g2, 2);
      walk_reset(&wstq, g2, 2);
    }
    int terminate = 0;
#pragma omp for schedule(static, 1)
    for (long ii = 0; ii < (long)S0; ii++) {
      size_t i = (size_t)ii, J = 0, j;
      if (terminate) continue;
      for (j = 0; j < S1; j++)
        if (radiates[i * S1 + j] == 1) { J = j; break; }
      if (j == S1) continue;
      const double *defl = deflection + i * N_R;
      gsl_interp_accel_reset(acc_a);
      gsl_interp_accel_reset(acc_l);
      j = 0;
      while (defl[j] <= kHalfPi) j++;
      const double *xalt = cos_defl + i * N_R + (N_R - j - 1);
      const double *yalt = ca_alt + i * N_R + (N_R - j - 1);
      gsl_interp *ialt = gsl_interp_alloc(gsl_interp_steffen, j + 1);
      gsl_interp_init(ialt, xalt, yalt, j + 1);
      gsl_interp_accel_reset(acc_alt);
      gsl_interp_init(ia, defl, cos_alpha + i * N_R, N_R);
      gsl_interp_init(il, defl, lag + i * N_R, N_R);
      const double *ya = cos_alpha + i * N_R, *yl = lag + i * N_R;

      double radius = radius_arr[i];
      double Grav_z = sqrt(1.0 - u_arr[i]);
      double cos_gamma = cos_gammaArray[i];
      double sin_gamma = sqrt(1.0 - cos_gamma * cos_gamma);
      double cos_th = cos(theta[i * S1]), sin_th = sin(theta[i * S1]);
      double th_over_pi = theta[i * S1] / kPi;
      double beta = radius * omega * sin_th / (kC * Grav_z);
      double Lorentz = sqrt(1.0 - beta * beta);
      double cos_a = -1.0, deriv = -1.0;
      int IO = image_order_limit > 0 ? image_order_limit
                                     : (int)ceil(maxDeflection[i] / kPi);
      const double *VEC = srcCellParams + (i * S1 + J) * n_params;
      for (int I = 0; I < IO; I++) {
        int InvisFlag = 2, CalcRays = 0;
        size_t InvisPhase = 0;
        double InvisStep;
        for (size_t k = 0; k < leaf_lim; k++) {
          double cos_psi = cos_i * cos_th + sin_i * sin_th * cos(leaves[k]);
          double psi = image_deflection(I, acos(cos_psi));
          double sin_psi = sin(psi);
          if (!are_equal(psi, 0.0) && are_equal(sin_psi, 0.0)) {
            double _i = (cos_i >= 0.0) ? inclination + inclination * 1.0e-6
                                       : inclination - inclination * 1.0e-6;
            cos_psi = cos(_i) * cos_th + sin(_i) * sin_th * cos(leaves[k]);
            psi = image_deflection(I, acos(cos_psi));
            sin_psi = sin(psi);
          }
          double sin_alpha = 0.0, mu = 0.0;
          if (psi <= maxDeflection[i]) {
            if (psi < ia->xmin || psi > ia->xmax) { terminate = 1; break; }
            if (psi <= kHalfPi && cos_psi >= ialt->xmin)
              cos_a = gsl_interp_eval(ialt, xalt, yalt, cos_psi, acc_alt);
            else
              cos_a = gsl_interp_eval(ia, defl, ya, psi, acc_a);
            sin_alpha = sqrt(1.0 - cos_a * cos_a);
            mu = cos_a * cos_gamma;
            if (!are_equal(psi, 0.0)) {
              double cos_delta = (cos_i - cos_th * cos_psi) / (sin_th * sin_psi);
              if (th_over_pi < 0.5) mu = mu + sin_alpha * sin_gamma * cos_delta;
              else mu = mu - sin_alpha * sin_gamma * cos_delta;
            }
            CalcRays = (mu > 0.0) ? 1 : 0; /* R_in = 1e6: no disk */
          } else {
            CalcRays = 0;
          }
          if (CalcRays == 1) {
            if (psi <= kHalfPi && cos_psi >= ialt->xmin) {
              deriv = gsl_interp_eval_deriv(ialt, xalt, yalt, cos_psi, acc_alt);
            } else {
              deriv = gsl_interp_eval_deriv(ia, defl, ya, psi, acc_a);
              deriv = exp(log(fabs(deriv)) - log(fabs(sin_psi)));
            }
            if (psi < il->xmin || psi > il->xmax) { terminate = 1; break; }
            double plag = gsl_interp_eval(il, defl, yl, psi, acc_l);
            for (int ks = 0; ks < 2; ks++) {
              if ((0 < k && k < leaf_lim - 1) || (k == 0 && ks == 0) ||
                  (k == leaf_lim - 1 && N_L % 2 == 1 && ks == 0) ||
                  (k == leaf_lim - 1 && N_L % 2 == 0)) {
                size_t kdx = (ks == 0) ? k : N_L - 1 - k;
                double superlum, eta;
                if (!are_equal(psi, 0.0)) {
                  double cos_xi = sin_alpha * sin_i * sin(leaves[kdx]) / sin_psi;
                  superlum = 1.0 + beta * cos_xi;
                  eta = Lorentz / superlum;
                } else {
                  superlum = 1.0;
                  eta = Lorentz;
                }
                double Z = eta * Grav_z;
                double ABB = mu * eta;
                double GEOM = mu * fabs(deriv) * Grav_z * eta * eta * eta / superlum;
                PHASE[kdx] = leaves[kdx] + plag;
                double c2chi = 0.0, s2chi = 0.0;
                if (ns == 3) {
                  double cos_xi = are_equal(psi, 0.0) ? 0.0
                                                      : sin_alpha * sin_i * sin(leaves[kdx]) / sin_psi;
                  double chi = pol_angle(leaves[kdx], sin_psi, cos_psi, sin_alpha, cos_a, sin_th,
                                         cos_th, sin_i, cos_i, sin_gamma, cos_gamma, Grav_z, mu,
                                         eta, beta, Lorentz, cos_xi);
                  c2chi = cos(2 * chi);
                  s2chi = sin(2 * chi);
                }
                for (size_t p = 0; p < N_E; p++) {
                  double Ep = energies[p] / Z;
                  double I_E, Q_E = 0.0;
                  if (atm_ext == 2) {
                    I_E = eval_num4d(atmos, &nst, Ep, ABB, VEC);
                  } else if (atm_ext == 4 || atm_ext == 6) {
                    /* Pol_Num2D at (mu, log10 E') (hot_Num2D.pyx:187-232,
                     * 369-400), or the reduced split table at E' in electron
                     * rest energies (integrator_for_azimuthal_invariance_split.pyx:457-460,
                     * integratorIQU_for_azimuthal_invariance_split.pyx:515-520);
                     * I clipped at 0, Q not */
                    double q[2] = {ABB, atm_ext == 4 ? log10(Ep) : Ep * 0.001956951};
                    I_E = walk_eval(g2, n2, 2, atmos->I, &wst, q);
                    if (I_E < 0.0) I_E = 0.0;
                    if (ns == 3 && atmos->Q) Q_E = walk_eval(g2, n2, 2, atmos->Q, &wstq, q);
                  } else if (atm_ext == 3) { /* hot_BB_burst.pyx: I and Q */
                    I_E = eval_bb(Ep, VEC) * (0.421 + 0.868 * ABB);
                    Q_E = (0.1171 * (ABB - 1.) / (1. + 3.582 * ABB)) * I_E;
                  } else {
                    I_E = eval_bb(Ep, VEC);
                  }
                  double corr = 0.0;
                  if (perform_correction)
                    corr = eval_bb(Ep, correction + (i * S1 + J) * n_correction) *
                           (kErg * kPlanck);
                  PROFILE[p * N_L + kdx] = (I_E * norm - corr) * GEOM;
                  if (ns == 3) {
                    PROFILE[(N_E + p) * N_L + kdx] = ((Q_E * c2chi) * norm) * GEOM;
                    PROFILE[(2 * N_E + p) * N_L + kdx] = ((Q_E * s2chi) * norm) * GEOM;
                  }
                }
              }
            }
            if (k == 0) {
              PHASE[N_L - 1] = PHASE[0] + kTwoPi;
              for (size_t p = 0; p < NR; p++) PROFILE[p * N_L + N_L - 1] = PROFILE[p * N_L];
            } else if (k > 0 && InvisFlag == 2) {
              InvisStep = leaves[k] / (double)k;
              for (size_t m = N_L - k; m < N_L; m++) PHASE[m] = PHASE[m - 1] + InvisStep;
              for (size_t p = 0; p < NR; p++)
                for (size_t m = N_L - k; m < N_L; m++) PROFILE[p * N_L + m] = 0.0;
              PHASE[0] = PHASE[N_L - 1] - kTwoPi;
              for (size_t m = 1; m < k; m++) PHASE[m] = PHASE[m - 1] + InvisStep;
              for (size_t p = 0; p < NR; p++) {
                PROFILE[p * N_L] = 0.0;
                for (size_t m = 1; m < k; m++) PROFILE[p * N_L + m] = 0.0;
              }
            } else if (InvisFlag == 1) {
              InvisStep = PHASE[k] - PHASE[InvisPhase - 1];
              InvisStep = InvisStep / (double)(k - InvisPhase + 1);
              for (size_t m = InvisPhase; m < k; m++) PHASE[m] = PHASE[m - 1] + InvisStep;
              InvisStep = PHASE[N_L - InvisPhase] - PHASE[N_L - 1 - k];
              InvisStep = InvisStep / (double)(k - InvisPhase + 1);
              for (size_t m = N_L - k; m < N_L - InvisPhase; m++) PHASE[m] = PHASE[m - 1] + InvisStep;
            }
            InvisFlag = 0;
          } else {
            if (InvisFlag == 0) {
              InvisStep = PHASE[N_L - k] - PHASE[k - 1];
              InvisStep = InvisStep / (double)(N_L - 2 * k + 1);
              for (size_t m = k; m < N_L - k; m++) PHASE[m] = PHASE[m - 1] + InvisStep;
              for (size_t p = 0; p < NR; p++)
                for (size_t m = k; m < N_L - k; m++) PROFILE[p * N_L + m] = 0.0;
              InvisFlag = 1;
              InvisPhase = k;
            }
          }
        }
        if (terminate) break;
        if (InvisFlag == 2) break;
        for (size_t m = 1; m < N_L; m++)
          if (PHASE[m] <= PHASE[m - 1]) { terminate = 1; break; }
        if (terminate) break;
        for (size_t p = 0; p < N_E && !terminate; p++) {
          const double *prof = PROFILE + p * N_L;
          const double *profq = PROFILE + (N_E + p) * N_L, *profu = PROFILE + (2 * N_E + p) * N_L;
          gsl_interp_accel_reset(acc_p);
          gsl_interp_init(ip, PHASE, prof, N_L);
          if (ns == 3) {
            gsl_interp_accel_reset(acc_q);
            gsl_interp_init(iq, PHASE, profq, N_L);
            gsl_interp_accel_reset(acc_u);
            gsl_interp_init(iu, PHASE, profu, N_L);
          }
          for (j = 0; j < S1 && !terminate; j++) {
            if (radiates[i * S1 + j] != 1) continue;
            double shift = phi[i * S1 + j];
            double A = cellArea[i * S1 + j];
            for (size_t k = 0; k < N_P; k++) {
              double x = phases[k] + shift;
              if (x > PHASE[N_L - 1]) {
                while (x > PHASE[N_L - 1]) x = x - kTwoPi;
              } else if (x < PHASE[0]) {
                while (x < PHASE[0]) x = x + kTwoPi;
              }
              if (x < ip->xmin || x > ip->xmax) { terminate = 1; break; }
              double s = gsl_interp_eval(ip, PHASE, prof, x, acc_p);
              if (s > 0.0 || perform_correction) {
                pflux[p * N_P + k] += A * s;
                if (ns == 3) {
                  pflux[(N_E + p) * N_P + k] += A * gsl_interp_eval(iq, PHASE, profq, x, acc_q);
                  pflux[(2 * N_E + p) * N_P + k] += A * gsl_interp_eval(iu, PHASE, profu, x, acc_u);
                }
              }
            }
          }
        }
        if (terminate) break;
      }
      gsl_interp_free(ialt);
    }
    if (terminate) terminate_any = 1;
    gsl_interp_free(ia); gsl_interp_free(il); gsl_interp_free(ip);
    gsl_interp_free(iq); gsl_interp_free(iu);
    gsl_interp_accel_free(acc_a); gsl_interp_accel_free(acc_alt);
    gsl_interp_accel_free(acc_l); gsl_interp_accel_free(acc_p);
    gsl_interp_accel_free(acc_q); gsl_interp_accel_free(acc_u);
    free(PHASE); free(PROFILE);
  }
  gsl_set_error_handler(prev);
  /* :605-612 (IQU: :715-725) */
  double *outs[3] = {flux, flux_Q, flux_U};
  for (int c = 0; c < ns; c++)
    for (size_t p = 0; p < N_E; p++)
      for (size_t k = 0; k < N_P; k++) {
        double s = 0.0;
        for (int T = 0; T < nt; T++)
          s += priv[(size_t)T * ns * N_E * N_P + ((size_t)c * N_E + p) * N_P + k];
        outs[c][p * N_P + k] = s / (energies[p] * kKeV);
      }
  free(priv); free(cos_defl); free(ca_alt);
  return terminate_any ? 1 : 0;
}

/* ================================================================== */
/* split integrator: cellmesh/integrator_for_azimuthal_invariance_split.pyx */
/* the 5-D split atmosphere (t_e, t_bb, tau, mu, E) is reduced once to  */
/* (mu, E) at the first cell's parameters (hot_Num5D_split.pyx:566-640, */
/* produce_2D_data and make_atmosphere_2D), then integrated as above    */
/* ================================================================== */
typedef struct {
  const double *grid[5];
  size_t n[5];
  const double *I;
} xo_atmos5d;

static double *split_reduce(const xo_atmos5d *atm5, const double *vec) {
  const size_t nmu = atm5->n[3], nE = atm5->n[4];
  double *I2 = (double *)malloc(nmu * nE * sizeof(double));
  walk_state st;
  walk_reset(&st, atm5->grid, 5);
  for (size_t i = 0; i < nmu; i++)
    for (size_t j = 0; j < nE; j++) {
      const double v[5] = {vec[0], vec[1], vec[2], atm5->grid[3][i], atm5->grid[4][j]};
      I2[i * nE + j] = walk_eval(atm5->grid, atm5->n, 5, atm5->I, &st, v);
    }
  return I2;
}

int xo_integrate_split(int n_threads, double R, double omega, double r_s,
                       double inclination, size_t S0, size_t S1,
                       const double *cellArea, const double *radius_arr,
                       const double *u_arr, const double *theta, const double *phi,
                       const double *srcCellParams, size_t n_params,
                       const int *radiates, const double *correction,
                       size_t n_correction, size_t N_R, const double *deflection,
                       const double *cos_alpha, const double *lag,
                       const double *maxDeflection, const double *cos_gammaArray,
                       size_t N_E, const double *energies, size_t N_L,
                       const double *leaves, size_t N_P, const double *phases,
                       const xo_atmos5d *atm5, int image_order_limit, double *flux) {
  double *I2 = split_reduce(atm5, srcCellParams);
  xo_atmos4d a2 = {NULL, NULL, atm5->grid[3], atm5->grid[4], I2, 0, 0, atm5->n[3],
                   atm5->n[4], NULL};
  int rc = xo_integrate(n_threads, R, omega, r_s, inclination, S0, S1, cellArea, radius_arr,
                        u_arr, theta, phi, srcCellParams, n_params, radiates, correction,
                        n_correction, N_R, deflection, cos_alpha, lag, maxDeflection,
                        cos_gammaArray, N_E, energies, N_L, leaves, N_P, phases, 6, &a2,
                        image_order_limit, flux, NULL, NULL);
  free(I2);
  return rc;
}

/* integratorIQU_for_azimuthal_invariance_split.pyx:75-758: the I and Q
 * split tables each reduced to (mu, E) at the first cell's vector by its own
 * fresh evaluator (:310-322), then I, Q cos 2chi, Q sin 2chi per leaf and
 * energy (:515-530) */
int xo_integrate_split_iqu(int n_threads, double R, double omega, double r_s,
                           double inclination, size_t S0, size_t S1,
                           const double *cellArea, const double *radius_arr,
                           const double *u_arr, const double *theta, const double *phi,
                           const double *srcCellParams, size_t n_params,
                           const int *radiates, const double *correction,
                           size_t n_correction, size_t N_R, const double *deflection,
                           const double *cos_alpha, const double *lag,
                           const double *maxDeflection, const double *cos_gammaArray,
                           size_t N_E, const double *energies, size_t N_L,
                           const double *leaves, size_t N_P, const double *phases,
                           const xo_atmos5d *atm5_I, const xo_atmos5d *atm5_Q,
                           int image_order_limit, double *flux, double *flux_Q,
                           double *flux_U) {
  for (int d = 3; d < 5; d++) {
    if (atm5_I->n[d] != atm5_Q->n[d]) return -1;
    for (size_t k = 0; k < atm5_I->n[d]; k++)
      if (atm5_I->grid[d][k] != atm5_Q->grid[d][k]) return -1;
  }
  double *I2 = split_reduce(atm5_I, srcCellParams);
  double *Q2 = split_reduce(atm5_Q, srcCellParams);
  xo_atmos4d a2 = {NULL, NULL, atm5_I->grid[3], atm5_I->grid[4], I2, 0, 0,
                   atm5_I->n[3], atm5_I->n[4], Q2};
  int rc = xo_integrate(n_threads, R, omega, r_s, inclination, S0, S1, cellArea, radius_arr,
                        u_arr, theta, phi, srcCellParams, n_params, radiates, correction,
                        n_correction, N_R, deflection, cos_alpha, lag, maxDeflection,
                        cos_gammaArray, N_E, energies, N_L, leaves, N_P, phases, 6, &a2,
                        image_order_limit, flux, flux_Q, flux_U);
  free(I2);
  free(Q2);
  return rc;
}

/* ================================================================== */
/* general integrator (HotRegion symmetry=False):                     */
/* cellmesh/integrator.pyx:48-667                                     */
/* per cell: the leaf profiles of Z, mu eta and the geometric factor  */
/* are splined in phase (Steffen, Steffen, Akima periodic) and the    */
/* atmosphere is evaluated at every (cell, phase, energy)             */
/* ================================================================== */
int xo_integrate_general(int n_threads, double R, double omega, double r_s,
                         double inclination, size_t S0, size_t S1,
                         const double *cellArea, const double *radius_arr,
                         const double *u_arr, const double *theta,
                         const double *phi, const double *srcCellParams,
                         size_t n_params, const int *radiates,
                         const double *correction, size_t n_correction,
                         size_t N_R, const double *deflection,
                         const double *cos_alpha, const double *lag,
                         const double *maxDeflection,
                         const double *cos_gammaArray, size_t N_E,
                         const double *energies, size_t N_L,
                         const double *leaves, size_t N_P, const double *phases,
                         int atm_ext, const xo_atmos4d *atmos,
                         int image_order_limit, double *flux, double *flux_Q,
                         double *flux_U) {
  (void)R;
  (void)r_s;
  const double sin_i = sin(inclination), cos_i = cos(inclination);
  const size_t leaf_lim = (N_L % 2 == 0) ? N_L / 2 : (N_L + 1) / 2;
  /* hot_Num4D.pyx:441-461, hot_Num2D.pyx:359-367, hot_BB(_burst).pyx */
  const double norm = (atm_ext == 2 || atm_ext == 4) ? kErg / kHKeV : kErg * kPlanck;
  const int perform_correction = correction != NULL;
  /* Stokes Q and U (integratorIQU.pyx:76-717) when flux_Q and flux_U are
   * given */
  const int ns = (flux_Q != NULL && flux_U != NULL) ? 3 : 1;
  int nt = n_threads > 0 ? n_threads : 1;
  int terminate_any = 0;
  double *priv = (double *)calloc((size_t)nt * ns * N_P * N_E, sizeof(double));
  /* :255-270 */
  double *cos_defl = (double *)malloc(S0 * N_R * sizeof(double));
  double *ca_alt = (double *)malloc(S0 * N_R * sizeof(double));
  for (size_t i = 0; i < S0; i++)
    for (size_t j = 0; j < N_R; j++) {
      cos_defl[i * N_R + j] = cos(deflection[i * N_R + N_R - j - 1]);
      ca_alt[i * N_R + j] = cos_alpha[i * N_R + N_R - j - 1];
    }
  gsl_error_handler_t *prev = gsl_set_error_handler_off();

#pragma omp parallel num_threads(nt) reduction(| : terminate_any)
  {
    int T = 0;
#ifdef _OPENMP
    T = omp_get_thread_num();
#endif
    double *pflux = priv + (size_t)T * ns * N_P * N_E; /* ns x [N_P][N_E] as :120 */
    gsl_interp_accel *acc_a = gsl_interp_accel_alloc(), *acc_alt = gsl_interp_accel_alloc();
    gsl_interp_accel *acc_l = gsl_interp_accel_alloc();
    gsl_interp_accel *acc_g = gsl_interp_accel_alloc(), *acc_z = gsl_interp_accel_alloc();
    gsl_interp_accel *acc_b = gsl_interp_accel_alloc();
    gsl_interp *ia = gsl_interp_alloc(gsl_interp_steffen, N_R);
    gsl_interp *il = gsl_interp_alloc(gsl_interp_steffen, N_R);
    gsl_interp *iz = gsl_interp_alloc(gsl_interp_steffen, N_L);
    gsl_interp *ib = gsl_interp_alloc(gsl_interp_steffen, N_L);
    gsl_interp *ig = gsl_interp_alloc(gsl_interp_akima_periodic, N_L);
    double *PH = (double *)malloc(N_L * sizeof(double));
    double *ZZ = (double *)malloc(N_L * sizeof(double));
    double *AB = (double *)malloc(N_L * sizeof(double));
    double *GE = (double *)malloc(N_L * sizeof(double));
    num4d_state nst;
    if (atm_ext == 2) num4d_reset(&nst, atmos);
    /* Pol_Num2D's I and Q evaluators (hot_Num2D.pyx:56-146), one per thread */
    walk_state wst, wstq;
    const double *g2[2] = {atmos ? atmos->mu : NULL, atmos ? atmos->logE : NULL};
    const size_t n2[2] = {atmos ? atmos->nmu : 0, atmos ? atmos->nE : 0};
    if (atm_ext == 4) {
      walk_reset(&wst, g2, 2);
      walk_reset(&wstq, g2, 2);
    }
    /* the polarisation angle's inputs as the reference leaves them after a
     * leaf loop (integratorIQU.pyx:593-596 reads the loop's last values:
     * cos psi and sin psi of the last leaf, cos alpha, sin alpha and mu of
     * the last leaf within the maximum deflection, eta, cos xi and the leaf
     * index of the last (leaf, mirror) assignment); thread-private and
     * carried from parallel to parallel as Cython's first/lastprivate
     * variables are */
    double x_cpsi = NAN, x_spsi = NAN, x_ca = NAN, x_sa = NAN, x_mu = NAN, x_eta = NAN,
           x_cxi = NAN;
    size_t x_kdx = 0;
    int terminate = 0;
#pragma omp for schedule(static, 1)
    for (long ii = 0; ii < (long)S0; ii++) {
      size_t i = (size_t)ii, j;
      if (terminate) continue;
      for (j = 0; j < S1; j++)
        if (radiates[i * S1 + j] == 1) break;
      if (j == S1) continue;
      const double *defl = deflection + i * N_R;
      gsl_interp_accel_reset(acc_a);
      gsl_interp_accel_reset(acc_l);
      j = 0;
      while (defl[j] <= kHalfPi) j++;
      const double *xalt = cos_defl + i * N_R + (N_R - j - 1);
      const double *yalt = ca_alt + i * N_R + (N_R - j - 1);
      gsl_interp *ialt = gsl_interp_alloc(gsl_interp_steffen, j + 1);
      gsl_interp_init(ialt, xalt, yalt, j + 1);
      gsl_interp_accel_reset(acc_alt);
      gsl_interp_init(ia, defl, cos_alpha + i * N_R, N_R);
      gsl_interp_init(il, defl, lag + i * N_R, N_R);
      const double *ya = cos_alpha + i * N_R, *yl = lag + i * N_R;

      double radius = radius_arr[i];
      double Grav_z = sqrt(1.0 - u_arr[i]);
      double cos_gamma = cos_gammaArray[i];
      double sin_gamma = sqrt(1.0 - cos_gamma * cos_gamma);
      double cos_th = cos(theta[i * S1]), sin_th = sin(theta[i * S1]);
      double th_over_pi = theta[i * S1] / kPi;
      double beta = radius * omega * sin_th / (kC * Grav_z);
      double Lorentz = sqrt(1.0 - beta * beta);
      double cos_a = -1.0, deriv = -1.0;
      x_ca = -1.0; /* :326 */
      int IO = image_order_limit > 0 ? image_order_limit
                                     : (int)ceil(maxDeflection[i] / kPi);
      for (int I = 0; I < IO; I++) {
        int InvisFlag = 2;
        size_t InvisPhase = 0;
        double InvisStep, Zs, As;
        for (size_t k = 0; k < N_L; k++) { /* :321-505 (all leaves) */
          double cos_psi = cos_i * cos_th + sin_i * sin_th * cos(leaves[k]);
          double psi = image_deflection(I, acos(cos_psi));
          double sin_psi = sin(psi);
          if (!are_equal(psi, 0.0) && are_equal(sin_psi, 0.0)) {
            double _i = (cos_i >= 0.0) ? inclination + inclination * 1.0e-6
                                       : inclination - inclination * 1.0e-6;
            cos_psi = cos(_i) * cos_th + sin(_i) * sin_th * cos(leaves[k]);
            psi = image_deflection(I, acos(cos_psi));
            sin_psi = sin(psi);
          }
          int visible = 0;
          double sin_alpha = 0.0, mu = 0.0;
          x_cpsi = cos_psi;
          x_spsi = sin_psi;
          if (psi <= maxDeflection[i]) {
            if (psi < ia->xmin || psi > ia->xmax) { terminate = 1; break; }
            if (psi <= kHalfPi && cos_psi >= ialt->xmin)
              cos_a = gsl_interp_eval(ialt, xalt, yalt, cos_psi, acc_alt);
            else
              cos_a = gsl_interp_eval(ia, defl, ya, psi, acc_a);
            sin_alpha = sqrt(1.0 - cos_a * cos_a);
            mu = cos_a * cos_gamma;
            if (!are_equal(psi, 0.0)) {
              double cos_delta = (cos_i - cos_th * cos_psi) / (sin_th * sin_psi);
              if (th_over_pi < 0.5) mu = mu + sin_alpha * sin_gamma * cos_delta;
              else mu = mu - sin_alpha * sin_gamma * cos_delta;
            }
            visible = mu > 0.0;
            x_ca = cos_a;
            x_sa = sin_alpha;
            x_mu = mu;
          }
          if (visible) {
            if (psi <= kHalfPi && cos_psi >= ialt->xmin) {
              deriv = gsl_interp_eval_deriv(ialt, xalt, yalt, cos_psi, acc_alt);
            } else {
              deriv = gsl_interp_eval_deriv(ia, defl, ya, psi, acc_a);
              deriv = exp(log(fabs(deriv)) - log(fabs(sin_psi)));
            }
            if (psi < il->xmin || psi > il->xmax) { terminate = 1; break; }
            double plag = gsl_interp_eval(il, defl, yl, psi, acc_l);
            for (int ks = 0; ks < 2; ks++) {
              if ((0 < k && k < leaf_lim - 1) || (k == 0 && ks == 0) ||
                  (k == leaf_lim - 1 && N_L % 2 == 1 && ks == 0) ||
                  (k == leaf_lim - 1 && N_L % 2 == 0)) {
                size_t kdx = (ks == 0) ? k : N_L - 1 - k;
                double superlum, eta, cos_xi;
                if (!are_equal(psi, 0.0)) {
                  cos_xi = sin_alpha * sin_i * sin(leaves[kdx]) / sin_psi;
                  superlum = 1.0 + beta * cos_xi;
                  eta = Lorentz / superlum;
                } else {
                  cos_xi = 0.0;
                  superlum = 1.0;
                  eta = Lorentz;
                }
                x_kdx = kdx;
                x_eta = eta;
                x_cxi = cos_xi;
                ZZ[kdx] = eta * Grav_z;
                AB[kdx] = mu * eta;
                GE[kdx] = mu * fabs(deriv) * Grav_z * eta * eta * eta / superlum;
                PH[kdx] = leaves[kdx] + plag;
              }
            }
            if (k == 0) { /* :422-427 */
              PH[N_L - 1] = PH[0] + kTwoPi;
              ZZ[N_L - 1] = ZZ[0];
              AB[N_L - 1] = AB[0];
              GE[N_L - 1] = GE[0];
            } else if (k > 0 && InvisFlag == 2) { /* :428-460 */
              InvisStep = leaves[k] / (double)k;
              Zs = (ZZ[k] - ZZ[N_L - k - 1]) / (2.0 * (double)k);
              As = (AB[k] - AB[N_L - k - 1]) / (2.0 * (double)k);
              for (size_t m = N_L - k; m < N_L; m++) {
                PH[m] = PH[m - 1] + InvisStep;
                ZZ[m] = ZZ[m - 1] + Zs;
                AB[m] = AB[m - 1] + As;
                GE[m] = 0.0;
              }
              PH[0] = PH[N_L - 1] - kTwoPi;
              ZZ[0] = ZZ[N_L - 1];
              AB[0] = AB[N_L - 1];
              GE[0] = GE[N_L - 1];
              for (size_t m = 1; m < k; m++) {
                PH[m] = PH[m - 1] + InvisStep;
                ZZ[m] = ZZ[m - 1] + Zs;
                AB[m] = AB[m - 1] + As;
                GE[m] = 0.0;
              }
            } else if (InvisFlag == 1) { /* :461-488 */
              InvisStep = (PH[k] - PH[InvisPhase - 1]) / (double)(k - InvisPhase + 1);
              Zs = (ZZ[k] - ZZ[InvisPhase - 1]) / (double)(k - InvisPhase + 1);
              As = (AB[k] - AB[InvisPhase - 1]) / (double)(k - InvisPhase + 1);
              for (size_t m = InvisPhase; m < k; m++) {
                PH[m] = PH[m - 1] + InvisStep;
                ZZ[m] = ZZ[m - 1] + Zs;
                AB[m] = AB[m - 1] + As;
              }
              InvisStep = (PH[N_L - InvisPhase] - PH[N_L - 1 - k]) / (double)(k - InvisPhase + 1);
              Zs = (ZZ[N_L - InvisPhase] - ZZ[N_L - 1 - k]) / (double)(k - InvisPhase + 1);
              As = (AB[N_L - InvisPhase] - AB[N_L - 1 - k]) / (double)(k - InvisPhase + 1);
              for (size_t m = N_L - k; m < N_L - InvisPhase; m++) {
                PH[m] = PH[m - 1] + InvisStep;
                ZZ[m] = ZZ[m - 1] + Zs;
                AB[m] = AB[m - 1] + As;
              }
            }
            InvisFlag = 0;
          } else if (InvisFlag == 0) { /* :491-505, :507-525 */
            InvisStep = (PH[N_L - k] - PH[k - 1]) / (double)(N_L - 2 * k + 1);
            Zs = (ZZ[N_L - k] - ZZ[k - 1]) / (double)(N_L - 2 * k + 1);
            As = (AB[N_L - k] - AB[k - 1]) / (double)(N_L - 2 * k + 1);
            for (size_t m = k; m < N_L - k; m++) {
              PH[m] = PH[m - 1] + InvisStep;
              ZZ[m] = ZZ[m - 1] + Zs;
              AB[m] = AB[m - 1] + As;
              GE[m] = 0.0;
            }
            InvisFlag = 1;
            InvisPhase = k;
          }
        }
        if (terminate) break;
        if (InvisFlag == 2) break;
        for (size_t m = 1; m < N_L; m++)
          if (PH[m] <= PH[m - 1]) { terminate = 1; break; }
        if (terminate) break;
        gsl_interp_accel_reset(acc_z);
        gsl_interp_init(iz, PH, ZZ, N_L);
        gsl_interp_accel_reset(acc_b);
        gsl_interp_init(ib, PH, AB, N_L);
        gsl_interp_accel_reset(acc_g);
        gsl_interp_init(ig, PH, GE, N_L);
        double c2chi = 0.0, s2chi = 0.0;
        if (ns == 3) { /* integratorIQU.pyx:593-596, the same for every entry */
          double chi = pol_angle(leaves[x_kdx], x_spsi, x_cpsi, x_sa, x_ca, sin_th, cos_th,
                                 sin_i, cos_i, sin_gamma, cos_gamma, Grav_z, x_mu, x_eta, beta,
                                 Lorentz, x_cxi);
          c2chi = cos(2 * chi);
          s2chi = sin(2 * chi);
        }
        for (j = 0; j < S1 && !terminate; j++) { /* :549-594 */
          if (radiates[i * S1 + j] != 1) continue;
          const double shift = phi[i * S1 + j];
          const double A = cellArea[i * S1 + j];
          const double *VEC = srcCellParams + (i * S1 + j) * n_params;
          for (size_t k = 0; k < N_P; k++) {
            double x = phases[k] + shift;
            if (x > PH[N_L - 1]) {
              while (x > PH[N_L - 1]) x = x - kTwoPi;
            } else if (x < PH[0]) {
              while (x < PH[0]) x = x + kTwoPi;
            }
            if (x < ig->xmin || x > ig->xmax) { terminate = 1; break; }
            double G = gsl_interp_eval(ig, PH, GE, x, acc_g);
            if (G > 0.0) {
              double Z = gsl_interp_eval(iz, PH, ZZ, x, acc_z);
              double ABB = gsl_interp_eval(ib, PH, AB, x, acc_b);
              for (size_t p = 0; p < N_E; p++) {
                double Ep = energies[p] / Z;
                double I_E, Q_E = 0.0;
                if (atm_ext == 2) {
                  I_E = eval_num4d(atmos, &nst, Ep, ABB, VEC);
                } else if (atm_ext == 3) { /* hot_BB_burst.pyx */
                  I_E = eval_bb(Ep, VEC) * (0.421 + 0.868 * ABB);
                  Q_E = (0.1171 * (ABB - 1.) / (1. + 3.582 * ABB)) * I_E;
                } else if (atm_ext == 4) { /* hot_Num2D.pyx:187-400 */
                  double q[2] = {ABB, log10(Ep)};
                  I_E = walk_eval(g2, n2, 2, atmos->I, &wst, q);
                  if (I_E < 0.0) I_E = 0.0;
                  if (ns == 3 && atmos->Q) Q_E = walk_eval(g2, n2, 2, atmos->Q, &wstq, q);
                } else {
                  I_E = eval_bb(Ep, VEC);
                }
                I_E = I_E * norm;
                double corr = 0.0;
                if (perform_correction)
                  corr = eval_bb(Ep, correction + (i * S1 + j) * n_correction) *
                         (kErg * kPlanck);
                pflux[k * N_E + p] += A * (I_E - corr) * G;
                if (ns == 3) { /* integratorIQU.pyx:606-633 */
                  Q_E = Q_E * norm;
                  double Q_obs = Q_E * c2chi, U_obs = Q_E * s2chi;
                  pflux[(N_P + k) * N_E + p] += A * Q_obs * G;
                  pflux[(2 * N_P + k) * N_E + p] += A * U_obs * G;
                }
              }
            }
          }
        }
        if (terminate) break;
      }
      gsl_interp_free(ialt);
    }
    if (terminate) terminate_any = 1;
    gsl_interp_free(ia); gsl_interp_free(il); gsl_interp_free(iz); gsl_interp_free(ib);
    gsl_interp_free(ig);
    gsl_interp_accel_free(acc_a); gsl_interp_accel_free(acc_alt); gsl_interp_accel_free(acc_l);
    gsl_interp_accel_free(acc_g); gsl_interp_accel_free(acc_z); gsl_interp_accel_free(acc_b);
    free(PH); free(ZZ); free(AB); free(GE);
  }
  gsl_set_error_handler(prev);
  /* :603-610 */
  double *outs[3] = {flux, flux_Q, flux_U};
  for (int c = 0; c < ns; c++)
    for (size_t p = 0; p < N_E; p++)
      for (size_t k = 0; k < N_P; k++) {
        double s = 0.0;
        for (int T = 0; T < nt; T++)
          s += priv[(size_t)T * ns * N_P * N_E + ((size_t)c * N_P + k) * N_E + p];
        outs[c][p * N_P + k] = s / (energies[p] * kKeV);
      }
  free(priv); free(cos_defl); free(ca_alt);
  return terminate_any ? 1 : 0;
}

/* ================================================================== */
/* time-invariant integrator (the photosphere elsewhere):             */
/* cellmesh/integrator_for_time_invariance.pyx:59-338                 */
/* flux[N_E]; cellArea is the closed mesh's one cell area             */
/* ================================================================== */
int xo_integrate_time_invariant(int n_threads, double R, double omega,
                                double r_s, double inclination, size_t S,
                                double cellArea, const double *radius_arr,
                                const double *u_arr, const double *theta,
                                const double *phi, const double *srcCellParams,
                                size_t n_params, size_t N_R,
                                const double *deflection,
                                const double *cos_alpha,
                                const double *maxDeflection,
                                const double *cos_gammaArray, size_t N_E,
                                const double *energies, int atm_ext,
                                const xo_atmos4d *atmos, int image_order_limit,
                                double *flux) {
  (void)R;
  (void)r_s;
  const double sin_i = sin(inclination), cos_i = cos(inclination);
  /* elsewhere_wrapper.pyx:84-96 -> hot_BB.pyx:84-98, hot_Num4D.pyx:441-461 */
  const double norm = (atm_ext == 2) ? kErg / kHKeV : kErg * kPlanck;
  int nt = n_threads > 0 ? n_threads : 1;
  int terminate_any = 0;
  double *priv = (double *)calloc((size_t)nt * N_E, sizeof(double));
  /* :151-164 */
  double *cos_defl = (double *)malloc(S * N_R * sizeof(double));
  double *ca_alt = (double *)malloc(S * N_R * sizeof(double));
  for (size_t i = 0; i < S; i++)
    for (size_t j = 0; j < N_R; j++) {
      cos_defl[i * N_R + j] = cos(deflection[i * N_R + N_R - j - 1]);
      ca_alt[i * N_R + j] = cos_alpha[i * N_R + N_R - j - 1];
    }
  gsl_error_handler_t *prev = gsl_set_error_handler_off();

#pragma omp parallel num_threads(nt) reduction(| : terminate_any)
  {
    int T = 0;
#ifdef _OPENMP
    T = omp_get_thread_num();
#endif
    double *pflux = priv + (size_t)T * N_E;
    gsl_interp_accel *acc_a = gsl_interp_accel_alloc(), *acc_alt = gsl_interp_accel_alloc();
    gsl_interp *ia = gsl_interp_alloc(gsl_interp_steffen, N_R);
    num4d_state nst;
    if (atm_ext == 2) num4d_reset(&nst, atmos);
    int terminate = 0;
#pragma omp for schedule(static, 1)
    for (long ii = 0; ii < (long)S; ii++) {
      size_t i = (size_t)ii, j;
      if (terminate) continue;
      const double *defl = deflection + i * N_R;
      const double *ya = cos_alpha + i * N_R;
      gsl_interp_accel_reset(acc_a);
      j = 0;
      while (defl[j] <= kHalfPi) j++;
      const double *xalt = cos_defl + i * N_R + (N_R - j - 1);
      const double *yalt = ca_alt + i * N_R + (N_R - j - 1);
      gsl_interp *ialt = gsl_interp_alloc(gsl_interp_steffen, j + 1);
      gsl_interp_init(ialt, xalt, yalt, j + 1);
      gsl_interp_accel_reset(acc_alt);
      gsl_interp_init(ia, defl, ya, N_R);

      double radius = radius_arr[i];
      double Grav_z = sqrt(1.0 - u_arr[i]);
      double cos_gamma = cos_gammaArray[i];
      double sin_gamma = sqrt(1.0 - cos_gamma * cos_gamma);
      double cos_th = cos(theta[i * S]), sin_th = sin(theta[i * S]);
      double th_over_pi = theta[i * S] / kPi;
      double beta = radius * omega * sin_th / (kC * Grav_z);
      double Lorentz = sqrt(1.0 - beta * beta);
      for (j = 0; j < S && !terminate; j++) {
        double ph = phi[i * S + j];
        double c_psi0 = cos_i * cos_th + sin_i * sin_th * cos(ph);
        double psi0 = acos(c_psi0);
        int IO = image_order_limit > 0 ? image_order_limit
                                       : (int)ceil(maxDeflection[i] / kPi);
        for (int I = 0; I < IO; I++) {
          double cos_psi = c_psi0;
          double psi = image_deflection(I, psi0);
          double sin_psi = sin(psi);
          if (!are_equal(psi, 0.0) && are_equal(sin_psi, 0.0)) { /* :231-244 */
            double _i = (cos_i >= 0.0) ? inclination + inclination * 1.0e-6
                                       : inclination - inclination * 1.0e-6;
            cos_psi = cos(_i) * cos_th + sin(_i) * sin_th * cos(ph);
            psi = image_deflection(I, acos(cos_psi));
            sin_psi = sin(psi);
          }
          if (psi > maxDeflection[i]) break; /* :246-247 */
          if (psi < ia->xmin || psi > ia->xmax) { terminate = 1; break; }
          int use_alt = (psi <= kHalfPi && cos_psi >= ialt->xmin);
          double cos_a = use_alt ? gsl_interp_eval(ialt, xalt, yalt, cos_psi, acc_alt)
                                 : gsl_interp_eval(ia, defl, ya, psi, acc_a);
          double sin_alpha = sqrt(1.0 - cos_a * cos_a);
          double mu = cos_a * cos_gamma;
          if (!are_equal(psi, 0.0)) {
            double cos_delta = (cos_i - cos_th * cos_psi) / (sin_th * sin_psi);
            if (th_over_pi < 0.5) mu = mu + sin_alpha * sin_gamma * cos_delta;
            else mu = mu - sin_alpha * sin_gamma * cos_delta;
          }
          if (!(mu > 0.0)) continue; /* :275 */
          double superlum, eta;
          if (!are_equal(sin_psi, 0.0)) {
            double cos_xi = sin_alpha * sin_i * sin(ph) / sin_psi;
            superlum = 1.0 + beta * cos_xi;
            eta = Lorentz / superlum;
          } else {
            eta = Lorentz;
          }
          double deriv;
          if (use_alt) {
            deriv = gsl_interp_eval_deriv(ialt, xalt, yalt, cos_psi, acc_alt);
          } else {
            deriv = gsl_interp_eval_deriv(ia, defl, ya, psi, acc_a);
            deriv = exp(log(fabs(deriv)) - log(fabs(sin_psi)));
          }
          double Z = eta * Grav_z;
          double ABB = mu * eta;
          double GEOM = mu * fabs(deriv) * Grav_z * eta * eta * eta;
          const double *VEC = srcCellParams + (i * S + j) * n_params;
          for (size_t e = 0; e < N_E; e++) {
            double Ep = energies[e] / Z;
            double I_E = (atm_ext == 2) ? eval_num4d(atmos, &nst, Ep, ABB, VEC)
                                        : eval_bb(Ep, VEC);
            pflux[e] += I_E * GEOM;
          }
        }
      }
      gsl_interp_free(ialt);
    }
    if (terminate) terminate_any = 1;
    gsl_interp_free(ia);
    gsl_interp_accel_free(acc_a); gsl_interp_accel_free(acc_alt);
  }
  gsl_set_error_handler(prev);
  /* :318-323 */
  for (size_t e = 0; e < N_E; e++) {
    double s = 0.0;
    for (int T = 0; T < nt; T++) s += priv[(size_t)T * N_E + e];
    flux[e] = s * (cellArea * norm / (energies[e] * kKeV));
  }
  free(priv); free(cos_defl); free(ca_alt);
  return terminate_any ? 1 : 0;
}

/* ================================================================== */
/* energy integrator: tools/energy_integrator.pyx:27-114              */
/* out[n_edges-1][N_P] (the reference returns binned.T)               */
/* ================================================================== */
void xo_energy_integrator(int n_threads, size_t N_E, size_t N_P,
                          const double *signal, const double *logE,
                          size_t n_edges, const double *logEdges, double *out) {
  const double maxE = logE[N_E - 1];
  memset(out, 0, (n_edges - 1) * N_P * sizeof(double));
#pragma omp parallel num_threads(n_threads > 0 ? n_threads : 1)
  {
    gsl_interp *ip = gsl_interp_alloc(gsl_interp_akima_periodic, N_E);
    gsl_interp_accel *acc = gsl_interp_accel_alloc();
    double *cpy = (double *)malloc(N_E * sizeof(double));
#pragma omp for schedule(static, 1)
    for (long ii = 0; ii < (long)N_P; ii++) {
      size_t i = (size_t)ii;
      for (size_t j = 0; j < N_E; j++) cpy[j] = pow(10.0, logE[j]) * signal[j * N_P + i] * log(10.0);
      gsl_interp_accel_reset(acc);
      gsl_interp_init(ip, logE, cpy, N_E);
      for (size_t j = 0; j + 1 < n_edges; j++) {
        double up = logEdges[j + 1] > maxE ? maxE : logEdges[j + 1];
        out[j * N_P + i] = gsl_interp_eval_integ(ip, logE, cpy, logEdges[j], up, acc);
        if (logEdges[j + 1] > maxE) break;
      }
    }
    free(cpy);
    gsl_interp_accel_free(acc);
    gsl_interp_free(ip);
  }
}

/* ================================================================== */
/* background-marginalised Poisson likelihood                          */
/* ================================================================== */
/* default_background_marginalisation.pyx:38-68 */
void xo_precomputation(size_t K, size_t B, const int *counts, double *out) {
  for (size_t i = 0; i < K; i++) {
    double s = 0.0;
    for (size_t j = 0; j < B; j++) s += gsl_sf_lnfact((unsigned)counts[i * B + j]);
    out[i] = -s;
  }
}

typedef struct {
  size_t n;
  double SCALE, T_exp, A, std;
  const double *data;
  double *star;
} marg_args;

/* :84-138 */
static double marginal_integrand(double B, void *params) {
  marg_args *a = (marg_args *)params;
  double x = 0.0;
  for (size_t j = 0; j < a->n; j++) {
    double c = a->SCALE * (a->star[j] + B);
    if (c > 0.0) x += a->data[j] * log(c) - c;
    else if (are_equal(c, 0.0) && are_equal(a->data[j], 0.0)) {}
    else return 0.0;
  }
  return exp(x - a->A);
}

/* :140-173 */
static double newton_delta(double B, marg_args *a) {
  double x = 0.0, y = 0.0;
  for (size_t j = 0; j < a->n; j++) {
    y += a->data[j] / (a->star[j] + B);
    x += a->data[j] / pow(a->star[j] + B, 2.0);
  }
  y = 2.0 * a->T_exp - 2.0 * y;
  x *= 2.0;
  a->std = sqrt(2.0 / x);
  return -1.0 * y / x;
}

/* :176-447; returns 1 on success, 0 when the integral vanished (LOGLIKE
 * then holds the llzero draw, the caller stops) */
static int channel_marginal(marg_args *a, double precomp_i, double *LOGLIKE,
                            double av_DATA, double av_STAR, double epsabs,
                            double epsrel, double epsilon, double sigmas,
                            double llzero, const double *support,
                            double *mcl_bg, double *mcl_bg_s,
                            gsl_integration_cquad_workspace *w,
                            unsigned *rng_state) {
  double T = a->T_exp, B, lower, upper;
  if (are_equal(av_DATA, 0.0) && are_equal(av_STAR, 0.0)) {
    lower = 0.0;
    if (lower < support[0]) lower = support[0];
    upper = 10.0 / T;
    if (upper > support[1] && support[1] > 0.0) upper = support[1];
    B = 0.0;
    LOGLIKE[0] += log((exp(-1.0 * lower * T) - exp(-1.0 * upper * T)) / T);
  } else {
    double B_min = 0.0;
    B = av_DATA - av_STAR;
    if (B <= B_min) {
      double min_counts = -1.0;
      for (size_t j = 0; j < a->n; j++)
        if (are_equal(a->star[j], 0.0)) { min_counts = -2.0; break; }
      if (are_equal(min_counts, -2.0)) {
        for (size_t j = 0; j < a->n; j++)
          if ((are_equal(min_counts, -2.0) && a->data[j] > 0.0) ||
              (0.0 < a->data[j] && a->data[j] < min_counts))
            min_counts = a->data[j];
      }
      if (!are_equal(min_counts, -1.0)) {
        if (are_equal(min_counts, -2.0)) { B = 0.0; B_min = 0.0; }
        else { B = 0.01 * min_counts / a->SCALE; B_min = 0.1 * B; }
      } else {
        B = B_min;
      }
    }
    double dB = newton_delta(B, a);
    int counter = 0;
    while (fabs(dB) > epsilon * a->std && counter < 2) {
      B += dB;
      if (B < B_min) {
        if (B_min > 0.0) counter += 1;
        else counter = 2;
        B = B_min;
      }
      dB = newton_delta(B, a);
    }
    double std_est = 0.0;
    for (size_t j = 0; j < a->n; j++) std_est += a->data[j] / pow(a->star[j] + B, 2.0);
    if (std_est > 0.0) std_est = sqrt(1.0 / std_est);
    else std_est = 1e90;
    lower = B - sigmas * std_est;
    upper = B + sigmas * std_est;
    if (lower < B_min) lower = B_min;
    double Bi = B;
    if (lower < support[0]) {
      lower = support[0];
      if (upper < support[0] && support[1] > 0.0) { upper = support[1]; Bi = support[0]; }
      else if (upper < support[0]) { upper = support[0] + sigmas * std_est; Bi = support[0]; }
    }
    if (upper > support[1] && support[1] > 0.0) {
      upper = support[1];
      if (lower > support[1]) { lower = support[0]; Bi = support[1]; }
    }
    if (Bi < lower) Bi = lower;
    else if (Bi > upper) Bi = upper;
    a->A = 0.0;
    for (size_t j = 0; j < a->n; j++) {
      double c = a->SCALE * (a->star[j] + Bi);
      if (c > 0.0) a->A += a->data[j] * log(c) - c;
      else if (are_equal(c, 0.0) && are_equal(a->data[j], 0.0)) {}
      else a->A += llzero;
    }
    gsl_function f;
    f.function = marginal_integrand;
    f.params = a;
    double result, abserr;
    size_t nev;
    gsl_integration_cquad(&f, lower, upper, epsabs, epsrel, w, &result, &abserr, &nev);
    if (result > 0.0) {
      LOGLIKE[0] += log(result) + a->A + precomp_i;
    } else {
      *rng_state = *rng_state * 1103515245u + 12345u;
      LOGLIKE[0] = llzero * (0.1 + 0.9 * ((*rng_state >> 8) & 0xffffff) / 16777215.0);
      return 0;
    }
  }
  mcl_bg[0] = B * T;
  if (B < support[0]) B = support[0];
  else if (B > support[1] && support[1] > 0.0) B = support[1];
  mcl_bg_s[0] = B * T;
  for (size_t j = 0; j < a->n; j++) a->star[j] = a->SCALE * (a->star[j] + B);
  return 1;
}

/* compute_expected_counts.pyx:66-197 for one channel */
static void star_rate_channel(size_t B, const double *phase_edges, size_t H,
                              const double *const *components,
                              const size_t *n_phase,
                              const double *const *component_phases,
                              const double *shifts, gsl_interp **ip,
                              gsl_interp_accel **acc, double *STAR,
                              size_t channel, const int *allow_negative) {
  for (size_t p = 0; p < H; p++) {
    size_t np = n_phase[p];
    const double *pulse = components[p] + channel * np;
    if (np > 1) {
      gsl_interp_init(ip[p], component_phases[p], pulse, np);
      for (size_t j = 0; j < B; j++) {
        double pa = phase_edges[j] + shifts[p];
        double pb = phase_edges[j + 1] + shifts[p];
        if (are_equal(pb - pa, 1.0)) { pa = 0.0; pb = 1.0; }
        else { pa -= floor(pa); pb -= floor(pb); }
        double v;
        if (pa < pb) {
          v = gsl_interp_eval_integ(ip[p], component_phases[p], pulse, pa, pb, acc[p]);
          if (v > 0.0 || allow_negative[p] == 1) STAR[j] += v;
        } else {
          v = gsl_interp_eval_integ(ip[p], component_phases[p], pulse, pa, 1.0, acc[p]);
          if (v > 0.0 || allow_negative[p] == 1) STAR[j] += v;
          v = gsl_interp_eval_integ(ip[p], component_phases[p], pulse, 0.0, pb, acc[p]);
          if (v > 0.0 || allow_negative[p] == 1) STAR[j] += v;
        }
      }
    } else {
      STAR[0] = pulse[0];
    }
  }
  for (size_t j = 0; j < B; j++)
    if (STAR[j] < 0.0) STAR[j] = 0.0;
}

/* tools/compute_expected_counts.pyx:200-276: out[K][B] = exposure x (the
 * components' bin-integrated rates, clamped at zero, + background rate) */
void xo_expected_counts(double exposure_time, size_t B, const double *phase_edges,
                        size_t K, size_t H, const double *const *components,
                        const size_t *n_phase, const double *const *component_phases,
                        const double *shifts, const double *background,
                        const int *allow_negative, double *out) {
  gsl_interp **ip = (gsl_interp **)calloc(H, sizeof(gsl_interp *));
  gsl_interp_accel **acc = (gsl_interp_accel **)calloc(H, sizeof(gsl_interp_accel *));
  for (size_t p = 0; p < H; p++) {
    if (n_phase[p] > 1) {
      ip[p] = gsl_interp_alloc(gsl_interp_akima_periodic, n_phase[p]);
      acc[p] = gsl_interp_accel_alloc();
    }
  }
  for (size_t i = 0; i < K; i++) {
    double *STAR = out + i * B;
    for (size_t j = 0; j < B; j++) STAR[j] = 0.0;
    star_rate_channel(B, phase_edges, H, components, n_phase, component_phases, shifts, ip,
                      acc, STAR, i, allow_negative);
    for (size_t j = 0; j < B; j++) {
      STAR[j] += background ? background[i * B + j] : 0.0;
      STAR[j] *= exposure_time;
    }
  }
  for (size_t p = 0; p < H; p++) {
    if (ip[p]) gsl_interp_free(ip[p]);
    if (acc[p]) gsl_interp_accel_free(acc[p]);
  }
  free(ip);
  free(acc);
}

/* tools/phase_integrator.pyx:23-121 */
void xo_phase_integrator(double exposure_time, size_t n_edges, const double *phases,
                         size_t rows, size_t n_phases, const double *signal,
                         const double *signal_phases, double phase_shift, int allow_negative,
                         double *out) {
  gsl_interp *ip = gsl_interp_alloc(gsl_interp_akima_periodic, n_phases);
  gsl_interp_accel *acc = gsl_interp_accel_alloc();
  const size_t B = n_edges - 1;
  for (size_t i = 0; i < rows; i++) {
    gsl_interp_accel_reset(acc);
    const double *y = signal + i * n_phases;
    gsl_interp_init(ip, signal_phases, y, n_phases);
    for (size_t j = 0; j < B; j++) {
      double a = phases[j] + phase_shift, b = phases[j + 1] + phase_shift, v;
      double *o = out + i * B + j;
      *o = 0.0;
      if (b - a == 1.0) { a = 0.0; b = 1.0; }
      else { a -= floor(a); b -= floor(b); }
      if (a < b) {
        v = gsl_interp_eval_integ(ip, signal_phases, y, a, b, acc);
        if (v > 0.0 || allow_negative) *o = v;
      } else {
        v = gsl_interp_eval_integ(ip, signal_phases, y, a, 1.0, acc);
        if (v > 0.0 || allow_negative) *o = v;
        v = gsl_interp_eval_integ(ip, signal_phases, y, 0.0, b, acc);
        if (v > 0.0 || allow_negative) *o += v;
      }
      *o *= exposure_time;
    }
  }
  gsl_interp_free(ip);
  gsl_interp_accel_free(acc);
}

/* default_background_marginalisation.pyx:450-734.  Returns 0 normally,
 * 1 when the slim cut fired, 2 when a channel integral vanished. */
int xo_eval_marginal_likelihood(
    double exposure_time, size_t B, const double *phase_edges, size_t K,
    const double *counts, size_t H, const double *const *components,
    const size_t *n_phase, const double *const *component_phases,
    const double *shifts, const double *precomp, const double *support,
    double epsabs, double epsrel, double epsilon, double sigmas,
    double llzero, const int *allow_negative, double slim,
    const double *background, unsigned rng_seed, double *loglike,
    double *STAR, double *mcl_bg, double *mcl_bg_s) {
  double n = (double)B;
  double SCALE = exposure_time / n;
  double LOGLIKE = 0.0;
  int status = 0;
  unsigned rng = rng_seed;
  gsl_interp **ip = (gsl_interp **)calloc(H, sizeof(gsl_interp *));
  gsl_interp_accel **acc = (gsl_interp_accel **)calloc(H, sizeof(gsl_interp_accel *));
  for (size_t p = 0; p < H; p++) {
    if (n_phase[p] > 1) {
      ip[p] = gsl_interp_alloc(gsl_interp_akima_periodic, n_phase[p]);
      acc[p] = gsl_interp_accel_alloc();
    }
  }
  gsl_integration_cquad_workspace *w = gsl_integration_cquad_workspace_alloc(1000);
  memset(STAR, 0, K * B * sizeof(double));
  memset(mcl_bg, 0, K * sizeof(double));
  memset(mcl_bg_s, 0, K * sizeof(double));
  marg_args a;
  a.n = B;
  a.SCALE = SCALE;
  a.T_exp = exposure_time;
  for (size_t i = 0; i < K; i++) {
    double *row = STAR + i * B;
    star_rate_channel(B, phase_edges, H, components, n_phase, component_phases,
                      shifts, ip, acc, row, i, allow_negative);
    double av_DATA = 0.0, av_STAR = 0.0;
    for (size_t j = 0; j < B; j++) {
      if (background) row[j] += background[i * B + j];
      row[j] *= n;
      av_STAR += row[j];
      av_DATA += counts[i * B + j];
    }
    if (slim >= 0.0) {
      double limit = av_STAR * SCALE - slim * sqrt(av_STAR * SCALE) - av_DATA;
      if (limit > 0.0) {
        rng = rng * 1103515245u + 12345u;
        LOGLIKE = llzero * (0.1 + 0.9 * ((rng >> 8) & 0xffffff) / 16777215.0);
        status = 1;
        break;
      }
    }
    av_STAR /= n;
    av_DATA /= exposure_time;
    a.data = counts + i * B;
    a.star = row;
    int out = channel_marginal(&a, precomp[i], &LOGLIKE, av_DATA, av_STAR, epsabs,
                               epsrel, epsilon, sigmas, llzero, support + 2 * i,
                               mcl_bg + i, mcl_bg_s + i, w, &rng);
    if (out == 0) { status = 2; break; }
  }
  for (size_t p = 0; p < H; p++) {
    if (ip[p]) gsl_interp_free(ip[p]);
    if (acc[p]) gsl_interp_accel_free(acc[p]);
  }
  free(ip); free(acc);
  gsl_integration_cquad_workspace_free(w);
  *loglike = LOGLIKE;
  return status;
}

/* ---- oracle-side exposure of the quadrature subset for tests ---- */
double xo_lnfact(unsigned n) { return gsl_sf_lnfact(n); }

/* ================================================================== */
/* tools/phase_interpolator.pyx:25-95: each signal row's Akima-periodic */
/* interpolant at new_phases + phase_shift (wrapped into [0, 1)), kept   */
/* when positive unless allow_negative; out[rows][n_new]                 */
/* ================================================================== */
void xo_phase_interpolator(size_t n_new, const double *new_phases, size_t n_phases,
                           const double *phases, size_t rows, const double *signal,
                           double phase_shift, int allow_negative, double *out) {
  gsl_interp *ip = gsl_interp_alloc(gsl_interp_akima_periodic, n_phases);
  gsl_interp_accel *acc = gsl_interp_accel_alloc();
  for (size_t i = 0; i < rows; i++) {
    gsl_interp_accel_reset(acc);
    const double *y = signal + i * n_phases;
    gsl_interp_init(ip, phases, y, n_phases);
    for (size_t j = 0; j < n_new; j++) {
      double PHASE = new_phases[j] + phase_shift;
      PHASE -= floor(PHASE);
      const double v = gsl_interp_eval(ip, phases, y, PHASE, acc);
      out[i * n_new + j] = (v > 0.0 || allow_negative) ? v : 0.0;
    }
  }
  gsl_interp_accel_free(acc);
  gsl_interp_free(ip);
}

/* ================================================================== */
/* tools/energy_interpolator.pyx:27-113: each column of signal[N_E][n]  */
/* splined (Steffen) in log10 E, in log10 of the signal when the column */
/* is positive throughout; zero above the last energy;                  */
/* out[n][n_new] (the reference returns its transpose, :125)           */
/* ================================================================== */
void xo_energy_interpolator(size_t N_E, size_t n_cols, const double *signal,
                            const double *energies, size_t n_new, const double *new_energies,
                            double *out) {
  gsl_interp *ip = gsl_interp_alloc(gsl_interp_steffen, N_E);
  gsl_interp_accel *acc = gsl_interp_accel_alloc();
  double *cpy = (double *)malloc(N_E * sizeof(double));
  const double max_energy = energies[N_E - 1];
  for (size_t i = 0; i < n_cols; i++) {
    int mode = 1;
    for (size_t j = 0; j < N_E; j++)
      if (signal[j * n_cols + i] <= 0.0) mode = 0;
    for (size_t j = 0; j < N_E; j++)
      cpy[j] = mode ? log10(signal[j * n_cols + i]) : signal[j * n_cols + i];
    gsl_interp_accel_reset(acc);
    gsl_interp_init(ip, energies, cpy, N_E);
    for (size_t j = 0; j < n_new; j++) {
      double v = 0.0;
      if (!(new_energies[j] > max_energy)) {
        v = gsl_interp_eval(ip, energies, cpy, new_energies[j], acc);
        if (mode) v = pow(10.0, v);
      }
      out[i * n_new + j] = v;
    }
  }
  free(cpy);
  gsl_interp_accel_free(acc);
  gsl_interp_free(ip);
}

/* cellmesh/common_functions.pyx:7-66 (compute_pol_ang), exported for the
 * unit tests that mirror xpsi/tests/test_cellmesh.py */
double xo_pol_angle(double leaf, double sin_psi, double cos_psi, double sin_alpha,
                    double cos_alpha, double sin_th, double cos_th, double sin_i, double cos_i,
                    double sin_gamma, double cos_gamma, double Grav_z, double mu, double eta,
                    double beta, double Lorentz, double cos_xi) {
  return pol_angle(leaf, sin_psi, cos_psi, sin_alpha, cos_alpha, sin_th, cos_th, sin_i, cos_i,
                   sin_gamma, cos_gamma, Grav_z, mu, eta, beta, Lorentz, cos_xi);
}
