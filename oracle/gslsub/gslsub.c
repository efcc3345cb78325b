/*
 * gslsub.c -- the oracle's own implementation of the GSL API subset that the
 * X-PSI likelihood path calls.  TEST INFRASTRUCTURE: only the oracle, the
 * reference build recipe and tests link it.  It is not GSL; every routine is
 * written here from the published method it names.
 *
 *   Steffen, M. 1990, A&A 239, 443      monotone cubic (slopes eq. 11; the
 *                                       "simplest" end slopes of sect. 2.2)
 *   Akima, H. 1970, J. ACM 17, 589      local cubic; periodic end extension;
 *                                       a segment whose two weights vanish is
 *                                       taken as the straight chord
 *   Piessens et al. 1983, QUADPACK      QAG globally adaptive bisection with
 *                                       Gauss-Kronrod 21/61 rules (nodes
 *                                       derived in gen_gk_nodes.py)
 *
 * gsl_integration_cquad (Gonnet 2010) is NOT reproduced: its call sites in
 * X-PSI (mesh areas, mesh_tools.pyx:122-154; background marginal integral,
 * default_background_marginalisation.pyx:416-419) ask for epsrel 1e-8 on
 * smooth or piecewise-smooth integrands; here the same QAG machinery with the
 * 21-point rule is run to epsrel min(epsrel, 1e-13), which converges to the
 * same integral with a smaller error.  Differences from a GSL build are thus
 * bounded by that GSL routine's own quadrature error.  When every interior
 * node sees zero but an endpoint does not (a channel without counts gives a
 * window of width ~1e91 whose integrand decays on a scale 1 / exposure),
 * the window is cut into dyadic pieces toward that endpoint, mirroring how a
 * Clenshaw-Curtis rule, whose nodes include the endpoints, finds the mass.
 */
#include "gslsub.h"

#include <float.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "gk_nodes.h"

/* ------------------------------------------------------------------ */
/* error handling                                                      */
/* ------------------------------------------------------------------ */
static gsl_error_handler_t *g_handler = NULL; /* NULL: report and abort */

static void quiet_handler(const char *r, const char *f, int l, int e) {
  (void)r; (void)f; (void)l; (void)e;
}

gsl_error_handler_t *gsl_set_error_handler(gsl_error_handler_t *h) {
  gsl_error_handler_t *prev = g_handler;
  g_handler = h;
  return prev;
}

gsl_error_handler_t *gsl_set_error_handler_off(void) {
  return gsl_set_error_handler(quiet_handler);
}

void gsl_error(const char *reason, const char *file, int line, int code) {
  if (g_handler) {
    g_handler(reason, file, line, code);
    return;
  }
  fprintf(stderr, "gslsub: %s:%d: ERROR: %s (code %d)\n", file, line, reason,
          code);
  fflush(stderr);
  abort();
}

const char *gsl_strerror(const int code) {
  switch (code) {
    case GSL_SUCCESS: return "success";
    case GSL_EDOM: return "input domain error";
    case GSL_EINVAL: return "invalid argument supplied by user";
    case GSL_EFAILED: return "generic failure";
    case GSL_ENOMEM: return "malloc failed";
    case GSL_EMAXITER: return "exceeded max number of iterations";
    case GSL_EBADTOL: return "user specified an invalid tolerance";
    case GSL_EROUND: return "failed because of roundoff error";
    case GSL_ESING: return "apparent singularity detected";
    default: return "error";
  }
}

#define RAISE(reason, code)                          \
  do {                                               \
    gsl_error(reason, __FILE__, __LINE__, code);     \
    return code;                                     \
  } while (0)

int gsl_isnan(const double x) { return isnan(x) ? 1 : 0; }
int gsl_isinf(const double x) { return isinf(x) ? (x > 0 ? 1 : -1) : 0; }
int gsl_finite(const double x) { return isfinite(x) ? 1 : 0; }

/* ------------------------------------------------------------------ */
/* interval location                                                   */
/* ------------------------------------------------------------------ */
size_t gsl_interp_bsearch(const double xa[], double x, size_t lo, size_t hi) {
  /* largest i in [lo, hi) with xa[i] <= x, assuming xa[lo] <= x */
  while (hi > lo + 1) {
    size_t mid = (lo + hi) / 2;
    if (xa[mid] > x)
      hi = mid;
    else
      lo = mid;
  }
  return lo;
}

gsl_interp_accel *gsl_interp_accel_alloc(void) {
  gsl_interp_accel *a = (gsl_interp_accel *)calloc(1, sizeof(*a));
  return a;
}

size_t gsl_interp_accel_find(gsl_interp_accel *a, const double xa[],
                             size_t size, double x) {
  size_t i = a->cache;
  if (x < xa[i]) {
    a->miss_count++;
    a->cache = gsl_interp_bsearch(xa, x, 0, i);
  } else if (x >= xa[i + 1]) {
    a->miss_count++;
    a->cache = gsl_interp_bsearch(xa, x, i, size - 1);
  } else {
    a->hit_count++;
  }
  return a->cache;
}

int gsl_interp_accel_reset(gsl_interp_accel *a) {
  a->cache = 0;
  a->miss_count = 0;
  a->hit_count = 0;
  return GSL_SUCCESS;
}

void gsl_interp_accel_free(gsl_interp_accel *a) { free(a); }

static size_t locate(const double xa[], size_t size, double x,
                     gsl_interp_accel *a) {
  if (a) return gsl_interp_accel_find(a, xa, size, x);
  return gsl_interp_bsearch(xa, x, 0, size - 1);
}

/* ------------------------------------------------------------------ */
/* shared cubic-piece algebra                                          */
/* piece i: y(x) = y_i + t (k1 + t (k2 + t k3)),  t = x - x_i          */
/* ------------------------------------------------------------------ */
typedef struct {
  double *k1, *k2, *k3; /* size n */
  double *m;            /* size n + 4 (Akima slopes with 2 ghosts per side) */
  size_t n;
} cubic_state;

static void *cubic_alloc(size_t n) {
  cubic_state *s = (cubic_state *)calloc(1, sizeof(*s));
  if (!s) return NULL;
  s->n = n;
  s->k1 = (double *)calloc(n, sizeof(double));
  s->k2 = (double *)calloc(n, sizeof(double));
  s->k3 = (double *)calloc(n, sizeof(double));
  s->m = (double *)calloc(n + 4, sizeof(double));
  if (!s->k1 || !s->k2 || !s->k3 || !s->m) {
    free(s->k1); free(s->k2); free(s->k3); free(s->m); free(s);
    return NULL;
  }
  return s;
}

static void cubic_free(void *v) {
  cubic_state *s = (cubic_state *)v;
  if (!s) return;
  free(s->k1); free(s->k2); free(s->k3); free(s->m); free(s);
}

static int cubic_eval(const void *v, const double xa[], const double ya[],
                      size_t size, double x, size_t i, double *y) {
  const cubic_state *s = (const cubic_state *)v;
  (void)size;
  double t = x - xa[i];
  *y = ya[i] + t * (s->k1[i] + t * (s->k2[i] + t * s->k3[i]));
  return GSL_SUCCESS;
}

static int cubic_deriv(const void *v, const double xa[], const double ya[],
                       size_t size, double x, size_t i, double *d) {
  const cubic_state *s = (const cubic_state *)v;
  (void)ya; (void)size;
  double t = x - xa[i];
  *d = s->k1[i] + t * (2.0 * s->k2[i] + 3.0 * s->k3[i] * t);
  return GSL_SUCCESS;
}

static int cubic_deriv2(const void *v, const double xa[], const double ya[],
                        size_t size, double x, size_t i, double *d2) {
  const cubic_state *s = (const cubic_state *)v;
  (void)ya; (void)size;
  double t = x - xa[i];
  *d2 = 2.0 * s->k2[i] + 6.0 * s->k3[i] * t;
  return GSL_SUCCESS;
}

/* exact integral of piece i over [x_i + u, x_i + w] */
static double piece_integral(double y0, double k1, double k2, double k3,
                             double u, double w) {
  double Fw = w * (y0 + w * (0.5 * k1 + w * (k2 / 3.0 + 0.25 * k3 * w)));
  double Fu = u * (y0 + u * (0.5 * k1 + u * (k2 / 3.0 + 0.25 * k3 * u)));
  return Fw - Fu;
}

static int cubic_integ(const void *v, const double xa[], const double ya[],
                       size_t size, double a, double b, size_t ia, size_t ib,
                       double *result) {
  const cubic_state *s = (const cubic_state *)v;
  (void)size;
  double acc = 0.0;
  for (size_t i = ia; i <= ib; i++) {
    double h = xa[i + 1] - xa[i];
    if (h == 0.0) {
      *result = 0.0;
      return GSL_EINVAL;
    }
    double u = (i == ia) ? a - xa[i] : 0.0;
    double w = (i == ib) ? b - xa[i] : h;
    acc += piece_integral(ya[i], s->k1[i], s->k2[i], s->k3[i], u, w);
  }
  *result = acc;
  return GSL_SUCCESS;
}

/* ---- Steffen (1990) ---- */
static int steffen_init(void *v, const double xa[], const double ya[],
                        size_t n) {
  cubic_state *s = (cubic_state *)v;
  /* node slopes stored temporarily in m[0..n-1] */
  double *yp = s->m;
  double h0 = xa[1] - xa[0];
  yp[0] = (ya[1] - ya[0]) / h0; /* simplest end condition, Steffen 2.2 */
  for (size_t i = 1; i + 1 < n; i++) {
    double hl = xa[i] - xa[i - 1], hr = xa[i + 1] - xa[i];
    double sl = (ya[i] - ya[i - 1]) / hl, sr = (ya[i + 1] - ya[i]) / hr;
    double p = (sl * hr + sr * hl) / (hl + hr);
    double mag = fmin(fabs(sl), fmin(fabs(sr), 0.5 * fabs(p)));
    yp[i] = (copysign(1.0, sl) + copysign(1.0, sr)) * mag;
  }
  double hn = xa[n - 1] - xa[n - 2];
  yp[n - 1] = (ya[n - 1] - ya[n - 2]) / hn;
  for (size_t i = 0; i + 1 < n; i++) {
    double h = xa[i + 1] - xa[i];
    double sl = (ya[i + 1] - ya[i]) / h;
    s->k1[i] = yp[i];
    s->k2[i] = (3.0 * sl - 2.0 * yp[i] - yp[i + 1]) / h;
    s->k3[i] = (yp[i] + yp[i + 1] - 2.0 * sl) / (h * h);
  }
  return GSL_SUCCESS;
}

/* ---- Akima (1970) ---- */
static void akima_segments(cubic_state *s, const double xa[], size_t n) {
  const double *m = s->m + 2; /* m[-2..n] valid */
  for (size_t i = 0; i + 1 < n; i++) {
    long k = (long)i;
    double wl = fabs(m[k + 1] - m[k]) + fabs(m[k - 1] - m[k - 2]);
    if (wl == 0.0) {
      /* both Akima weights vanish: the segment is the chord */
      s->k1[i] = m[k];
      s->k2[i] = 0.0;
      s->k3[i] = 0.0;
      continue;
    }
    double h = xa[i + 1] - xa[i];
    double wr = fabs(m[k + 2] - m[k + 1]) + fabs(m[k] - m[k - 1]);
    double f = fabs(m[k - 1] - m[k - 2]) / wl;
    double tl = (1.0 - f) * m[k - 1] + f * m[k];
    double tr;
    if (wr == 0.0) {
      tr = m[k];
    } else {
      double g = fabs(m[k] - m[k - 1]) / wr;
      tr = (1.0 - g) * m[k] + g * m[k + 1];
    }
    s->k1[i] = tl;
    s->k2[i] = (3.0 * m[k] - 2.0 * tl - tr) / h;
    s->k3[i] = (tl + tr - 2.0 * m[k]) / (h * h);
  }
}

static void akima_chords(cubic_state *s, const double xa[], const double ya[],
                         size_t n) {
  double *m = s->m + 2;
  for (size_t i = 0; i + 1 < n; i++)
    m[i] = (ya[i + 1] - ya[i]) / (xa[i + 1] - xa[i]);
}

static int akima_init(void *v, const double xa[], const double ya[], size_t n) {
  cubic_state *s = (cubic_state *)v;
  double *m = s->m + 2;
  akima_chords(s, xa, ya, n);
  /* Akima's end extension: parabola through the end points */
  m[-2] = 3.0 * m[0] - 2.0 * m[1];
  m[-1] = 2.0 * m[0] - m[1];
  m[n - 1] = 2.0 * m[n - 2] - m[n - 3];
  m[n] = 3.0 * m[n - 2] - 2.0 * m[n - 3];
  akima_segments(s, xa, n);
  return GSL_SUCCESS;
}

static int akima_periodic_init(void *v, const double xa[], const double ya[],
                               size_t n) {
  cubic_state *s = (cubic_state *)v;
  double *m = s->m + 2;
  akima_chords(s, xa, ya, n);
  /* periodic extension: last chords precede the first ones */
  m[-2] = m[n - 3];
  m[-1] = m[n - 2];
  m[n - 1] = m[0];
  m[n] = m[1];
  akima_segments(s, xa, n);
  return GSL_SUCCESS;
}

/* ---- linear ---- */
static void *linear_alloc(size_t n) { (void)n; return malloc(1); }
static void linear_free(void *v) { free(v); }
static int linear_init(void *v, const double xa[], const double ya[], size_t n) {
  (void)v; (void)xa; (void)ya; (void)n;
  return GSL_SUCCESS;
}
static int linear_eval(const void *v, const double xa[], const double ya[],
                       size_t size, double x, size_t i, double *y) {
  (void)v; (void)size;
  double h = xa[i + 1] - xa[i];
  double t = (x - xa[i]) / h;
  *y = ya[i] + t * (ya[i + 1] - ya[i]);
  return GSL_SUCCESS;
}
static int linear_deriv(const void *v, const double xa[], const double ya[],
                        size_t size, double x, size_t i, double *d) {
  (void)v; (void)size; (void)x;
  *d = (ya[i + 1] - ya[i]) / (xa[i + 1] - xa[i]);
  return GSL_SUCCESS;
}
static int linear_deriv2(const void *v, const double xa[], const double ya[],
                         size_t size, double x, size_t i, double *d2) {
  (void)v; (void)xa; (void)ya; (void)size; (void)x; (void)i;
  *d2 = 0.0;
  return GSL_SUCCESS;
}
static int linear_integ(const void *v, const double xa[], const double ya[],
                        size_t size, double a, double b, size_t ia, size_t ib,
                        double *result) {
  (void)v; (void)size;
  double acc = 0.0;
  for (size_t i = ia; i <= ib; i++) {
    double h = xa[i + 1] - xa[i];
    double sl = (ya[i + 1] - ya[i]) / h;
    double u = (i == ia) ? a - xa[i] : 0.0;
    double w = (i == ib) ? b - xa[i] : h;
    acc += (w - u) * (ya[i] + 0.5 * sl * (w + u));
  }
  *result = acc;
  return GSL_SUCCESS;
}

static const gsl_interp_type linear_type = {
    "linear", 2, linear_alloc, linear_init, linear_eval,
    linear_deriv, linear_deriv2, linear_integ, linear_free};
static const gsl_interp_type steffen_type = {
    "steffen", 3, cubic_alloc, steffen_init, cubic_eval,
    cubic_deriv, cubic_deriv2, cubic_integ, cubic_free};
static const gsl_interp_type akima_type = {
    "akima", 5, cubic_alloc, akima_init, cubic_eval,
    cubic_deriv, cubic_deriv2, cubic_integ, cubic_free};
static const gsl_interp_type akima_periodic_type = {
    "akima-periodic", 5, cubic_alloc, akima_periodic_init, cubic_eval,
    cubic_deriv, cubic_deriv2, cubic_integ, cubic_free};

const gsl_interp_type *gsl_interp_linear = &linear_type;
const gsl_interp_type *gsl_interp_steffen = &steffen_type;
const gsl_interp_type *gsl_interp_akima = &akima_type;
const gsl_interp_type *gsl_interp_akima_periodic = &akima_periodic_type;
/* not provided by the oracle (X-PSI selects them only on user request) */
const gsl_interp_type *gsl_interp_polynomial = NULL;
const gsl_interp_type *gsl_interp_cspline = NULL;
const gsl_interp_type *gsl_interp_cspline_periodic = NULL;

gsl_interp *gsl_interp_alloc(const gsl_interp_type *T, size_t n) {
  if (T == NULL) {
    gsl_error("interpolation type not provided by the oracle", __FILE__,
              __LINE__, GSL_EUNIMPL);
    return NULL;
  }
  if (n < T->min_size) {
    gsl_error("insufficient number of points for interpolation type",
              __FILE__, __LINE__, GSL_EINVAL);
    return NULL;
  }
  gsl_interp *g = (gsl_interp *)calloc(1, sizeof(*g));
  if (!g) return NULL;
  g->type = T;
  g->size = n;
  g->state = T->alloc(n);
  if (!g->state) {
    free(g);
    return NULL;
  }
  return g;
}

int gsl_interp_init(gsl_interp *g, const double xa[], const double ya[],
                    size_t size) {
  if (size != g->size) RAISE("data must match size of interpolation object", GSL_EINVAL);
  for (size_t i = 0; i + 1 < size; i++)
    if (!(xa[i] < xa[i + 1])) RAISE("x values must be strictly increasing", GSL_EINVAL);
  g->xmin = xa[0];
  g->xmax = xa[size - 1];
  return g->type->init(g->state, xa, ya, size);
}

const char *gsl_interp_name(const gsl_interp *g) { return g->type->name; }
unsigned int gsl_interp_min_size(const gsl_interp *g) { return g->type->min_size; }
unsigned int gsl_interp_type_min_size(const gsl_interp_type *T) { return T->min_size; }

void gsl_interp_free(gsl_interp *g) {
  if (!g) return;
  g->type->free(g->state);
  free(g);
}

int gsl_interp_eval_e(const gsl_interp *g, const double xa[],
                      const double ya[], double x, gsl_interp_accel *a,
                      double *y) {
  if (x < g->xmin || x > g->xmax) {
    *y = NAN;
    RAISE("interpolation error", GSL_EDOM);
  }
  size_t i = locate(xa, g->size, x, a);
  return g->type->eval(g->state, xa, ya, g->size, x, i, y);
}

double gsl_interp_eval(const gsl_interp *g, const double xa[],
                       const double ya[], double x, gsl_interp_accel *a) {
  double y;
  int st = gsl_interp_eval_e(g, xa, ya, x, a, &y);
  if (st != GSL_SUCCESS) return NAN;
  return y;
}

int gsl_interp_eval_deriv_e(const gsl_interp *g, const double xa[],
                            const double ya[], double x, gsl_interp_accel *a,
                            double *d) {
  if (x < g->xmin || x > g->xmax) {
    *d = NAN;
    RAISE("interpolation error", GSL_EDOM);
  }
  size_t i = locate(xa, g->size, x, a);
  return g->type->eval_deriv(g->state, xa, ya, g->size, x, i, d);
}

double gsl_interp_eval_deriv(const gsl_interp *g, const double xa[],
                             const double ya[], double x,
                             gsl_interp_accel *a) {
  double d;
  int st = gsl_interp_eval_deriv_e(g, xa, ya, x, a, &d);
  if (st != GSL_SUCCESS) return NAN;
  return d;
}

int gsl_interp_eval_deriv2_e(const gsl_interp *g, const double xa[],
                             const double ya[], double x,
                             gsl_interp_accel *a, double *d2) {
  if (x < g->xmin || x > g->xmax) {
    *d2 = NAN;
    RAISE("interpolation error", GSL_EDOM);
  }
  size_t i = locate(xa, g->size, x, a);
  return g->type->eval_deriv2(g->state, xa, ya, g->size, x, i, d2);
}

double gsl_interp_eval_deriv2(const gsl_interp *g, const double xa[],
                              const double ya[], double x,
                              gsl_interp_accel *a) {
  double d;
  int st = gsl_interp_eval_deriv2_e(g, xa, ya, x, a, &d);
  if (st != GSL_SUCCESS) return NAN;
  return d;
}

int gsl_interp_eval_integ_e(const gsl_interp *g, const double xa[],
                            const double ya[], double a, double b,
                            gsl_interp_accel *acc, double *result) {
  if (a > b || a < g->xmin || b > g->xmax) {
    *result = NAN;
    RAISE("interpolation error", GSL_EDOM);
  }
  if (a == b) {
    *result = 0.0;
    return GSL_SUCCESS;
  }
  size_t ia = locate(xa, g->size, a, acc);
  size_t ib = locate(xa, g->size, b, acc);
  return g->type->eval_integ(g->state, xa, ya, g->size, a, b, ia, ib, result);
}

double gsl_interp_eval_integ(const gsl_interp *g, const double xa[],
                             const double ya[], double a, double b,
                             gsl_interp_accel *acc) {
  double r;
  int st = gsl_interp_eval_integ_e(g, xa, ya, a, b, acc, &r);
  if (st != GSL_SUCCESS) return NAN;
  return r;
}

/* ------------------------------------------------------------------ */
/* QUADPACK QAG                                                        */
/* ------------------------------------------------------------------ */
typedef struct {
  const double *x, *wk, *wg;
  int half; /* nodes with x >= 0; x[half-1] == 0 is the centre */
} gk_rule;

static const gk_rule RULE21 = {GSLSUB_K21_X, GSLSUB_K21_WK, GSLSUB_K21_WG,
                               GSLSUB_K21_HALF};
static const gk_rule RULE61 = {GSLSUB_K61_X, GSLSUB_K61_WK, GSLSUB_K61_WG,
                               GSLSUB_K61_HALF};

/* one Gauss-Kronrod panel with the QUADPACK error estimate */
static void gk_apply(const gk_rule *R, const gsl_function *f, double a,
                     double b, double *result, double *abserr,
                     double *resabs, double *resasc, size_t *nev) {
  const int nh = R->half - 1; /* symmetric pairs */
  double c = 0.5 * (a + b), h = 0.5 * (b - a), ah = fabs(h);
  double fv1[32], fv2[32];
  double fc = GSL_FN_EVAL(f, c);
  double rk = R->wk[nh] * fc;
  double rg = R->wg[nh] * fc;
  double ra = fabs(rk);
  for (int j = 0; j < nh; j++) {
    double dx = h * R->x[j];
    double f1 = GSL_FN_EVAL(f, c - dx);
    double f2 = GSL_FN_EVAL(f, c + dx);
    fv1[j] = f1;
    fv2[j] = f2;
    rk += R->wk[j] * (f1 + f2);
    rg += R->wg[j] * (f1 + f2);
    ra += R->wk[j] * (fabs(f1) + fabs(f2));
  }
  double mean = 0.5 * rk;
  double rasc = R->wk[nh] * fabs(fc - mean);
  for (int j = 0; j < nh; j++)
    rasc += R->wk[j] * (fabs(fv1[j] - mean) + fabs(fv2[j] - mean));
  *result = rk * h;
  ra *= ah;
  rasc *= ah;
  double err = fabs((rk - rg) * h);
  if (rasc != 0.0 && err != 0.0) {
    double sc = pow(200.0 * err / rasc, 1.5);
    err = sc < 1.0 ? rasc * sc : rasc;
  }
  if (ra > DBL_MIN / (50.0 * DBL_EPSILON)) {
    double floor_err = 50.0 * DBL_EPSILON * ra;
    if (floor_err > err) err = floor_err;
  }
  *abserr = err;
  *resabs = ra;
  *resasc = rasc;
  if (nev) *nev += (size_t)(2 * nh + 1);
}

gsl_integration_workspace *gsl_integration_workspace_alloc(size_t n) {
  if (n == 0) {
    gsl_error("workspace length n must be positive integer", __FILE__,
              __LINE__, GSL_EDOM);
    return NULL;
  }
  gsl_integration_workspace *w =
      (gsl_integration_workspace *)calloc(1, sizeof(*w));
  w->limit = n;
  w->alist = (double *)malloc(n * sizeof(double));
  w->blist = (double *)malloc(n * sizeof(double));
  w->rlist = (double *)malloc(n * sizeof(double));
  w->elist = (double *)malloc(n * sizeof(double));
  return w;
}

void gsl_integration_workspace_free(gsl_integration_workspace *w) {
  if (!w) return;
  free(w->alist); free(w->blist); free(w->rlist); free(w->elist);
  free(w);
}

static size_t worst_interval(const gsl_integration_workspace *w) {
  size_t k = 0;
  for (size_t i = 1; i < w->size; i++)
    if (w->elist[i] > w->elist[k]) k = i;
  return k;
}

static int qag_core(const gsl_function *f, double a, double b, double epsabs,
                    double epsrel, size_t limit, const gk_rule *R,
                    gsl_integration_workspace *w, double *result,
                    double *abserr, size_t *nev, int quiet) {
#define QAG_FAIL(msg, code)                                  \
  do {                                                      \
    if (!quiet) gsl_error(msg, __FILE__, __LINE__, code);   \
    return code;                                            \
  } while (0)
  *result = 0.0;
  *abserr = 0.0;
  if (limit > w->limit) QAG_FAIL("iteration limit exceeds available workspace", GSL_EINVAL);
  if (epsabs <= 0.0 && (epsrel < 50.0 * DBL_EPSILON || epsrel < 0.5e-28))
    QAG_FAIL("tolerance cannot be achieved with given epsabs and epsrel", GSL_EBADTOL);

  double r0, e0, ra0, rc0;
  gk_apply(R, f, a, b, &r0, &e0, &ra0, &rc0, nev);
  w->size = 1;
  w->alist[0] = a; w->blist[0] = b; w->rlist[0] = r0; w->elist[0] = e0;

  double tol = fmax(epsabs, epsrel * fabs(r0));
  double roundoff_floor = 50.0 * DBL_EPSILON * ra0;
  if (e0 <= roundoff_floor && e0 > tol) {
    *result = r0; *abserr = e0;
    QAG_FAIL("cannot reach tolerance because of roundoff error on first attempt", GSL_EROUND);
  } else if ((e0 <= tol && e0 != rc0) || e0 == 0.0) {
    *result = r0; *abserr = e0;
    return GSL_SUCCESS;
  } else if (limit == 1) {
    *result = r0; *abserr = e0;
    QAG_FAIL("a maximum of one iteration was insufficient", GSL_EMAXITER);
  }

  double area = r0, errsum = e0;
  int rnd1 = 0, rnd2 = 0, fail_kind = 0;
  size_t iter = 1;
  size_t k = 0;
  do {
    double ai = w->alist[k], bi = w->blist[k], ri = w->rlist[k], ei = w->elist[k];
    double a1 = ai, b1 = 0.5 * (ai + bi), a2 = b1, b2 = bi;
    double r1, e1, ra1, rc1, r2, e2, ra2, rc2;
    gk_apply(R, f, a1, b1, &r1, &e1, &ra1, &rc1, nev);
    gk_apply(R, f, a2, b2, &r2, &e2, &ra2, &rc2, nev);
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
      if (rnd1 >= 6 || rnd2 >= 20) fail_kind = 2;
      double edge = (1.0 + 100.0 * DBL_EPSILON) * (fabs(a2) + 1000.0 * DBL_MIN);
      if (fabs(a1) <= edge && fabs(b2) <= edge) fail_kind = 3;
    }
    /* the half with the larger error keeps slot k, the other is appended */
    size_t nw = w->size++;
    if (e2 > e1) {
      w->alist[k] = a2; w->blist[k] = b2; w->rlist[k] = r2; w->elist[k] = e2;
      w->alist[nw] = a1; w->blist[nw] = b1; w->rlist[nw] = r1; w->elist[nw] = e1;
    } else {
      w->alist[k] = a1; w->blist[k] = b1; w->rlist[k] = r1; w->elist[k] = e1;
      w->alist[nw] = a2; w->blist[nw] = b2; w->rlist[nw] = r2; w->elist[nw] = e2;
    }
    k = worst_interval(w);
    iter++;
  } while (iter < limit && !fail_kind && errsum > tol);

  double sum = 0.0;
  for (size_t i = 0; i < w->size; i++) sum += w->rlist[i];
  *result = sum;
  *abserr = errsum;
  if (errsum <= tol) return GSL_SUCCESS;
  if (fail_kind == 2) QAG_FAIL("roundoff error prevents tolerance from being achieved", GSL_EROUND);
  if (fail_kind == 3) QAG_FAIL("bad integrand behavior found in the integration interval", GSL_ESING);
  if (iter == limit) QAG_FAIL("maximum number of subdivisions reached", GSL_EMAXITER);
  QAG_FAIL("could not integrate function", GSL_EFAILED);
#undef QAG_FAIL
}

int gsl_integration_qag(const gsl_function *f, double a, double b,
                        double epsabs, double epsrel, size_t limit, int key,
                        gsl_integration_workspace *w, double *result,
                        double *abserr) {
  const gk_rule *R;
  switch (key) {
    case GSL_INTEG_GAUSS21: R = &RULE21; break;
    case GSL_INTEG_GAUSS61: R = &RULE61; break;
    default:
      gsl_error("only the 21- and 61-point rules are provided by the oracle",
                __FILE__, __LINE__, GSL_EINVAL);
      return GSL_EINVAL;
  }
  return qag_core(f, a, b, epsabs, epsrel, limit, R, w, result, abserr, NULL,
                  0);
}

/* ---- stand-in for the doubly adaptive CQUAD routine ---- */
static unsigned long long g_cquad_evals = 0, g_cquad_calls = 0;
#define CQUAD_SUB_LIMIT 4000
gsl_integration_cquad_workspace *gsl_integration_cquad_workspace_alloc(const size_t n) {
  if (n < 3) {
    gsl_error("workspace size n must be at least 3", __FILE__, __LINE__, GSL_EDOM);
    return NULL;
  }
  gsl_integration_cquad_workspace *ws =
      (gsl_integration_cquad_workspace *)calloc(1, sizeof(*ws));
  ws->size = n;
  ws->w = gsl_integration_workspace_alloc(CQUAD_SUB_LIMIT);
  return ws;
}

void gsl_integration_cquad_workspace_free(gsl_integration_cquad_workspace *ws) {
  if (!ws) return;
  gsl_integration_workspace_free(ws->w);
  free(ws);
}

/* Dyadic pieces toward an endpoint where all the integrand's mass sits: the
 * window [lo, hi] is cut at lo + L 2^-k (toward lo) or hi - L 2^-k (toward
 * hi), each piece integrated adaptively, until the pieces stop contributing.
 * This is what a Clenshaw-Curtis scheme does implicitly for a spike at an
 * endpoint (its nodes include the endpoints); an interior Gauss-Kronrod rule
 * would otherwise see only zeros. */
static double dyadic_to_end(const gsl_function *f, double lo, double hi, int toward_lo,
                            double er, gsl_integration_workspace *w, size_t *nev) {
  const double L = hi - lo;
  double sum = 0.0;
  int seen = 0, quiet_after = 0;
  for (int k = 0; k < 2100; k++) {
    double s1 = ldexp(L, -(k + 1)), s0 = ldexp(L, -k);
    double p0 = toward_lo ? lo + s1 : hi - s0;
    double p1 = toward_lo ? lo + s0 : hi - s1;
    if (!(p0 < p1) || (toward_lo ? p0 <= lo : p1 >= hi)) break;
    double r, e;
    qag_core(f, p0, p1, 0.0, er, CQUAD_SUB_LIMIT, &RULE21, w, &r, &e, nev, 1);
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

int gsl_integration_cquad(const gsl_function *f, double a, double b,
                          double epsabs, double epsrel,
                          gsl_integration_cquad_workspace *ws, double *result,
                          double *abserr, size_t *nevals) {
  size_t nev = 0;
  double sign = 1.0;
  if (b < a) {
    double t = a; a = b; b = t; sign = -1.0;
  }
  if (a == b) {
    *result = 0.0; *abserr = 0.0;
    if (nevals) *nevals = 0;
    return GSL_SUCCESS;
  }
  double er = epsrel < 1.0e-13 ? epsrel : 1.0e-13;
  if (epsabs <= 0.0 && er < 50.0 * DBL_EPSILON) er = 50.0 * DBL_EPSILON;
  double r, e;
  /* quiet: a panel that stalls on round-off still returns its best sum */
  qag_core(f, a, b, epsabs, er, CQUAD_SUB_LIMIT, &RULE21, ws->w, &r, &e, &nev, 1);
  if (r == 0.0) {
    double fa = GSL_FN_EVAL(f, a), fb = GSL_FN_EVAL(f, b);
    nev += 2;
    if (fa != 0.0 || fb != 0.0) {
      double m = 0.5 * (a + b), rl, rr;
      if (fa != 0.0) rl = dyadic_to_end(f, a, m, 1, er, ws->w, &nev);
      else qag_core(f, a, m, 0.0, er, CQUAD_SUB_LIMIT, &RULE21, ws->w, &rl, &e, &nev, 1);
      if (fb != 0.0) rr = dyadic_to_end(f, m, b, 0, er, ws->w, &nev);
      else qag_core(f, m, b, 0.0, er, CQUAD_SUB_LIMIT, &RULE21, ws->w, &rr, &e, &nev, 1);
      r = rl + rr;
    }
  }
  *result = sign * r;
  *abserr = e;
  if (nevals) *nevals = nev;
  g_cquad_evals += nev;
  g_cquad_calls += 1;
  return GSL_SUCCESS;
}

/* test hook: integrand evaluations spent in the CQUAD stand-in so far */
unsigned long long gslsub_cquad_evals(int reset) {
  unsigned long long v = g_cquad_evals;
  if (reset) { g_cquad_evals = 0; g_cquad_calls = 0; }
  return v;
}
unsigned long long gslsub_cquad_calls(void) { return g_cquad_calls; }

/* ------------------------------------------------------------------ */
/* special functions                                                   */
/* ------------------------------------------------------------------ */
double gsl_sf_lnfact(const unsigned int n) { return lgamma((double)n + 1.0); }

/* ------------------------------------------------------------------ */
/* random numbers: splitmix64 + Poisson by inversion / PTRS.  Used     */
/* only by X-PSI's synthesis module, never on the likelihood path.      */
/* ------------------------------------------------------------------ */
static const gsl_rng_type splitmix_type = {"splitmix64"};
const gsl_rng_type *gsl_rng_default = &splitmix_type;
const gsl_rng_type *gsl_rng_env_setup(void) { return gsl_rng_default; }
gsl_rng *gsl_rng_alloc(const gsl_rng_type *T) {
  gsl_rng *r = (gsl_rng *)calloc(1, sizeof(*r));
  r->type = T;
  r->s = 0x9e3779b97f4a7c15ULL;
  return r;
}
void gsl_rng_set(const gsl_rng *r, unsigned long int s) {
  ((gsl_rng *)r)->s = (unsigned long long)s * 0x9e3779b97f4a7c15ULL + 1ULL;
}
void gsl_rng_free(gsl_rng *r) { free(r); }
double gsl_rng_uniform(const gsl_rng *r) {
  gsl_rng *q = (gsl_rng *)r;
  unsigned long long z = (q->s += 0x9e3779b97f4a7c15ULL);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  z ^= z >> 31;
  return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}
unsigned int gsl_ran_poisson(const gsl_rng *r, double mu) {
  if (mu <= 0.0) return 0;
  if (mu < 30.0) { /* inversion */
    double p = exp(-mu), s = p, u = gsl_rng_uniform(r);
    unsigned int k = 0;
    while (u > s && k < 100000) {
      k++;
      p *= mu / k;
      s += p;
    }
    return k;
  }
  /* Hormann 1993 transformed rejection (PTRS) */
  double smu = sqrt(mu), b = 0.931 + 2.53 * smu, a = -0.059 + 0.02483 * b;
  double inv_alpha = 1.1239 + 1.1328 / (b - 3.4), vr = 0.9277 - 3.6224 / (b - 2);
  for (;;) {
    double U = gsl_rng_uniform(r) - 0.5, V = gsl_rng_uniform(r);
    double us = 0.5 - fabs(U);
    double k = floor((2 * a / us + b) * U + mu + 0.43);
    if (us >= 0.07 && V <= vr) return (unsigned int)k;
    if (k < 0 || (us < 0.013 && V > us)) continue;
    if (log(V) + log(inv_alpha) - log(a / (us * us) + b) <=
        -mu + k * log(mu) - lgamma(k + 1))
      return (unsigned int)k;
  }
}
