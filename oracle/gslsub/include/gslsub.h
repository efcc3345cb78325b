/*
 * gslsub.h -- declarations of the small part of the GNU Scientific Library
 * API that X-PSI's likelihood path calls (xpsi/include/GSL.pxd names them).
 *
 * TEST INFRASTRUCTURE (oracle only).  This is NOT GSL: GSL is not installed
 * in this environment, so the oracle carries its own implementation of the
 * algorithms behind these names, written from the published methods:
 *   Steffen (1990) monotone cubic, Akima (1970) with periodic ends,
 *   QUADPACK QAG (Piessens et al. 1983) with Gauss-Kronrod 21/61 rules.
 * gsl_integration_cquad is served by the same adaptive Gauss-Kronrod scheme
 * run to a tighter relative tolerance (see gslsub.c).
 * Only names and argument meanings follow GSL's public API.
 */
#ifndef XPSI_ORACLE_GSLSUB_H
#define XPSI_ORACLE_GSLSUB_H

#include <stddef.h>
#include <math.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- error codes and handler (gsl_errno.h) ---- */
enum {
  GSL_SUCCESS = 0, GSL_FAILURE = -1, GSL_CONTINUE = -2, GSL_EDOM = 1,
  GSL_ERANGE = 2, GSL_EFAULT = 3, GSL_EINVAL = 4, GSL_EFAILED = 5,
  GSL_EFACTOR = 6, GSL_ESANITY = 7, GSL_ENOMEM = 8, GSL_EBADFUNC = 9,
  GSL_ERUNAWAY = 10, GSL_EMAXITER = 11, GSL_EZERODIV = 12, GSL_EBADTOL = 13,
  GSL_ETOL = 14, GSL_EUNDRFLW = 15, GSL_EOVRFLW = 16, GSL_ELOSS = 17,
  GSL_EROUND = 18, GSL_EBADLEN = 19, GSL_ENOTSQR = 20, GSL_ESING = 21,
  GSL_EDIVERGE = 22, GSL_EUNSUP = 23, GSL_EUNIMPL = 24, GSL_ECACHE = 25,
  GSL_ETABLE = 26, GSL_ENOPROG = 27, GSL_ENOPROGJ = 28, GSL_ETOLF = 29,
  GSL_ETOLX = 30, GSL_ETOLG = 31, GSL_EOF = 32
};
typedef void gsl_error_handler_t(const char *reason, const char *file,
                                 int line, int gsl_errno);
gsl_error_handler_t *gsl_set_error_handler(gsl_error_handler_t *h);
gsl_error_handler_t *gsl_set_error_handler_off(void);
void gsl_error(const char *reason, const char *file, int line, int gsl_errno);
const char *gsl_strerror(const int gsl_errno);

/* ---- math helpers (gsl_math.h / gsl_sys.h) ---- */
typedef struct {
  double (*function)(double x, void *params);
  void *params;
} gsl_function;
#define GSL_FN_EVAL(F, x) (*((F)->function))(x, (F)->params)
typedef struct {
  double (*f)(double x, void *params);
  double (*df)(double x, void *params);
  void (*fdf)(double x, void *params, double *f, double *df);
  void *params;
} gsl_function_fdf;
#define GSL_FN_FDF_EVAL_F(FDF, x) (*((FDF)->f))(x, (FDF)->params)
#define GSL_FN_FDF_EVAL_DF(FDF, x) (*((FDF)->df))(x, (FDF)->params)
#define GSL_FN_FDF_EVAL_F_DF(FDF, x, y, dy) (*((FDF)->fdf))(x, (FDF)->params, (y), (dy))
int gsl_isnan(const double x);
int gsl_isinf(const double x);
int gsl_finite(const double x);

/* ---- 1-D interpolation (gsl_interp.h) ---- */
typedef struct gsl_interp_type {
  const char *name;
  unsigned int min_size;
  void *(*alloc)(size_t size);
  int (*init)(void *state, const double xa[], const double ya[], size_t size);
  int (*eval)(const void *state, const double xa[], const double ya[],
              size_t size, double x, size_t i, double *y);
  int (*eval_deriv)(const void *state, const double xa[], const double ya[],
                    size_t size, double x, size_t i, double *d);
  int (*eval_deriv2)(const void *state, const double xa[], const double ya[],
                     size_t size, double x, size_t i, double *d2);
  int (*eval_integ)(const void *state, const double xa[], const double ya[],
                    size_t size, double a, double b, size_t ia, size_t ib,
                    double *result);
  void (*free)(void *state);
} gsl_interp_type;

typedef struct {
  const gsl_interp_type *type;
  double xmin;
  double xmax;
  size_t size;
  void *state;
} gsl_interp;

typedef struct {
  size_t cache;
  size_t miss_count;
  size_t hit_count;
} gsl_interp_accel;

extern const gsl_interp_type *gsl_interp_linear;
extern const gsl_interp_type *gsl_interp_polynomial;
extern const gsl_interp_type *gsl_interp_cspline;
extern const gsl_interp_type *gsl_interp_cspline_periodic;
extern const gsl_interp_type *gsl_interp_akima;
extern const gsl_interp_type *gsl_interp_akima_periodic;
extern const gsl_interp_type *gsl_interp_steffen;

gsl_interp_accel *gsl_interp_accel_alloc(void);
size_t gsl_interp_accel_find(gsl_interp_accel *a, const double xa[],
                             size_t size, double x);
int gsl_interp_accel_reset(gsl_interp_accel *a);
void gsl_interp_accel_free(gsl_interp_accel *a);
size_t gsl_interp_bsearch(const double xa[], double x, size_t lo, size_t hi);

gsl_interp *gsl_interp_alloc(const gsl_interp_type *T, size_t n);
int gsl_interp_init(gsl_interp *obj, const double xa[], const double ya[],
                    size_t size);
const char *gsl_interp_name(const gsl_interp *interp);
unsigned int gsl_interp_min_size(const gsl_interp *interp);
unsigned int gsl_interp_type_min_size(const gsl_interp_type *T);
int gsl_interp_eval_e(const gsl_interp *obj, const double xa[],
                      const double ya[], double x, gsl_interp_accel *a,
                      double *y);
double gsl_interp_eval(const gsl_interp *obj, const double xa[],
                       const double ya[], double x, gsl_interp_accel *a);
int gsl_interp_eval_deriv_e(const gsl_interp *obj, const double xa[],
                            const double ya[], double x, gsl_interp_accel *a,
                            double *d);
double gsl_interp_eval_deriv(const gsl_interp *obj, const double xa[],
                             const double ya[], double x,
                             gsl_interp_accel *a);
int gsl_interp_eval_deriv2_e(const gsl_interp *obj, const double xa[],
                             const double ya[], double x,
                             gsl_interp_accel *a, double *d2);
double gsl_interp_eval_deriv2(const gsl_interp *obj, const double xa[],
                              const double ya[], double x,
                              gsl_interp_accel *a);
int gsl_interp_eval_integ_e(const gsl_interp *obj, const double xa[],
                            const double ya[], double a, double b,
                            gsl_interp_accel *acc, double *result);
double gsl_interp_eval_integ(const gsl_interp *obj, const double xa[],
                             const double ya[], double a, double b,
                             gsl_interp_accel *acc);
void gsl_interp_free(gsl_interp *interp);

/* ---- spline wrapper (gsl_spline.h): declared for completeness ---- */
typedef struct {
  gsl_interp *interp;
  double *x;
  double *y;
  size_t size;
} gsl_spline;

/* ---- integration (gsl_integration.h) ---- */
enum {
  GSL_INTEG_GAUSS15 = 1, GSL_INTEG_GAUSS21 = 2, GSL_INTEG_GAUSS31 = 3,
  GSL_INTEG_GAUSS41 = 4, GSL_INTEG_GAUSS51 = 5, GSL_INTEG_GAUSS61 = 6
};
typedef struct gsl_integration_workspace {
  size_t limit;
  size_t size;
  double *alist, *blist, *rlist, *elist;
} gsl_integration_workspace;
typedef struct gsl_integration_cquad_ival { double a, b, r, e; } gsl_integration_cquad_ival;
typedef struct gsl_integration_cquad_workspace {
  size_t size;
  gsl_integration_workspace *w;
} gsl_integration_cquad_workspace;
typedef struct gsl_integration_qaws_table gsl_integration_qaws_table;
typedef struct gsl_integration_qawo_table gsl_integration_qawo_table;

gsl_integration_workspace *gsl_integration_workspace_alloc(size_t n);
void gsl_integration_workspace_free(gsl_integration_workspace *w);
int gsl_integration_qag(const gsl_function *f, double a, double b,
                        double epsabs, double epsrel, size_t limit, int key,
                        gsl_integration_workspace *workspace, double *result,
                        double *abserr);
gsl_integration_cquad_workspace *gsl_integration_cquad_workspace_alloc(const size_t n);
void gsl_integration_cquad_workspace_free(gsl_integration_cquad_workspace *w);
int gsl_integration_cquad(const gsl_function *f, double a, double b,
                          double epsabs, double epsrel,
                          gsl_integration_cquad_workspace *ws, double *result,
                          double *abserr, size_t *nevals);

/* ---- special functions (gsl_sf_gamma.h, gsl_sf_result.h) ---- */
typedef struct { double val; double err; } gsl_sf_result;
typedef struct { double val; double err; int e10; } gsl_sf_result_e10;
double gsl_sf_lnfact(const unsigned int n);

/* ---- random numbers (gsl_rng.h, gsl_randist.h): synthesis only ---- */
typedef struct gsl_rng_type { const char *name; } gsl_rng_type;
typedef struct gsl_rng { const gsl_rng_type *type; unsigned long long s; } gsl_rng;
extern const gsl_rng_type *gsl_rng_default;
const gsl_rng_type *gsl_rng_env_setup(void);
gsl_rng *gsl_rng_alloc(const gsl_rng_type *T);
void gsl_rng_set(const gsl_rng *r, unsigned long int s);
void gsl_rng_free(gsl_rng *r);
double gsl_rng_uniform(const gsl_rng *r);
unsigned int gsl_ran_poisson(const gsl_rng *r, double mu);

/* ---- opaque types named by GSL.pxd but unused on the path ---- */
typedef struct { size_t size; double *data; } gsl_block;
typedef struct { size_t size; size_t stride; double *data; gsl_block *block; int owner; } gsl_vector;
typedef struct { gsl_vector vector; } gsl_vector_view;
typedef struct { gsl_vector vector; } gsl_vector_const_view;
typedef struct { size_t size1, size2, tda; double *data; gsl_block *block; int owner; } gsl_matrix;
typedef struct { gsl_matrix matrix; } gsl_matrix_view;
typedef struct { gsl_matrix matrix; } gsl_matrix_const_view;
typedef struct gsl_interp2d_type gsl_interp2d_type;
typedef struct gsl_interp2d gsl_interp2d;
typedef struct gsl_spline2d gsl_spline2d;
typedef struct gsl_odeiv2_system gsl_odeiv2_system;
typedef struct gsl_odeiv2_step gsl_odeiv2_step;
typedef struct gsl_odeiv2_control gsl_odeiv2_control;
typedef struct gsl_odeiv2_evolve gsl_odeiv2_evolve;
typedef struct gsl_odeiv2_driver gsl_odeiv2_driver;
typedef struct gsl_odeiv2_step_type gsl_odeiv2_step_type;
typedef struct gsl_odeiv2_control_type gsl_odeiv2_control_type;
typedef enum { GSL_SF_LEGENDRE_SCHMIDT, GSL_SF_LEGENDRE_SPHARM, GSL_SF_LEGENDRE_FULL, GSL_SF_LEGENDRE_NONE } gsl_sf_legendre_t;

#ifdef __cplusplus
}
#endif
#endif
