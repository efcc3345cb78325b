/*
 * xpsi_gb300.h -- C ABI of the GB300 pulse-likelihood kernels.
 *
 * Plain C types only: pointers, sizes, doubles and int32 flags.  Two layers:
 *
 *  1. Drop-in entry points, one per native callable on X-PSI's likelihood
 *     path.  They take HOST arrays with the reference's layouts (C-contiguous
 *     float64, int32 flags), copy them to the GPU, run the kernels and copy the
 *     result back before returning.  Return value: >= 0 is the reference's own
 *     status word; < 0 is a CUDA or usage failure (xgpu_last_error() says why).
 *
 *  2. Batched entry points that take DEVICE pointers and a cudaStream_t
 *     (passed as void*), for many parameter vectors per launch.
 *
 * No entry point raises; errors are return codes, as in the reference
 * (HotRegion.py:12-19 maps the integer statuses to exceptions).
 */
#ifndef XPSI_GB300_H
#define XPSI_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* 2: xgpu_integrate takes the elsewhere correction (correction_srcCellParams,
 * n_correction, else_atm_ext); the elsewhere, general, Stokes, synthesis and
 * Gaussian-likelihood entry points were added.
 * 3: xgpu_atmos5d, xgpu_integrate_split and xgpu_integrate_split_stokes (split
 * atmospheres); xgpu_integrate_stokes takes the I and Q tables of atm_ext 4
 * (Pol_Num2D), which xgpu_integrate and xgpu_integrate_general also take;
 * xgpu_integrate_general_stokes; xgpu_phase_interpolator, xgpu_energy_interpolator.
 * 4: xgpu_atmos_cache_invalidate; xgpu_integrate takes beam_opt and xgpu_mesh
 * carries it; xgpu_poisson_loglike_batch, xgpu_poisson_likelihood_given_background;
 * xgpu_fold_batch_tc takes a status word; xgpu_fold_tc_timeout_selftest. */
#define XGPU_ABI_VERSION 4

/* Status words of the batched layer (per parameter vector). */
enum {
  XGPU_OK = 0,
  XGPU_RAY_FAIL = 1,      /* rays.pyx:331-339 -> HotRegion.RayError */
  XGPU_PULSE_FAIL = 2,    /* integrator terminate -> HotRegion.PulseError */
  XGPU_ATMOS_BOUNDS = 3,  /* Photosphere.py:486-507 */
  XGPU_QUAD_FAIL = 4,     /* vanished marginal integral -> random llzero */
  XGPU_SLIM_CUT = 5,      /* slim early exit */
  XGPU_BAD_INPUT = 6,
  XGPU_DEVICE_TIMEOUT = 8 /* a bounded wait in a kernel ran out */
};

int xgpu_abi_version(void);
/* Text of the last failure on the calling thread ("" if none). */
const char *xgpu_last_error(void);

/* Numerical 4-D atmosphere (hot_Num4D.pyx), the tuple X-PSI preloads:
 * grids logT[nT], logg[ng], mu[nmu], logE[nE] and the row-major intensity
 * table [nT][ng][nmu][nE] (preload.pyx:6-35). */
typedef struct {
  const double *logT, *logg, *mu, *logE, *intensity;
  size_t nT, ng, nmu, nE;
  /* optional FP32 copy of the intensity table, read by the mixed-precision
   * integrator only (NULL: it converts from the FP64 table) */
  const float *intensity_f32;
} xgpu_atmos4d;

/* The drop-in entry points keep one device copy of the last Num4D table per
 * device, keyed by the host pointers, the sizes and a strided sample of the
 * table (the reference preloads a table once and never edits it).  A caller
 * that edits a table in place, or frees one and allocates another at the
 * same address, calls this before its next call on the calling thread's
 * current device; it waits for the device and frees the copy.  No counterpart
 * in the reference (which reads the host table directly). */
int xgpu_atmos_cache_invalidate(void);

/* ---------------------------------------------------------------------- */
/* 1. drop-in entry points (host arrays)                                  */
/* ---------------------------------------------------------------------- */

/* Replaces xpsi.cellmesh.rays.compute_rays (xpsi/cellmesh/rays.pyx:249-390).
 * maxAlpha[N_u] is clamped in place as the reference does (:317-318).
 * Outputs deflection, cos_alpha, lag [N_u][N_R] and maxDeflection[N_u].
 * Returns the reference's terminate flag (0 or 1). */
int xgpu_compute_rays(size_t N_u, double r_s, const double *r_s_over_R,
                      double *maxAlpha, size_t N_R, double *deflection,
                      double *cos_alpha, double *lag, double *maxDeflection);

/* Replaces xpsi.cellmesh.integrator_for_azimuthal_invariance.integrate
 * (xpsi/cellmesh/integrator_for_azimuthal_invariance.pyx:70-98) for uniform
 * hot regions with no disk (R_in >= 1e6).  beam_opt 0-3 as the reference's
 * (hot_wrapper.pyx:153-199); options 1-3 read (abb, bbb, cbb, dbb, nimu) from
 * parameters 2-6 of each parallel's first radiating cell (n_params >= 7),
 * and option 3 takes atm_ext 1 or 2.  atm_ext 1 = blackbody,
 * 2 = Num4D (atmos required), 3 = the burst blackbody's intensity
 * (hot_BB_burst.pyx), 4 = Pol_Num2D's intensity (hot_Num2D.pyx:
 * atmos->mu, logE and intensity [nmu][nE] on (mu, log10 E/keV); the other
 * fields unused).  correction_srcCellParams[S0][S1][n_correction]
 * or NULL is the elsewhere correction (:257-261,469-478,593-594); the GPU
 * path corrects for a blackbody elsewhere (else_atm_ext 1).
 * image_order_limit 0 means "infer" (the reference's None).  flux[N_E][N_P]
 * is written on success.  Returns 0 (SUCCESS) or 1 (ERROR, :657-665). */
int xgpu_integrate(double R, double omega, double r_s, double inclination,
                   size_t S0, size_t S1, const double *cellArea,
                   const double *radialCoords_of_parallels,
                   const double *r_s_over_r, const double *theta,
                   const double *phi, const double *srcCellParams,
                   size_t n_params, const int32_t *cell_radiates,
                   const double *correction_srcCellParams, size_t n_correction,
                   size_t N_R, const double *deflection,
                   const double *cos_alpha, const double *lag,
                   const double *maxDeflection, const double *cos_gammaArray,
                   size_t N_E, const double *energies, size_t N_L,
                   const double *leaves, size_t N_P, const double *phases,
                   int atm_ext, const xgpu_atmos4d *atmos, int else_atm_ext,
                   int image_order_limit, int beam_opt, double *flux);

/* A split atmosphere (hot_Num5D_split.pyx:77-220): grids of t_e, t_bb,
 * tau, mu and E (electron rest energies), intensity [n0][n1][n2][n3][n4]. */
typedef struct {
  const double *grid[5];
  size_t n[5];
  const double *intensity;
} xgpu_atmos5d;

/* Replaces xpsi.cellmesh.integrator_for_azimuthal_invariance_split.integrate
 * (xpsi/cellmesh/integrator_for_azimuthal_invariance_split.pyx:74-103), the
 * integrator of a uniform hot region with a split atmosphere: the 5-D table
 * is reduced to (mu, E) at the first cell's (t_e, t_bb, tau) (:270-275) and
 * evaluated per leaf and energy at E / Z in electron rest energies
 * (:457-471).  Other arguments and the return value as xgpu_integrate
 * (beam_opt 0, no disk). */
int xgpu_integrate_split(double R, double omega, double r_s, double inclination,
                         size_t S0, size_t S1, const double *cellArea,
                         const double *radialCoords_of_parallels,
                         const double *r_s_over_r, const double *theta,
                         const double *phi, const double *srcCellParams,
                         size_t n_params, const int32_t *CELL_RADIATES,
                         const double *correction_srcCellParams,
                         size_t n_correction, size_t N_R,
                         const double *deflection, const double *cos_alpha,
                         const double *lag, const double *maxDeflection,
                         const double *cos_gammaArray, size_t N_E,
                         const double *energies, size_t N_L,
                         const double *leaves, size_t N_P,
                         const double *phases, const xgpu_atmos5d *atmos,
                         int else_atm_ext, int image_order_limit, double *flux);

/* Replaces xpsi.cellmesh.integratorIQU_for_azimuthal_invariance.integrate
 * (xpsi/cellmesh/integratorIQU_for_azimuthal_invariance.pyx:68-743), the
 * Stokes integrator of HotRegion.integrate_stokes: arguments as
 * xgpu_integrate, atm_ext 1 (blackbody, Q = U = 0), 3 (burst blackbody,
 * hot_BB_burst.pyx) or 4 (Pol_Num2D, hot_Num2D.pyx: atmos_I and atmos_Q
 * hold the I and Q tables [nmu][nE] on the same (mu, log10 E/keV) grids in
 * mu, logE and intensity; other fields unused; NULL otherwise); outputs
 * flux_I, flux_Q, flux_U [N_E][N_P].  Returns 0 (SUCCESS) or 1 (ERROR),
 * < 0 on a usage or CUDA failure. */
int xgpu_integrate_stokes(double R, double omega, double r_s, double inclination,
                          size_t S0, size_t S1, const double *cellArea,
                          const double *radialCoords_of_parallels,
                          const double *r_s_over_r, const double *theta,
                          const double *phi, const double *srcCellParams,
                          size_t n_params, const int32_t *cell_radiates,
                          const double *correction_srcCellParams,
                          size_t n_correction, size_t N_R,
                          const double *deflection, const double *cos_alpha,
                          const double *lag, const double *maxDeflection,
                          const double *cos_gammaArray, size_t N_E,
                          const double *energies, size_t N_L,
                          const double *leaves, size_t N_P, const double *phases,
                          int atm_ext, const xgpu_atmos4d *atmos_I,
                          const xgpu_atmos4d *atmos_Q, int else_atm_ext,
                          int image_order_limit, double *flux_I, double *flux_Q,
                          double *flux_U);

/* Replaces xpsi.cellmesh.integratorIQU_for_azimuthal_invariance_split.integrate
 * (xpsi/cellmesh/integratorIQU_for_azimuthal_invariance_split.pyx:75-758),
 * the Stokes integrator of a split hot region: the I and Q split tables
 * (same mu and E grids) are each reduced to (mu, E) at the first cell's
 * (t_e, t_bb, tau) (:310-322), then I, Q cos 2chi and Q sin 2chi are
 * integrated as xgpu_integrate_split does I (:515-530).  Returns as
 * xgpu_integrate_stokes. */
int xgpu_integrate_split_stokes(double R, double omega, double r_s,
                                double inclination, size_t S0, size_t S1,
                                const double *cellArea,
                                const double *radialCoords_of_parallels,
                                const double *r_s_over_r, const double *theta,
                                const double *phi, const double *srcCellParams,
                                size_t n_params, const int32_t *CELL_RADIATES,
                                const double *correction_srcCellParams,
                                size_t n_correction, size_t N_R,
                                const double *deflection, const double *cos_alpha,
                                const double *lag, const double *maxDeflection,
                                const double *cos_gammaArray, size_t N_E,
                                const double *energies, size_t N_L,
                                const double *leaves, size_t N_P,
                                const double *phases, const xgpu_atmos5d *atmos_I,
                                const xgpu_atmos5d *atmos_Q, int else_atm_ext,
                                int image_order_limit, double *flux_I,
                                double *flux_Q, double *flux_U);

/* Replaces xpsi.cellmesh.integrator.integrate (xpsi/cellmesh/integrator.pyx:
 * 48-667), the general integrator of HotRegion(symmetry=False) for source
 * parameters that vary from cell to cell.  Same arguments as xgpu_integrate,
 * with atm_ext 3 (burst blackbody's intensity) also taken (the phase
 * interpolant of the geometric factor is Akima periodic, the reference's
 * default).  Returns 0 (SUCCESS) or 1 (ERROR, :657-665), < 0 on a
 * usage or CUDA failure. */
int xgpu_integrate_general(double R, double omega, double r_s,
                           double inclination, size_t S0, size_t S1,
                           const double *cellArea,
                           const double *radialCoords_of_parallels,
                           const double *r_s_over_r, const double *theta,
                           const double *phi, const double *srcCellParams,
                           size_t n_params, const int32_t *cell_radiates,
                           const double *correction_srcCellParams,
                           size_t n_correction, size_t N_R,
                           const double *deflection, const double *cos_alpha,
                           const double *lag, const double *maxDeflection,
                           const double *cos_gammaArray, size_t N_E,
                           const double *energies, size_t N_L,
                           const double *leaves, size_t N_P,
                           const double *phases, int atm_ext,
                           const xgpu_atmos4d *atmos, int else_atm_ext,
                           int image_order_limit, double *flux);

/* Replaces xpsi.cellmesh.integratorIQU.integrate
 * (xpsi/cellmesh/integratorIQU.pyx:76-717), the Stokes integrator of
 * HotRegion(symmetry=False): arguments as xgpu_integrate_general, with
 * atmos_I and atmos_Q as xgpu_integrate_stokes takes them (atm_ext 1, 2 with
 * Q = 0, 3, 4).  The polarisation angle of each (parallel, image) is the
 * reference's: computed from the leaf loop's last values (:593-596).
 * Outputs flux_I, flux_Q, flux_U [N_E][N_P]. */
int xgpu_integrate_general_stokes(double R, double omega, double r_s,
                                  double inclination, size_t S0, size_t S1,
                                  const double *cellArea,
                                  const double *radialCoords_of_parallels,
                                  const double *r_s_over_r, const double *theta,
                                  const double *phi, const double *srcCellParams,
                                  size_t n_params, const int32_t *cell_radiates,
                                  const double *correction_srcCellParams,
                                  size_t n_correction, size_t N_R,
                                  const double *deflection, const double *cos_alpha,
                                  const double *lag, const double *maxDeflection,
                                  const double *cos_gammaArray, size_t N_E,
                                  const double *energies, size_t N_L,
                                  const double *leaves, size_t N_P,
                                  const double *phases, int atm_ext,
                                  const xgpu_atmos4d *atmos_I,
                                  const xgpu_atmos4d *atmos_Q, int else_atm_ext,
                                  int image_order_limit, double *flux_I,
                                  double *flux_Q, double *flux_U);

/* Replaces xpsi.tools.phase_interpolator.phase_interpolator
 * (xpsi/tools/phase_interpolator.pyx:25-95, the default Akima-periodic
 * interpolant): signal[rows][n_phases] on phases (cycles, [0, 1]) evaluated
 * at new_phases + phase_shift wrapped into [0, 1); values <= 0 become 0
 * unless allow_negative.  out[rows][n_new]. */
int xgpu_phase_interpolator(size_t n_new, const double *new_phases, size_t n_phases,
                            const double *phases, size_t rows, const double *signal,
                            double phase_shift, int allow_negative, double *out);

/* Replaces xpsi.tools.energy_interpolator.energy_interpolator
 * (xpsi/tools/energy_interpolator.pyx:27-125, the default Steffen
 * interpolant): each column of signal[N_E][n_cols] splined in log10 E (in
 * log10 of the signal when the column is positive throughout) at
 * log10_new_energies; 0 above the last energy.  out[n_new][n_cols], the
 * reference's return. */
int xgpu_energy_interpolator(size_t N_E, size_t n_cols, const double *signal,
                             const double *log10_energies, size_t n_new,
                             const double *log10_new_energies, double *out);

/* Replaces xpsi.tools.energy_integrator.energy_integrator
 * (xpsi/tools/energy_integrator.pyx:27-31).  signal[N_E][N_P]; log10 energies
 * and log10 interval edges; out[n_edges-1][N_P] (the reference's return,
 * already transposed). */
int xgpu_energy_integrator(size_t N_E, size_t N_P, const double *signal,
                           const double *log10_energies, size_t n_edges,
                           const double *log10_edges, double *out);

/* Replaces Instrument.__call__'s fold (xpsi/Instrument.py:192-197):
 * out[K][N] = matrix[K][0:q] @ signal[q][N]; ld is the matrix row stride. */
int xgpu_response_fold(size_t K, size_t q, size_t N, const double *matrix,
                       size_t ld, const double *signal, double *out);

/* Replaces default_background_marginalisation.precomputation (:38-68). */
int xgpu_precomputation(size_t K, size_t B, const int32_t *counts,
                        double *out);

/* Replaces default_background_marginalisation.eval_marginal_likelihood
 * (:450-734).  H components (hot regions), each components[h] is [K][n_phases]
 * with phases component_phases[h][n_phases]; all components must share one
 * phase grid.  support[K][2]; background[K][B] or NULL.  Outputs: *loglike,
 * star[K][B], mcl_bg[K], mcl_bg_support[K].  Returns 0, or XGPU_SLIM_CUT /
 * XGPU_QUAD_FAIL when the reference would return a random llzero draw (the
 * draw is in *loglike). */
int xgpu_eval_marginal_likelihood(
    double exposure_time, size_t B, const double *phase_edges, size_t K,
    const double *counts, size_t H, const double *const *components,
    const size_t *n_phases, const double *const *component_phases,
    const double *phase_shifts, const double *neg_sum_ln_data_factorial,
    const double *support, double epsabs, double epsrel, double epsilon,
    double sigmas, double llzero, const int32_t *allow_negative, double slim,
    const double *background, double *loglike, double *star, double *mcl_bg,
    double *mcl_bg_support);

/* ---------------------------------------------------------------------- */
/* 2. batched entry points (device pointers, asynchronous on `stream`)    */
/* ---------------------------------------------------------------------- */

/* One cell mesh of one parameter vector (a hot region's superseding or
 * ceding member).  Rows of all meshes are packed: mesh m owns rows
 * [row_off, row_off+S0) and cells [cell_off, cell_off+S0*S1). */
typedef struct {
  int32_t S0, S1;
  int64_t row_off, cell_off;
  double omega, inclination;
  int32_t image_order_limit, atm_ext;
  int64_t flux_off;
  /* beaming modification of the hot intensity (hot_wrapper.pyx:153-199):
   * 0 none; 1, 2, 3 as the reference's beam_opt, reading (abb, bbb, cbb,
   * dbb, nimu) from parameters 2-6 of the parallel's first radiating cell
   * (n_params >= 7); 3 takes atm_ext 1 or 2; the mixed form takes 0 only. */
  int32_t beam_opt, reserved;
} xgpu_mesh;

/* Ray tables for n_rows packed rows (per-row u and r_s).  When lag_C and
 * lag_scale are non-NULL the lag is calibrated in place as
 * HotRegion.py:880-901 does: lag = (lag - lag_C[row]) * lag_scale[row].
 * row_status[row] gets XGPU_RAY_FAIL where the reference would terminate. */
int xgpu_rays_batch(int64_t n_rows, int N_R, const double *u,
                    const double *r_s, double *maxAlpha, double *deflection,
                    double *cos_alpha, double *lag, double *maxDeflection,
                    int32_t *row_status, const double *lag_C,
                    const double *lag_scale, void *stream);

/* Integrator over n_meshes packed meshes.  `meshes` is a HOST array; every
 * other pointer is device memory.  flux receives [N_E][N_P] per mesh at
 * meshes[m].flux_off; mesh_status[m] gets XGPU_PULSE_FAIL on terminate.
 * The work is cut on the device into about 4 target_ctas chunks of
 * consecutive parallels of equal estimated cost (images x radiating cells,
 * the image counts from maxDeflection); target_ctas <= 0 takes 8 per SM. */
typedef struct {
  const int32_t *row_mesh;
  const double *radius, *u, *cos_gamma, *theta0, *maxDeflection;
  const double *deflection, *cos_alpha, *lag;
  const double *cellArea, *phi, *params;
  int32_t n_params;
  const int32_t *radiates;
  const double *energies, *leaves, *phases;
  xgpu_atmos4d atmos; /* device pointers; intensity NULL when no mesh is Num4D */
  double *flux;
  int32_t *mesh_status;
  double *flop_counter; /* optional: algorithmic FLOPs of the launch are added */
  /* optional elsewhere correction for every mesh of the launch (FP64 form):
   * [cells][n_correction], log T of a blackbody elsewhere first; NULL: none */
  const double *correction;
  int32_t n_correction;
} xgpu_integrate_batch_data;

int xgpu_integrate_batch(int n_meshes, const xgpu_mesh *meshes, int64_t n_rows,
                         int N_R, int N_E, int N_L, int N_P,
                         const xgpu_integrate_batch_data *d, int target_ctas,
                         void *stream);

/* Mixed-precision form of xgpu_integrate_batch (same arguments): leaf
 * geometry, visibility and phase knots in FP64; atmosphere interpolation,
 * Akima pieces and the cell x phase sums in FP32; partial sums in FP64.
 * Not bitwise the reference; its error against the FP64 path is reported
 * per evaluation by the batched driver. */
int xgpu_integrate_batch_mixed(int n_meshes, const xgpu_mesh *meshes,
                               int64_t n_rows, int N_R, int N_E, int N_L,
                               int N_P, const xgpu_integrate_batch_data *d,
                               int target_ctas, void *stream);

/* Energy integration of n_signals [N_E][N_P] signals at in_off[s] (device
 * int64 offsets) into [n_edges-1][N_P] at out_off[s]; d_sq[s] divides the
 * signal first (Likelihood.py:361-364); accumulate adds into out. */
int xgpu_energy_batch(int n_signals, int N_E, int N_P, int n_edges,
                      const double *signal, const int64_t *in_off,
                      const double *log10_energies, const double *log10_edges,
                      const double *d_sq, double *out, const int64_t *out_off,
                      int accumulate, void *stream);

/* The fold of xgpu_fold_batch on the tensor cores for the mixed-precision form: every
 * FP64 operand is split as hi + lo in TF32 and out = M_hi in_hi + M_hi in_lo
 * + M_lo in_hi is accumulated in FP32 (tcgen05.mma, TMEM accumulator; FP32-
 * class relative error ~1e-7).  Same arguments and layouts as
 * xgpu_fold_batch; the operand splits use stream-ordered scratch memory. */
int xgpu_fold_batch_tc(int batch, int K, int q, int N, const double *matrix, int ld,
                       const double *in, double *out, int32_t *status, void *stream);
/* status (device int32, may be NULL; the caller zeroes it) of
 * xgpu_fold_batch_tc: 1 when a bounded wait on the TMA unit or the tensor
 * core ran out (the tile is written as NaN), 2 when the second, bounded wait
 * for the operations in flight ran out as well.  xgpu_fold_tc_timeout_selftest
 * runs one tile whose producer issues nothing, so that both waits run out
 * after a short limit without any copy or MMA in flight, and returns the
 * status word it reported (2) in *status_out: the failure path checked
 * without a GPU fault.  No counterpart in the reference. */
int xgpu_fold_tc_timeout_selftest(int32_t *status_out);

/* out[b][K][N] = matrix[K][0:q] @ in[b][q][N] for b < batch, FP64-class:
 * each row of the matrix and each column of in[b] is scaled by a power of two
 * and split into a pair of floats, and the products and sums run in
 * double-float arithmetic (~1e-14 of the sum of the terms' magnitudes; an
 * infinite input gives NaN where it reaches).  Stream-ordered scratch of
 * about the size of in plus 8 K q bytes. */
int xgpu_fold_batch(int batch, int K, int q, int N, const double *matrix,
                    int ld, const double *in, double *out, void *stream);

/* Background-marginalised log-likelihood for n_vec evaluations sharing one
 * data set: signals[n_vec][H][K][N_P], shifts[n_vec][H]; chan_ll and
 * chan_flag are [n_vec][K] scratch; star [n_vec][K][B] and the background
 * estimates [n_vec][K] may be NULL.  loglike[n_vec], status[n_vec]. */
typedef struct {
  int32_t n_vec, K, B, H, N_P;
  double exposure, epsabs, epsrel, epsilon, sigmas, llzero, slim;
  const double *phase_edges, *comp_phases, *counts, *precomp, *support;
  const double *background, *signals, *shifts;
  const int32_t *allow_negative;
  double *chan_ll;
  int32_t *chan_flag;
  double *star, *mcl_bg, *mcl_bg_support, *loglike;
  int32_t *status;
} xgpu_likelihood_batch_data;

int xgpu_likelihood_batch(const xgpu_likelihood_batch_data *d, void *stream);

/* Allocation-free form of xgpu_likelihood_batch.  It has no counterpart in
 * the reference: it exists for callers that cannot allocate device memory at
 * call time -- a host whose framework owns all device memory through its own
 * pool, or code held to a memory budget fixed in advance.  Inputs and outputs
 * are the caller's device buffers exactly as for xgpu_likelihood_batch; the
 * scratch arrays d->chan_ll and d->chan_flag are IGNORED and replaced by a
 * fixed 4 MiB device array inside this library (12 bytes per evaluation and
 * channel: n_vec * K <= 349525), which every GPU that loads the library
 * holds until the process exits.  No device memory is allocated or freed.
 * The first call on a device looks up that array's device address (with the
 * device current), and so does the first call after the device's context was
 * re-created (cudaDeviceReset); make such a call before any stream capture.  All calls share the one array, so calls that overlap on the GPU
 * (other streams, other threads) race: serialise them on one stream.
 * Returns 0, -2 for invalid sizes, -3 when n_vec * K exceeds the maximum,
 * -4 when the array's address cannot be obtained, -5 when the launch fails. */
int xgpu_likelihood_batch_static(const xgpu_likelihood_batch_data *d, void *stream);

/* Measurement helper (no counterpart in the reference): launches an FMA
 * throughput probe (fp64 != 0: FP64, else FP32) and returns the FLOPs it
 * issues, so that kernel rates can be quoted against the device's own FP64 /
 * FP32 issue peaks.  out: device scratch of 8 bytes. */
double xgpu_peak_probe(int fp64, int blocks, int threads, int iters, void *out,
                       void *stream);

/* ---------------------------------------------------------------------- */
/* 3. host-side cell meshes for the batched path (CPU, multithreaded)     */
/* ---------------------------------------------------------------------- */

/* Replaces xpsi.cellmesh.mesh_tools.allocate_cells
 * (xpsi/cellmesh/mesh_tools.pyx:892-1099); out4 = (super_sqrt_num_cells,
 * super_num_cells, cede_sqrt_num_cells, cede_num_cells). */
int xgpu_allocate_cells(size_t num_cells, size_t min_sqrt, size_t max_sqrt,
                        double R_eq, double Omega, double zeta, double epsilon,
                        int star_shape_ind, double super_radius,
                        double cede_radius, double super_colatitude,
                        double cede_colatitude, double super_azimuth,
                        double hole_colatitude, double hole_radius,
                        double hole_azimuth, double *out4);

/* Replaces construct_spot_cellMesh (xpsi/cellmesh/mesh.pyx:23-417, polar 0)
 * and construct_polar_cellMesh (xpsi/cellmesh/polar_mesh.pyx:23-430,
 * polar 1).  Arguments follow the reference (ceding = enclosing region,
 * superseding = omitted/superseding region inside it).  Outputs:
 * theta, phi, area [S][S]; r, maxAlpha, cos_gamma, effGrav [S]. */
int xgpu_cell_mesh(int polar, size_t num_cells, size_t S, double R_eq,
                   double zeta, double epsilon, int star_shape_ind,
                   double cede_radius, double cede_colatitude,
                   double super_radius, double super_colatitude,
                   double super_azimuth, double *theta, double *phi, double *r,
                   double *area, double *maxAlpha, double *cos_gamma,
                   double *effGrav);

typedef struct {
  int32_t polar;
  size_t num_cells, S;
  double R_eq, zeta, epsilon;
  int32_t star_shape_ind;
  double cede_radius, cede_colatitude, super_radius, super_colatitude,
      super_azimuth;
  double *theta, *phi, *r, *area, *maxAlpha, *cos_gamma, *effGrav;
} xgpu_mesh_request;

/* Many meshes at once on n_threads host threads (0: all cores). */
int xgpu_cell_mesh_many(int n, const xgpu_mesh_request *req, int n_threads);

/* Many cell budgets (xgpu_allocate_cells) at once on n_threads host threads
 * (0: all cores); each request's result lands in its out[4]. */
typedef struct {
  size_t num_cells, min_sqrt, max_sqrt;
  double R_eq, Omega, zeta, epsilon;
  int32_t star_shape_ind;
  double super_radius, cede_radius, super_colatitude, cede_colatitude,
      super_azimuth, hole_colatitude, hole_radius, hole_azimuth;
  double out[4];
} xgpu_alloc_request;

int xgpu_allocate_cells_many(int n, xgpu_alloc_request *req, int n_threads);

/* ---------------------------------------------------------------------- */
/* The meshes of a batch built on the GPU and written straight into the     */
/* packed arrays of xgpu_rays_batch / xgpu_integrate_batch (device          */
/* pointers).  Member m's mesh (the request fields as in xgpu_mesh_request) */
/* owns rows [row_off, row_off + S) and cells [cell_off, cell_off + S^2),   */
/* packed in member order.  Per row: u = r_s / r, r_s, maxAlpha, radius,    */
/* cos_gamma, theta0 (the row's colatitude), the lag calibration offset     */
/* lag_C (HotRegion.py:880-901) and lag_scale, row_mesh = m.  Per cell:     */
/* cellArea, phi (cell azimuth - omit_azimuth, + pi when antiphased),       */
/* params = (logT, log10 effective gravity of the row), radiates =          */
/* cellArea > 0.  Scratch comes from the stream-ordered allocator.          */
/* Returns 0, -2 on inconsistent members, -5 on a CUDA error.               */
/* ---------------------------------------------------------------------- */
typedef struct {
  int32_t polar;
  size_t num_cells, S;
  double R_eq, zeta, epsilon;
  int32_t star_shape_ind;
  double cede_radius, cede_colatitude, super_radius, super_colatitude,
      super_azimuth;
  int64_t row_off, cell_off;
  double r_s, lag_scale, omit_azimuth, logT;
  int32_t antiphased;
} xgpu_mesh_member;

typedef struct {
  double *u, *r_s, *maxAlpha, *radius, *cos_gamma, *theta0, *lag_C, *lag_scale;
  int32_t *row_mesh;
  double *cellArea, *phi, *params;
  int32_t *radiates;
} xgpu_mesh_batch_out;

int xgpu_mesh_batch(int n, const xgpu_mesh_member *members, int64_t n_rows,
                    int64_t n_cells, const xgpu_mesh_batch_out *out, void *stream);

/* ---------------------------------------------------------------------- */
/* The photosphere elsewhere: closed mesh and time-invariant integrator.    */
/* ---------------------------------------------------------------------- */

/* Replaces xpsi.cellmesh.global_mesh.construct_closed_cellMesh
 * (xpsi/cellmesh/global_mesh.pyx:21-137), host C++.  S = sqrt_numCell, even
 * and >= 4.  Outputs theta[S][S], phi[S][S], r[S], *cellArea (the one area
 * every cell has), maxAlpha[S], cos_gamma[S], effGrav[S].  Returns 0, or -1
 * for an odd or too small S. */
int xgpu_closed_cell_mesh(size_t S, size_t num_cells, double R_eq, double zeta,
                          double epsilon, int star_shape_ind, double *theta,
                          double *phi, double *r, double *cellArea,
                          double *maxAlpha, double *cos_gamma, double *effGrav);

/* Many closed meshes at once on n_threads host threads (0: all cores). */
typedef struct {
  size_t S, num_cells;
  double R_eq, zeta, epsilon;
  int32_t star_shape_ind;
  double *theta, *phi, *r, *cellArea, *maxAlpha, *cos_gamma, *effGrav;
} xgpu_closed_mesh_request;
int xgpu_closed_cell_mesh_many(int n, const xgpu_closed_mesh_request *req,
                               int n_threads);

/* Replaces xpsi.cellmesh.integrator_for_time_invariance.integrate
 * (xpsi/cellmesh/integrator_for_time_invariance.pyx:59-338).  Arguments in
 * the reference's order: the closed mesh's S = sqrt_numPix parallels of S
 * cells, its scalar cellArea, srcCellParams[S][S][n_params], ray tables
 * [S][N_R]; atm_ext 1 (blackbody) or 2 (Num4D, `atmos`); image_order_limit
 * 0 for the reference's None.  flux[N_E] receives the spectrum.  Returns 0,
 * 1 where the reference returns (ERROR, None), < 0 on a usage or CUDA
 * failure (including a parallel with more than 8 images). */
int xgpu_integrate_time_invariant(double R, double omega, double r_s,
                                  double inclination, size_t sqrt_numPix,
                                  double cellArea,
                                  const double *radialCoords_of_parallels,
                                  const double *r_s_over_r, const double *theta,
                                  const double *phi, const double *srcCellParams,
                                  size_t n_params, size_t N_R,
                                  const double *deflection,
                                  const double *cos_alpha,
                                  const double *maxDeflection,
                                  const double *cos_gammaArray, size_t N_E,
                                  const double *energies, int atm_ext,
                                  const xgpu_atmos4d *atmos,
                                  int image_order_limit, double *flux);

/* Batched form over n_meshes packed closed meshes.  `meshes` is a HOST
 * array; every other pointer is device memory.  Mesh m owns the packed
 * parallels [row_off, row_off + S) and cells [cell_off, cell_off + S*S).
 * flux receives [n_meshes][N_E]; mesh_status[m] gets XGPU_PULSE_FAIL where
 * the reference would return (ERROR, None) and XGPU_BAD_INPUT for a parallel
 * with more images than max_images (0: 8).  When `signal` is not NULL each
 * successful mesh's spectrum is also added to every phase column of
 * signal[m * signal_stride + e * signal_N_P + p] (the time-invariant
 * component added to the first hot region's signal, Photosphere.py:588-592);
 * the launch must follow the one that wrote the signal on the stream. */
typedef struct {
  int32_t S, row_off;
  int64_t cell_off;
  double omega, inclination, cellArea;
  int32_t image_order_limit, atm_ext;
} xgpu_elsewhere_mesh;

typedef struct {
  const int32_t *row_mesh;
  const double *radius, *u, *cos_gamma, *theta0, *maxDeflection;
  const double *deflection, *cos_alpha;
  const double *phi, *params;
  int32_t n_params;
  const double *energies;
  xgpu_atmos4d atmos; /* device pointers; intensity NULL when no mesh is Num4D */
  double *flux;
  int32_t *mesh_status;
  double *signal;            /* optional, see above */
  int64_t signal_stride;
  int32_t signal_N_P;
} xgpu_elsewhere_batch_data;

int xgpu_elsewhere_batch(int n_meshes, const xgpu_elsewhere_mesh *meshes,
                         int64_t n_rows, int N_R, int N_E, int max_images,
                         const xgpu_elsewhere_batch_data *d, void *stream);

/* ---------------------------------------------------------------------- */
/* Synthesis: expected counts, phase integration, Poisson realisations.     */
/* ---------------------------------------------------------------------- */

/* One component signal (count rates [K][ld], phases [n] in cycles on [0, 1],
 * phase shift in cycles). */
typedef struct {
  const double *signal;
  const double *phases;
  int64_t ld;
  int32_t n;
  double shift;
} xgpu_component;

/* Replaces compute_expected_counts (xpsi/tools/compute_expected_counts.pyx:
 * 200-276), the core of synthesise_exposure and
 * synthesise_given_total_count_number (xpsi/tools/synthesise.pyx).  HOST
 * arrays: H components over the phase-bin edges phases[B + 1]; background
 * count rates [K][B] or NULL; allow_negative[H].  out[K][B] = exposure x
 * (sum of the components' bin-integrated rates, clamped at zero, + the
 * background rate).  Returns 0, < 0 on a usage or CUDA failure. */
int xgpu_compute_expected_counts(double exposure_time, size_t B,
                                 const double *phases, size_t K, size_t H,
                                 const xgpu_component *components,
                                 const double *background,
                                 const int32_t *allow_negative, double *out);

/* Replaces xpsi.tools.phase_integrator.phase_integrator
 * (xpsi/tools/phase_integrator.pyx:23-121): signal[rows][n_phases] (HOST)
 * integrated over the phase-shifted bins of phases[n_edges], times the
 * exposure; out[rows][n_edges - 1]. */
int xgpu_phase_integrator(double exposure_time, size_t n_edges,
                          const double *phases, size_t rows, size_t n_phases,
                          const double *signal, const double *signal_phases,
                          double phase_shift, int allow_negative, double *out);

/* Poisson realisations of mean[n] (HOST): out[i] ~ Poisson(mean[i]) drawn
 * from Philox4x32-10 keyed by `seed` at element offset + i (so a draw
 * depends only on the seed and its element number).  The law is GSL's
 * gsl_ran_poisson's (synthesise.pyx:130-140); the stream is not GSL's.
 * Returns 0, 1 if a draw hit the rejection loop's bound, < 0 on failure. */
int xgpu_poisson(size_t n, const double *mean, uint64_t seed, uint64_t offset,
                 double *out);

/* Batched forms (device pointers; `components` is a HOST array of
 * n_sets x H descriptors whose pointers are device memory). */
int xgpu_expected_counts_batch(int n_sets, int K, int B, int H,
                               double exposure, const double *phase_edges,
                               const xgpu_component *components,
                               const int32_t *allow_negative,
                               const double *background, double *out,
                               void *stream);
/* Poisson log-likelihood of data counts[K][B] (device) given the expected
 * counts[n_sets][K][B] (star plus a known background, device) of n_sets
 * evaluations, the core of xpsi.likelihoods._poisson_likelihood_given_background
 * (xpsi/likelihoods/_poisson_likelihood_given_background.pyx:82-109):
 * loglike[set] = sum_i (precomp[i] + sum_j over E_ij > 0 of d_ij log E_ij -
 * E_ij), precomp (neg_sum_ln_data_factorial) may be NULL; n_penalty[set]
 * counts the bins with E_ij <= 0 that are not d_ij == E_ij == 0, each of
 * which the reference penalises by -1e90 (0.1 + 0.9 U(0, 1)) (left to the
 * caller, as it is random). */
int xgpu_poisson_loglike_batch(int n_sets, int K, int B, const double *expected,
                               const double *counts, const double *precomp, double *loglike,
                               int32_t *n_penalty, void *stream);

/* Replaces the numerical part of
 * xpsi.likelihoods._poisson_likelihood_given_background.poisson_likelihood_given_background
 * (xpsi/likelihoods/_poisson_likelihood_given_background.pyx:14-109), HOST
 * arrays: expected[K][B] = compute_expected_counts(exposure_time, phases,
 * components, background, allow_negative) as xgpu_compute_expected_counts
 * forms it, *loglike the log-likelihood before penalties, *n_penalty the
 * number of penalised bins (see xgpu_poisson_loglike_batch). */
int xgpu_poisson_likelihood_given_background(double exposure_time, size_t B,
                                             const double *phases, size_t K,
                                             const double *counts, size_t H,
                                             const xgpu_component *components,
                                             const double *background,
                                             const double *neg_sum_ln_data_factorial,
                                             const int32_t *allow_negative, double *expected,
                                             double *loglike, int64_t *n_penalty);

/* fail (device int32, may be NULL) is set to 1 if a draw hit the bound. */
int xgpu_poisson_batch(int64_t n, const double *mean, double *out,
                       uint64_t seed, uint64_t offset, int32_t *fail,
                       void *stream);

/* Gaussian log-likelihoods of polarimetry (HOST arrays):
 * -sum_ij (model_ij - data_ij)^2 / (2 errors_ij^2) + log(2 pi errors_ij^2)/2
 * over data[rows][cols]; model row i starts at model + i * model_row_stride
 * (0: one model row for every data row, as _gaussian_likelihood_QnUn.pyx:
 * 31-36 does; cols: the expected counts of
 * _gaussian_likelihood_given_background_IQU.pyx:70-78). */
int xgpu_gaussian_loglike(size_t rows, size_t cols, const double *model,
                          size_t model_row_stride, const double *data,
                          const double *errors, double *loglike);
/* Batched form (device pointers): n_sets models at model_set_stride against
 * one data set; loglike[n_sets]. */
int xgpu_gaussian_loglike_batch(int n_sets, int rows, int cols,
                                const double *model, int64_t model_set_stride,
                                int64_t model_row_stride, const double *data,
                                const double *errors, double *loglike,
                                void *stream);

#ifdef __cplusplus
}
#endif
#endif /* XPSI_GB300_H */
