// kernels.h -- argument blocks and launchers of the pulse-likelihood kernels.
// Every pointer here is a DEVICE pointer; host staging lives in abi.cu.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace xg {

constexpr int kMaxImages = 8;  // image orders tracked per parallel

// ---- K1 rays ----------------------------------------------------------
struct RaysArgs {
  int n_rows, N_R;
  const double *u;        // [rows] r_s / r of the parallel
  const double *r_s_row;  // [rows] Schwarzschild radius (m)
  double *maxAlpha;       // [rows] in/out (clamped, rays.pyx:317-318)
  double *deflection, *cos_alpha, *lag;  // [rows][N_R]
  double *maxDeflection;  // [rows]
  int32_t *row_status;    // [rows] or null
  const double *lag_C;     // [rows] lag calibration offset (s) or null
  const double *lag_scale; // [rows] 2 pi f_mode
};
void launch_rays(const RaysArgs &a, cudaStream_t st);

// ---- K2/K3 integrator ----------------------------------------------------
// One "member" is one cell mesh (a hot region's superseding or ceding part)
// of one parameter vector.  Rows of all members are packed: member m owns
// global rows [row_off, row_off + S0) and cells [cell_off, cell_off + S0*S1).
struct MemberDesc {
  int32_t S0, S1;
  int64_t row_off, cell_off;
  double omega, inclination;
  int32_t image_order_limit;  // 0: infer from the maximum deflection
  int32_t atm;                // 1 blackbody, 2 numerical 4-D table
  int64_t flux_off;           // offset of this member's [N_E][N_P] flux
  int32_t beam_opt;           // beaming modification 0-3 (hot_wrapper.pyx:153-199)
  int32_t reserved;
};

struct Atmos4D {
  const double *logT, *logg, *mu, *logE, *I;
  int nT, ng, nmu, nE;
  const float *I32;  // FP32 copy of the table for the mixed form (or null)
};

struct IntegrateArgs {
  int n_members;
  int64_t n_rows;
  const MemberDesc *members;
  // per packed row
  const int32_t *row_member;
  const double *radius, *u, *cos_gamma, *theta0, *maxDeflection;
  const double *deflection, *cos_alpha, *lag;  // [rows][N_R], lag calibrated
  int N_R;
  // per packed cell
  const double *cellArea, *phi, *params;  // params [cells][n_params]
  int n_params;
  const int32_t *radiates;
  // elsewhere correction (FP64 form only): a blackbody elsewhere whose
  // intensity at correction[cell of the parallel's first radiating cell][0]
  // (log T) is subtracted from every profile value; null: none
  const double *correction;   // [cells][n_correction]
  int n_correction;
  // shared grids
  int N_E, N_L, N_P;
  const double *energies, *leaves, *phases;
  Atmos4D atmos;
  // work chunks, planned on the device from per-parallel costs before the
  // integrator runs (integrator.cu, plan_chunks_kernel): chunk c covers rows
  // [chunk_r0[c], chunk_r1[c]) of one member; the grid is max_chunks CTAs and
  // CTA b takes chunk chunk_order[b] (heaviest first) while b < *chunk_count
  int max_chunks;           // bound on the planned chunks (2 target + members)
  int target_chunks;        // chunks the plan aims at
  int64_t *chunk_r0, *chunk_r1;  // [max_chunks]
  double *partial;          // [max_chunks][N_E][N_P], written by each chunk's CTA
  double *partial2 = nullptr;  // the same for the power sums' second cell half, or null
  int32_t *chunk_first;     // [n_members + 1] first chunk of each member
  int32_t *chunk_order;     // [max_chunks]
  int32_t *chunk_count;     // [1]
  float *row_cost;          // [n_rows] scratch: estimated cost of each parallel
  float *chunk_cost;        // [max_chunks] scratch
  // Num4D call-history state (see integrator.cu)
  uint8_t *row_has_eval, *row_last_top, *row_entry_top;  // [rows]
  int32_t *member_status;   // [n_members]
  double *flux;             // [..] at members[m].flux_off
  double *flop_counter;     // algorithmic FLOPs of the launch (atomic), or null
  double *slab;             // [max_chunks][nmu][nE] contracted Num4D table (scratch)
  // power sums of the cell x phase sums (FP64 form; scratch, or null for the
  // per-cell form): w_slots slots of 2 * w_cap * N_P run records, a CTA
  // holding one (w_slot_busy[slot] = 1) while it runs, see integrator.cu
  unsigned char *wsum = nullptr;
  int w_cap = 0;            // runs per (cell half, signal phase)
  int w_slots = 0;
  int32_t *w_slot_busy = nullptr;  // [w_slots], zero before the launch
  int mixed;                // 0: FP64 drop-in, 1: mixed-precision form
  double *flux_q = nullptr, *flux_u = nullptr;  // Stokes Q, U (launch_stokes only)
  // Stokes Q of a 2-D table atmosphere (atm 4, 6; launch_stokes only):
  // [nmu][nE] on the grids of atmos (whose I is the intensity table)
  const double *table_q = nullptr;
};
// the 5-D split atmosphere's reduction to (mu, E) at one parameter vector
struct SplitArgs {
  const double *grid[5];
  int n[5];
  const double *I;      // [n0][n1][n2][n3][n4]
  double vec[3];        // t_e, t_bb, tau
  double *out;          // [n3][n4]
};
void launch_split_reduce(const SplitArgs &a, cudaStream_t st);
void launch_integrate(const IntegrateArgs &a, cudaStream_t st);
// scratch bytes per chunk of the FP64 integrator's power sums for parallels
// of at most max_cells cells (w_cap runs per cell half and signal phase)
size_t integrate_wsum_bytes(int N_P, int max_cells, int *w_cap);
// Stokes I (a.flux), Q, U for blackbody (1) and burst blackbody (3) members;
// a.partial: stokes_partial_doubles(a) doubles, zeroed; a.chunk_* unused
size_t stokes_partial_doubles(const IntegrateArgs &a);
size_t stokes_smem_bytes(int N_L, int N_P, int N_E, int N_R, int nmu = 0, int nE = 0);
int launch_stokes(const IntegrateArgs &a, cudaStream_t st);

// ---- K4 energy integrator ------------------------------------------------
struct EnergyArgs {
  int n_signals;        // number of [N_E][N_P] inputs
  int N_E, N_P, n_edges;
  const double *signal;      // [n_signals][N_E][N_P]
  const int64_t *in_off;     // [n_signals] element offset of each signal
  const double *logE;        // [N_E]
  const double *logEdges;    // [n_edges]
  double scale;              // multiplies the signal (1 / d^2 folded in)
  const double *scale_per;   // [n_signals] or null
  double *out;               // [n_signals][n_edges-1][N_P] at out_off
  const int64_t *out_off;
  int accumulate;            // add into out instead of storing
};
void launch_energy(const EnergyArgs &a, cudaStream_t st);

// ---- K5 response fold -----------------------------------------------------
// out[b][K][N] = M[K][q] @ in[b][q][N] in FP64
struct FoldArgs {
  int batch, K, q, N;
  const double *M;  // [K][ldM], columns [0, q)
  int ldM;
  const double *in;  // [batch][q][N]
  double *out;       // [batch][K][N]
  // tensor-core form: set to 1 when a wait on the tensor core or the TMA
  // unit timed out (the tile is written as NaN), 2 when the wait for the
  // operations in flight timed out as well; may be null
  int32_t *status = nullptr;
};
// double-float form (FP64-class): scratch is fold_scratch_bytes(a) bytes of
// device memory, 16-byte aligned
size_t fold_scratch_bytes(const FoldArgs &a);
void launch_fold(const FoldArgs &a, void *scratch, cudaStream_t st);
// tensor-core form (3xTF32 split products, FP32 accumulation in TMEM);
// scratch: fold_tc_scratch_bytes(a) bytes of device memory, 16-byte aligned.
// Returns 0, or < 0 when the tile maps cannot be encoded.
size_t fold_tc_scratch_bytes(const FoldArgs &a);
int launch_fold_tc(const FoldArgs &a, void *scratch, cudaStream_t st);
// the tensor-core fold's timeout path exercised without a fault: one tile
// whose producer issues nothing, so its waits run out after a short limit;
// the kernel reports through a.status (expected 2) and frees its tensor
// memory.  a.K, a.q, a.N, a.batch small; scratch as launch_fold_tc.
int launch_fold_tc_timeout_selftest(const FoldArgs &a, void *scratch, cudaStream_t st);
double launch_peak_probe(int fp64, int blocks, int threads, int iters, void *out,
                         cudaStream_t st);

// ---- K6 likelihood ----------------------------------------------------------
struct LikeArgs {
  int n_vec;             // likelihood evaluations
  int K, B, H;           // channels, phase bins, components (hot regions)
  int N_P;               // phases per component signal
  double exposure, epsabs, epsrel, epsilon, sigmas, llzero, slim;
  const double *phase_edges;  // [B+1]
  const double *comp_phases;  // [N_P] phases (cycles) of every component
  const double *counts;       // [K][B]
  const double *precomp;      // [K]
  const double *support;      // [K][2]
  const double *background;   // [K][B] or null
  const double *signals;      // [n_vec][H][K][N_P]
  const double *shifts;       // [n_vec][H]
  const int32_t *allow_negative;  // [H]
  double *chan_ll;            // [n_vec][K] per-channel log-likelihood terms
  int32_t *chan_flag;         // [n_vec][K] 0 ok, 1 slim cut, 2 vanished integral
  double *star;               // [n_vec][K][B] or null
  double *mcl_bg, *mcl_bg_s;  // [n_vec][K] or null
  double *loglike;            // [n_vec]
  int32_t *status;            // [n_vec]
};
void launch_likelihood(const LikeArgs &a, cudaStream_t st);
void launch_precomputation(int K, int B, const int32_t *counts, double *out, cudaStream_t st);

// ---- the photosphere elsewhere (time-invariant integrator) --------------------
struct ElseMeshDesc {
  int32_t S;                  // parallels = cells per parallel (closed mesh)
  int32_t row_off;            // first packed parallel
  int64_t cell_off;           // first packed cell ([S][S] from here)
  double omega, inclination, cellArea;
  int32_t image_order_limit;  // 0: ceil(maxDeflection / pi) per parallel
  int32_t atm_ext;            // 1 blackbody, 2 Num4D
};
struct ElsewhereArgs {
  int n_meshes;
  int64_t n_rows;
  int N_R, N_E;
  int max_S;                  // largest S of the launch
  int max_images;             // images held per cell (parallels needing more report kBadInput)
  const ElseMeshDesc *meshes;
  const int32_t *row_mesh;    // [n_rows]
  const double *radius, *u, *cos_gamma, *theta0, *maxDeflection;  // [n_rows]
  const double *deflection, *cos_alpha;                           // [n_rows][N_R]
  const double *phi;          // [cells]
  const double *params;       // [cells][n_params]
  int n_params;
  const double *energies;     // [N_E]
  Atmos4D atmos;
  double *row_flux;           // [n_rows][N_E] scratch
  double *flux;               // [n_meshes][N_E]
  int32_t *status;            // [n_meshes], zeroed by the caller
  double *signal;             // or null: mesh m's spectrum is added to every phase
  int64_t signal_stride;      //   column of signal[m * signal_stride + e * signal_N_P + p]
  int signal_N_P;
};
size_t elsewhere_smem_bytes(int N_R, int max_S, int max_images);

// ---- the general integrator (HotRegion symmetry=False) -------------------------
struct GeneralArgs {
  int S0, S1, N_R, N_L, N_P, N_E;
  int IOmax;                  // images held per parallel in the entry scratch
  double omega, inclination;
  int image_order_limit;      // 0: ceil(maxDeflection / pi) per parallel
  int atm_ext;                // 1 blackbody, 2 Num4D, 3 burst blackbody, 4 Pol_Num2D
  int stokes;                 // 1: also Q and U (integratorIQU.pyx)
  const int32_t *radiates;    // [S0][S1]
  const double *cellArea, *phi, *params;  // [S0][S1], [S0][S1], [S0][S1][n_params]
  int n_params;
  const double *correction;   // [S0][S1][n_correction] or null (blackbody elsewhere)
  int n_correction;
  const double *radius, *u, *cos_gamma, *theta0, *maxDeflection;  // [S0]
  const double *deflection, *cos_alpha, *lag;                     // [S0][N_R]
  const double *energies, *leaves, *phases;
  Atmos4D atmos;              // Num4D table, or Pol_Num2D's I table (mu, logE, I)
  const double *table_q;      // Pol_Num2D's Q table on the same grids (Stokes)
  double *chi2;               // [S0][IOmax][2] cos, sin of twice the polarisation angle
  double *eG, *eZ, *eA;       // [S0][IOmax][S1][N_P] entry scratch
  int32_t *n_img;             // [S0] images evaluated per parallel
  double *partial;            // [S0][IOmax][1 or 3][N_E][N_P]
  double *flux;               // [N_E][N_P]
  double *flux_q, *flux_u;    // [N_E][N_P] (Stokes)
  int32_t *status;            // [1], zeroed by the caller
};
size_t general_geometry_smem_bytes(int N_R, int N_L);
int launch_general(const GeneralArgs &a, cudaStream_t st);

// ---- synthesis: expected counts, phase integration, Poisson draws ----------
struct CompDesc {             // one component signal of one set
  const double *signal;       // [K][ld] count rates
  const double *phases;       // [n] phases in cycles on [0, 1]
  int64_t ld;
  int n;
  double shift;               // phase shift in cycles
};
struct ExpectedArgs {
  int n_sets, K, B, H;
  double exposure;
  const double *phase_edges;  // [B + 1]
  const CompDesc *comps;      // [n_sets][H]
  const int32_t *allow_negative;  // [H]
  const double *background;   // [K][B] count rates, or null
  double *out;                // [n_sets][K][B]
};
void launch_expected_counts(const ExpectedArgs &a, cudaStream_t st);
// Poisson log-likelihood given the expected counts (star + known background)
// of n_sets evaluations sharing one data set
// (_poisson_likelihood_given_background.pyx:82-109): per set the channels'
// constants plus sum_ij (d_ij log E_ij - E_ij) over E_ij > 0, and the count
// of bins with E_ij <= 0 that are not (d_ij == 0 and E_ij == 0) (the
// reference's randomised -1e90 penalty, applied by the host)
struct PoissonArgs {
  int n_sets, K, B;
  const double *expected;   // [n_sets][K][B]
  const double *counts;     // [K][B]
  const double *precomp;    // [K] (neg_sum_ln_data_factorial) or null
  double *chan_ll;          // [n_sets][K] scratch
  int32_t *chan_pen;        // [n_sets][K] scratch
  double *loglike;          // [n_sets]
  int32_t *n_penalty;       // [n_sets]
};
void launch_poisson_loglike(const PoissonArgs &a, cudaStream_t st);
struct PhaseIntArgs {
  int64_t rows;
  int n_phases, B;
  double exposure, shift;
  int allow_negative;
  const double *phase_edges;    // [B + 1]
  const double *signal;         // [rows][n_phases]
  const double *signal_phases;  // [n_phases]
  double *out;                  // [rows][B]
};
// the phase (Akima periodic) and energy (Steffen) interpolators
struct InterpArgs {
  int64_t rows;          // signal rows (phase) or columns (energy)
  int n;                 // grid nodes
  int n_new;             // new abscissae
  const double *grid;    // [n] phases in cycles, or log10 energies
  const double *new_x;   // [n_new]
  const double *signal;  // [rows][n] (phase) or [n][rows] (energy)
  double shift;          // phase shift in cycles (phase)
  int allow_negative;    // (phase)
  double *out;           // [rows][n_new] (phase) or [n_new][rows] (energy)
};
void launch_phase_interpolator(const InterpArgs &a, cudaStream_t st);
void launch_energy_interpolator(const InterpArgs &a, cudaStream_t st);
void launch_phase_integrator(const PhaseIntArgs &a, cudaStream_t st);
void launch_poisson(int64_t n, const double *mean, double *out, uint64_t seed, uint64_t offset,
                    int32_t *fail, cudaStream_t st);
void launch_gaussian(int n_sets, int rows, int cols, const double *model,
                     int64_t model_set_stride, int64_t model_row_stride, const double *data,
                     const double *errors, double *loglike, cudaStream_t st);
int launch_elsewhere(const ElsewhereArgs &a, cudaStream_t st);

}  // namespace xg
