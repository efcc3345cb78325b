// integrator.cu -- K2+K3: the cell-mesh integrator for azimuthally invariant
// hot regions, replacing
// xpsi/cellmesh/integrator_for_azimuthal_invariance.pyx:70-665 with the
// blackbody (hot_BB.pyx:54-98) and numerical 4-D (hot_Num4D.pyx:248-461)
// atmospheres.
//
// Work decomposition (one CTA per chunk of consecutive parallels of one mesh):
//   1. leaf geometry, one thread per leaf pair (k, N_L-1-k): image deflection,
//      cos alpha / lag / d cos alpha from the Steffen ray tables, Doppler and
//      aberration factors (:342-441);
//   2. one thread runs the sequential visibility state machine that fills the
//      phase knots through invisible intervals (:480-549) and records, per
//      profile column, which leaf's radiation it carries (or zero);
//   3. per chunk of energies: the specific intensities of every column
//      (:445-478) -> Akima-periodic piece coefficients in shared memory
//      (:566-569) -> every (phase, cell) thread-task evaluates the piece once
//      per energy and accumulates A_ij * max(S, 0) (:571-598) in registers;
//   4. per-chunk partial sums are reduced in a fixed order and divided by
//      E keV (:605-612), so results are bitwise reproducible run to run.
//
// Num4D call history.  The reference evaluator keeps its stencil base node
// between calls and clamps an out-of-table cos(emission angle) only on the
// call that moves the node (hot_Num4D.pyx:300-351).  mu * eta exceeds the
// table's mu range on the approaching limb, so for such leaves the first
// energy is evaluated at the clamped mu = mu_max when the previously
// evaluated leaf sat below the table's third-to-last mu node, and every
// other energy extrapolates the last stencil.  The kernels reproduce the
// reference's single-thread call order exactly: a geometry pre-pass and a
// per-mesh scan hand each parallel the state its first evaluation sees.
#include <climits>
#include <type_traits>

#include "common.cuh"
#include "kernels.h"

namespace xg {

namespace {

constexpr int kThreads = 256;
constexpr int kEPT = 8;  // energies per accumulation task
constexpr int kMaxCellsF = 256;  // cells per parallel held as FP32 pairs in shared memory
constexpr int kMaxEnergiesF = 256;  // energies held in FP32 (mixed form)
constexpr int kStrip = 8;  // Akima pieces per thread, built from a sliding window of chords

// Akima piece of one energy row: value at the left knot and the three
// polynomial coefficients (FP64: 32 bytes, two 16-byte shared loads; FP32:
// one 16-byte load).
template <typename WT>
struct __align__(16) PieceT {
  WT y, k1, k2, k3;
};
using Piece = PieceT<double>;

struct RowCtx {
  int S1, N_R, J, IO;
  const double *D, *CA, *LG;  // ray tables of the row
  int jalt;                   // first ray with deflection > pi/2
  double radius, Grav_z, cos_gamma, sin_gamma, cos_th, sin_th, th_over_pi, beta, Lorentz;
  double maxDefl, cos_i, sin_i, inclination;
  double vec0, vec1;
};

struct GeoSmem {
  double *phase, *leafphase, *Z, *ABB, *GEOM;
  double *rD;  // the parallel's deflection table, staged for the binary searches
  int *src, *calc, *term, *clamp0;
  int *flags;  // [0] terminate, [1] invisible image, [2] any evaluation, [3] last_top
  double *lgE;  // [EC] log10 of the chunk's energies (FP64 path, Num4D)
  double *lzs;  // [N_L] log10(Z) + log10(E_eff) per leaf (FP64 path, Num4D)
  int *sc_exp;  // [EC] binary exponent of the largest |profile value| per energy row
  DF *ih, *ih2;  // [N_L] 1/h and 1/h^2 of the phase intervals (FP64 path)
  double *c2chi = nullptr, *s2chi = nullptr;  // [N_L] cos, sin of twice the polarisation
                                              // angle (Stokes kernel only)
};


// per-leaf geometry, integrator_for_azimuthal_invariance.pyx:342-441
__device__ void leaf_geometry(const RowCtx &c, int I, int k, int N_L, int leaf_lim,
                              const double *leaves, GeoSmem &g) {
  double cos_psi = c.cos_i * c.cos_th + c.sin_i * c.sin_th * cos(leaves[k]);
  double psi = image_deflection(I, acos(cos_psi));
  double sin_psi = sin(psi);
  if (!are_equal(psi, 0.0) && are_equal(sin_psi, 0.0)) {
    double _i = (c.cos_i >= 0.0) ? c.inclination + c.inclination * 1.0e-6
                                 : c.inclination - c.inclination * 1.0e-6;
    cos_psi = cos(_i) * c.cos_th + sin(_i) * c.sin_th * cos(leaves[k]);
    psi = image_deflection(I, acos(cos_psi));
    sin_psi = sin(psi);
  }
  const int N_R = c.N_R;
  MainX mx{c.D};
  AltX ax{c.D, c.jalt};
  AltY ay{c.CA, c.jalt};
  const double alt_xmin = cos(c.D[c.jalt]);
  int calc = 0, term = 0;
  double sin_alpha = 0.0, mu = 0.0, cos_a;
  if (psi <= c.maxDefl) {
    if (psi < c.D[0] || psi > c.D[N_R - 1]) {
      term = 1;
    } else {
      if (psi <= kHalfPi && cos_psi >= alt_xmin)
        steffen_eval(ax, ay, c.jalt + 1, cos_psi, &cos_a, nullptr);
      else
        steffen_eval(mx, ArrY{c.CA}, N_R, psi, &cos_a, nullptr);
      sin_alpha = sqrt(1.0 - cos_a * cos_a);
      mu = cos_a * c.cos_gamma;
      if (!are_equal(psi, 0.0)) {
        double cos_delta = (c.cos_i - c.cos_th * cos_psi) / (c.sin_th * sin_psi);
        if (c.th_over_pi < 0.5) mu = mu + sin_alpha * c.sin_gamma * cos_delta;
        else mu = mu - sin_alpha * c.sin_gamma * cos_delta;
      }
      calc = (mu > 0.0) ? 1 : 0;
    }
  }
  if (calc && !term) {
    double deriv;
    if (psi <= kHalfPi && cos_psi >= alt_xmin) {
      steffen_eval(ax, ay, c.jalt + 1, cos_psi, nullptr, &deriv);
    } else {
      steffen_eval(mx, ArrY{c.CA}, N_R, psi, nullptr, &deriv);
      // the reference's exp(log|deriv| - log|sin psi|), as the quotient
      // (the same zero, infinite and NaN cases; an ulp apart)
      deriv = fabs(deriv) / fabs(sin_psi);
    }
    double plag;
    steffen_eval(mx, ArrY{c.LG}, N_R, psi, &plag, nullptr);
    for (int ks = 0; ks < 2; ks++) {
      if ((0 < k && k < leaf_lim - 1) || (k == 0 && ks == 0) ||
          (k == leaf_lim - 1 && N_L % 2 == 1 && ks == 0) ||
          (k == leaf_lim - 1 && N_L % 2 == 0)) {
        int kdx = (ks == 0) ? k : N_L - 1 - k;
        double superlum, eta, cos_xi = 0.0;
        if (!are_equal(psi, 0.0)) {
          cos_xi = sin_alpha * c.sin_i * sin(leaves[kdx]) / sin_psi;
          superlum = 1.0 + c.beta * cos_xi;
          eta = c.Lorentz / superlum;
        } else {
          superlum = 1.0;
          eta = c.Lorentz;
        }
        g.Z[kdx] = eta * c.Grav_z;
        g.ABB[kdx] = mu * eta;
        g.GEOM[kdx] = mu * fabs(deriv) * c.Grav_z * eta * eta * eta / superlum;
        g.leafphase[kdx] = leaves[kdx] + plag;
        if (g.c2chi) {  // integratorIQU_for_azimuthal_invariance.pyx:463-466
          const double chi = pol_angle(leaves[kdx], sin_psi, cos_psi, sin_alpha, cos_a, c.sin_th,
                                       c.cos_th, c.sin_i, c.cos_i, c.sin_gamma, c.cos_gamma,
                                       c.Grav_z, mu, eta, c.beta, c.Lorentz, cos_xi);
          g.c2chi[kdx] = cos(2 * chi);
          g.s2chi[kdx] = sin(2 * chi);
        }
      }
    }
  }
  g.calc[k] = calc;
  g.term[k] = term;
}

// sequential visibility state machine, :480-563.  Runs on one thread.
// Returns through g.flags: [0] terminate, [1] no visibility in this image.
// Tracks the Num4D call-history flag `top` (last evaluated mu*eta above the
// table's third-to-last mu node) and marks columns whose first energy sees a
// clamped mu.
__device__ void state_machine(int N_L, int leaf_lim, const double *leaves, GeoSmem &g,
                              bool num4d, double mu_top3, double mu_max, int &top,
                              int &any_eval) {
  int InvisFlag = 2, InvisPhase = 0;
  double step;
  int term = 0;
  for (int m = 0; m < N_L; m++) g.src[m] = -1;
  for (int k = 0; k < leaf_lim; k++) {
    if (g.term[k]) { term = 1; break; }
    if (g.calc[k]) {
      for (int ks = 0; ks < 2; ks++) {
        if ((0 < k && k < leaf_lim - 1) || (k == 0 && ks == 0) ||
            (k == leaf_lim - 1 && N_L % 2 == 1 && ks == 0) ||
            (k == leaf_lim - 1 && N_L % 2 == 0)) {
          int kdx = (ks == 0) ? k : N_L - 1 - k;
          // the reference writes the knot when it reaches this leaf (:441);
          // earlier gap fills may have passed over this position
          g.phase[kdx] = g.leafphase[kdx];
          g.src[kdx] = kdx;
          if (num4d) {
            double a = g.ABB[kdx];
            g.clamp0[kdx] = (a > mu_max && !top) ? 1 : 0;
            top = (a > mu_top3) ? 1 : 0;
          }
          any_eval = 1;
        }
      }
      if (k == 0) {
        g.phase[N_L - 1] = g.phase[0] + kTwoPi;
        g.src[N_L - 1] = g.src[0];
      } else if (k > 0 && InvisFlag == 2) {
        step = leaves[k] / (double)k;
        for (int m = N_L - k; m < N_L; m++) g.phase[m] = g.phase[m - 1] + step;
        for (int m = N_L - k; m < N_L; m++) g.src[m] = -1;
        g.phase[0] = g.phase[N_L - 1] - kTwoPi;
        for (int m = 1; m < k; m++) g.phase[m] = g.phase[m - 1] + step;
        g.src[0] = -1;
        for (int m = 1; m < k; m++) g.src[m] = -1;
      } else if (InvisFlag == 1) {
        step = g.phase[k] - g.phase[InvisPhase - 1];
        step = step / (double)(k - InvisPhase + 1);
        for (int m = InvisPhase; m < k; m++) g.phase[m] = g.phase[m - 1] + step;
        step = g.phase[N_L - InvisPhase] - g.phase[N_L - 1 - k];
        step = step / (double)(k - InvisPhase + 1);
        for (int m = N_L - k; m < N_L - InvisPhase; m++) g.phase[m] = g.phase[m - 1] + step;
      }
      InvisFlag = 0;
    } else {
      if (InvisFlag == 0) {
        step = g.phase[N_L - k] - g.phase[k - 1];
        step = step / (double)(N_L - 2 * k + 1);
        for (int m = k; m < N_L - k; m++) g.phase[m] = g.phase[m - 1] + step;
        for (int m = k; m < N_L - k; m++) g.src[m] = -1;
        InvisFlag = 1;
        InvisPhase = k;
      }
    }
  }
  int invis = 0;
  if (!term) {
    if (InvisFlag == 2) {
      invis = 1;
    } else {
      for (int m = 1; m < N_L; m++)
        if (g.phase[m] <= g.phase[m - 1]) { term = 1; break; }
    }
  }
  g.flags[0] = term;
  g.flags[1] = invis;
}

__device__ bool load_row(const IntegrateArgs &a, const MemberDesc &M, int64_t row, int i,
                         RowCtx &c, int *s_J) {
  // first radiating cell of the parallel (:286-296), found by the first warp
  const int32_t *rad = a.radiates + M.cell_off + (int64_t)i * M.S1;
  if (threadIdx.x < 32) {
    int best = M.S1;
    for (int j = threadIdx.x; j < M.S1; j += 32)
      if (rad[j] == 1) { best = min(best, j); break; }
    for (int o = 16; o > 0; o >>= 1) best = min(best, __shfl_xor_sync(0xffffffffu, best, o));
    if (threadIdx.x == 0) *s_J = best;
  }
  __syncthreads();
  int J = *s_J;
  __syncthreads();
  if (J >= M.S1) return false;
  c.S1 = M.S1;
  c.N_R = a.N_R;
  c.J = J;
  c.D = a.deflection + row * a.N_R;
  c.CA = a.cos_alpha + row * a.N_R;
  c.LG = a.lag + row * a.N_R;
  c.jalt = a.N_R - 1;  // set by stage_deflection()
  c.radius = a.radius[row];
  c.Grav_z = sqrt(1.0 - a.u[row]);
  c.cos_gamma = a.cos_gamma[row];
  c.sin_gamma = sqrt(1.0 - c.cos_gamma * c.cos_gamma);
  double th = a.theta0[row];
  c.cos_th = cos(th);
  c.sin_th = sin(th);
  c.th_over_pi = th / kPi;
  c.beta = c.radius * M.omega * c.sin_th / (kC * c.Grav_z);
  c.Lorentz = sqrt(1.0 - c.beta * c.beta);
  c.maxDefl = a.maxDeflection[row];
  c.inclination = M.inclination;
  c.cos_i = cos(M.inclination);
  c.sin_i = sin(M.inclination);
  c.IO = M.image_order_limit > 0 ? M.image_order_limit : (int)ceil(c.maxDefl / kPi);
  const double *vec = a.params + (M.cell_off + (int64_t)i * M.S1 + J) * a.n_params;
  c.vec0 = vec[0];
  c.vec1 = vec[1];
  return true;
}

// Copy the parallel's deflection table to shared memory (the leaf searches
// probe it ~10 times per lookup) and find the first ray deflected beyond
// pi/2 (:301-303; the reference's scan is unbounded, here it stops at the
// last ray).  All threads of the CTA call it.
__device__ void stage_deflection(RowCtx &c, GeoSmem &g, int *s_jalt) {
  const int N_R = c.N_R;
  for (int t = threadIdx.x; t < N_R; t += blockDim.x) g.rD[t] = c.D[t];
  if (threadIdx.x == 0) *s_jalt = N_R - 1;
  __syncthreads();
  for (int t = threadIdx.x; t < N_R - 1; t += blockDim.x)
    if (g.rD[t] > kHalfPi) atomicMin(s_jalt, t);
  __syncthreads();
  c.jalt = *s_jalt;
  c.D = g.rD;
  __syncthreads();
}



struct AtmSmem {
  double *gmu, *gE;      // grids of mu and log10(E/kT)
  double *smu, *sE;      // inverse Lagrange denominators per stencil base, 4 each
  float *fgmu, *fgE, *fsmu, *fsE;  // FP32 copies for the mixed-precision form
  float *fgEo;           // [3 nE] offsets gE[b + i] - gE[b], i = 1..3 (mixed form)
  // FP64 form with a contracted 4-D table: the offsets gE[b + i] - gE[b]
  // (i = 1..3) and the inverse Lagrange denominators of the energy grid as
  // double-float pairs (in the space of the mixed form's FP32 arrays and of sE)
  DF *dgEo, *dsE;
  int *xe;               // [nE] binary exponent of each energy column of the slab
  float *fphase;         // FP32 copy of the phase knots
  float *fphase_lo;      // phase knot minus its FP32 copy
  float *fcphi, *fcphi_lo;  // cell azimuths of the parallel as float pairs (<= kMaxCellsF)
  float *fcarea, *fcarea_lo;  // cell areas of the parallel as float pairs (<= kMaxCellsF)
  float *finvZ, *fabb, *fgeom;  // per profile column: 1/Z, mu eta, geometric factor
  float *fE;                // energies
};

// inverse denominators of the 4-point Lagrange basis on grid[b..b+3]
// (hot_Num4D.pyx:177-188, computed in the reference's order)
__device__ __forceinline__ void lagrange_space(const double *P, int b, double s[4]) {
  double s0 = 1.0 / (P[b] - P[b + 1]); s0 /= P[b] - P[b + 2]; s0 /= P[b] - P[b + 3];
  double s1 = 1.0 / (P[b + 1] - P[b]); s1 /= P[b + 1] - P[b + 2]; s1 /= P[b + 1] - P[b + 3];
  double s2 = 1.0 / (P[b + 2] - P[b]); s2 /= P[b + 2] - P[b + 1]; s2 /= P[b + 2] - P[b + 3];
  double s3 = 1.0 / (P[b + 3] - P[b]); s3 /= P[b + 3] - P[b + 1]; s3 /= P[b + 3] - P[b + 2];
  s[0] = s0; s[1] = s1; s[2] = s2; s[3] = s3;
}

__device__ __forceinline__ void lagrange_w(const double *P, const double *S, int b, double x,
                                           double w[4]) {
  double d0 = (x - P[b + 1]) * (x - P[b + 2]) * (x - P[b + 3]);
  double d1 = (x - P[b]) * (x - P[b + 2]) * (x - P[b + 3]);
  double d2 = (x - P[b]) * (x - P[b + 1]) * (x - P[b + 3]);
  double d3 = (x - P[b]) * (x - P[b + 1]) * (x - P[b + 2]);
  w[0] = d0 * S[4 * b]; w[1] = d1 * S[4 * b + 1]; w[2] = d2 * S[4 * b + 2];
  w[3] = d3 * S[4 * b + 3];
}

// the table grids of a numerical atmosphere in shared memory: mu and E
// nodes, the inverse Lagrange denominators of every stencil base, and the
// FP32 copies the guided stencil searches use; ends with a block barrier
__device__ __forceinline__ void stage_table_grids(const Atmos4D &A, AtmSmem &as, int nmu,
                                                  int nEt) {
  for (int t = threadIdx.x; t < nmu; t += blockDim.x) as.gmu[t] = A.mu[t];
  for (int t = threadIdx.x; t < nEt; t += blockDim.x) as.gE[t] = A.logE[t];
  __syncthreads();
  for (int b = threadIdx.x; b <= nmu - 4; b += blockDim.x) lagrange_space(as.gmu, b, as.smu + 4 * b);
  for (int b = threadIdx.x; b <= nEt - 4; b += blockDim.x) lagrange_space(as.gE, b, as.sE + 4 * b);
  for (int t = threadIdx.x; t < nmu; t += blockDim.x) as.fgmu[t] = (float)as.gmu[t];
  for (int t = threadIdx.x; t < nEt; t += blockDim.x) as.fgE[t] = (float)as.gE[t];
  __syncthreads();
}

// stencil_base with the bisection run on the grid's FP32 copy (FP32 pipe)
// and finished with FP64 comparisons.  Rounding to float is monotone, so the
// float search never stops below the FP64 answer, and stepping down while
// g[lo] > v lands on it exactly: the result equals stencil_base(g, n, v).
__device__ __forceinline__ int stencil_base_guided(const double *g, const float *fg, int n,
                                                   double v) {
  const float vf = (float)v;
  int lo = 0, hi = n - 1;
  while (hi > lo + 1) {
    const int mid = (lo + hi) >> 1;
    if (fg[mid] > vf) hi = mid; else lo = mid;
  }
  while (lo > 0 && g[lo] > v) lo--;
  int b = lo - 1;
  if (b < 0) b = 0;
  if (b > n - 4) b = n - 4;
  return b;
}

// Num4D intensity for a parallel whose (log T, log g) stencil has been
// contracted into `slab` [nmu][nE]: the remaining 4 x 4 (mu, energy) stencil
// (hot_Num4D.pyx:248-439; the stencil bases are those the reference's cached
// walk lands on, see the file header for the mu > 1 case).  It is split in
// two: the mu stencil depends only on the profile column (its cos emission
// angle), so a thread evaluating one column at several energies forms it
// once.  The caller passes v3 = log10(E / E_eff) as log10 E - log10 Z -
// log10 E_eff from per-energy and per-leaf logarithms.
struct MuStencil {
  int b2;
  double w2[4];
};
__device__ __forceinline__ MuStencil mu_stencil(const Atmos4D &A, const AtmSmem &as, double mu,
                                                bool clamp_mu) {
  double v2 = mu;
  const double mu_hi = as.gmu[A.nmu - 1];
  if (v2 > mu_hi && clamp_mu) v2 = mu_hi;
  if (v2 < as.gmu[0]) v2 = as.gmu[0];
  MuStencil m;
  m.b2 = stencil_base_guided(as.gmu, as.fgmu, A.nmu, v2);
  lagrange_w(as.gmu, as.smu, m.b2, v2, m.w2);
  return m;
}
// the stencil sum itself (a Stokes Q table: no positive part, no factor)
__device__ __forceinline__ double eval_table_raw(const Atmos4D &A, const AtmSmem &as,
                                                 const double *slab, const MuStencil &m,
                                                 double v3) {
  if (v3 < as.gE[0]) v3 = as.gE[0];
  if (v3 > as.gE[A.nE - 1]) v3 = as.gE[A.nE - 1];
  const int b3 = stencil_base_guided(as.gE, as.fgE, A.nE, v3);
  double w3[4];
  lagrange_w(as.gE, as.sE, b3, v3, w3);
  double I = 0.0;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const double *r = slab + (size_t)(m.b2 + k) * A.nE + b3;
    const double t = w3[0] * r[0] + w3[1] * r[1] + w3[2] * r[2] + w3[3] * r[3];
    I += m.w2[k] * t;
  }
  return I;
}
__device__ __forceinline__ double eval_num4d_e(const Atmos4D &A, const AtmSmem &as,
                                               const double *slab, const MuStencil &m,
                                               double v3, double p3) {
  if (v3 < as.gE[0]) v3 = as.gE[0];
  if (v3 > as.gE[A.nE - 1]) v3 = as.gE[A.nE - 1];
  const int b3 = stencil_base_guided(as.gE, as.fgE, A.nE, v3);
  double w3[4];
  lagrange_w(as.gE, as.sE, b3, v3, w3);
  double I = 0.0;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const double *r = slab + (size_t)(m.b2 + k) * A.nE + b3;
    const double t = w3[0] * r[0] + w3[1] * r[1] + w3[2] * r[2] + w3[3] * r[3];
    I += m.w2[k] * t;
  }
  if (I < 0.0) return 0.0;
  return I * p3;
}

// a double-float pair times 2^d, d <= 0 (exact down to the float range)
__device__ __forceinline__ DF df_scale(DF a, int d) {
  if (d < -125) return DF{0.0f, 0.0f};
  const float f = __int_as_float((127 + d) << 23);
  return DF{a.h * f, a.l * f};
}

// Num4D intensity of the FP64 form from a slab held as double-float pairs
// whose energy-node columns are scaled by 2^-xe: the same stencils as
// eval_num4d_e, with the energy coordinate's offset from the stencil base
// formed in FP64 (as the reference's differences) and the Lagrange products
// and the 4 x 4 contraction in double-float arithmetic (~2^-48 relative, on
// the FP32 pipes).  The float pre-tests leave the FP64 comparisons to the
// grid's ends and to ties of the rounded coordinate.  Returns the stencil
// sum before the positive part (the caller clamps it at 0), in units of
// `scale` (the largest of the four nodes' column scales).
struct MuStencilDF {
  int b2;
  DF w2[4];
};
__device__ __forceinline__ MuStencilDF mu_stencil_df(const Atmos4D &A, const AtmSmem &as,
                                                     double mu, bool clamp_mu) {
  const MuStencil m = mu_stencil(A, as, mu, clamp_mu);
  MuStencilDF d;
  d.b2 = m.b2;
#pragma unroll
  for (int k = 0; k < 4; k++) d.w2[k] = df_split(m.w2[k]);
  return d;
}
// the contracted table's value at (mu stencil m, v3) as a double-float times
// 2^xr (xr the largest column exponent of the energy stencil)
__device__ __forceinline__ DF eval_num4d_dfx(const Atmos4D &A, const AtmSmem &as, const DF *slab,
                                             const MuStencilDF &m, double v3, int &xr) {
  const int nE = A.nE;
  float vf = (float)v3;
  if (vf <= as.fgE[0] && v3 < as.gE[0]) {
    v3 = as.gE[0];
    vf = as.fgE[0];
  }
  if (vf >= as.fgE[nE - 1] && v3 > as.gE[nE - 1]) {
    v3 = as.gE[nE - 1];
    vf = as.fgE[nE - 1];
  }
  // stencil_base_guided with the FP64 step-down tested only where the
  // rounded node does not lie below the rounded coordinate (g > v implies
  // fg >= vf, rounding being monotone)
  int lo = 0, hi = nE - 1;
  while (hi > lo + 1) {
    const int mid = (lo + hi) >> 1;
    if (as.fgE[mid] > vf) hi = mid; else lo = mid;
  }
  while (lo > 0 && as.fgE[lo] >= vf && as.gE[lo] > v3) lo--;
  int b3 = lo - 1;
  if (b3 < 0) b3 = 0;
  if (b3 > nE - 4) b3 = nE - 4;
  const DF u0 = df_split(v3 - as.gE[b3]);
  const DF *o = as.dgEo + 3 * b3;
  const DF u1 = df_sub(u0, o[0]), u2 = df_sub(u0, o[1]), u3 = df_sub(u0, o[2]);
  const DF u01 = df_mul(u0, u1), u23 = df_mul(u2, u3);
  const DF *S = as.dsE + 4 * b3;
  // the nodes' column scales relative to the largest of the four (<= 1)
  const int x0 = as.xe[b3], x1 = as.xe[b3 + 1], x2 = as.xe[b3 + 2], x3 = as.xe[b3 + 3];
  xr = max(max(x0, x1), max(x2, x3));
  const DF w3[4] = {df_scale(df_mul(df_mul(u1, u23), S[0]), x0 - xr),
                    df_scale(df_mul(df_mul(u0, u23), S[1]), x1 - xr),
                    df_scale(df_mul(df_mul(u01, u3), S[2]), x2 - xr),
                    df_scale(df_mul(df_mul(u01, u2), S[3]), x3 - xr)};
  float sh = 0.0f, sl = 0.0f;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const DF *r = slab + (size_t)(m.b2 + k) * nE + b3;
    float th = 0.0f, tl = 0.0f;
#pragma unroll
    for (int i = 0; i < 4; i++) df_acc_mul(w3[i], r[i], th, tl);
    df_acc_mul(m.w2[k], df_norm(th, tl), sh, sl);
  }
  return df_norm(sh, sl);
}
// the same with the factor 2^xr returned as a double
__device__ __forceinline__ DF eval_num4d_df(const Atmos4D &A, const AtmSmem &as, const DF *slab,
                                            const MuStencilDF &m, double v3, double &scale) {
  int xr;
  const DF v = eval_num4d_dfx(A, as, slab, m, v3, xr);
  scale = pow2_double(xr);
  return v;
}
// binary exponent x of |f| = m 2^x, m in [0.5, 1), of a nonzero finite float
// from its bit pattern
__device__ __forceinline__ int float_exponent(float f) {
  const int b = (__float_as_int(f) >> 23) & 0xff;
  return b != 0 ? b - 126 : -149 + (32 - __clz(__float_as_int(f) & 0x7fffff));
}
// a double-float times 2^d (0 where 2^d leaves the float range)
__device__ __forceinline__ DF df_times_pow2(DF a, int d) {
  if (d < -126 || d > 127) return DF{0.0f, 0.0f};
  const float f = __int_as_float((127 + d) << 23);
  return DF{a.h * f, a.l * f};
}

// FP32 forms for the mixed-precision integrator

// an Akima piece in double-float form, scaled by a power of two per energy
// row (same 32 bytes as the FP64 piece it replaces in shared memory)
struct __align__(16) PieceDF {
  DF y, k1, k2, k3;
};
__device__ __forceinline__ int stencil_base_f(const float *g, int n, float v) {
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

__device__ __forceinline__ void lagrange_wf(const float *P, const float *S, int b, float x,
                                            float w[4]) {
  float d0 = (x - P[b + 1]) * (x - P[b + 2]) * (x - P[b + 3]);
  float d1 = (x - P[b]) * (x - P[b + 2]) * (x - P[b + 3]);
  float d2 = (x - P[b]) * (x - P[b + 1]) * (x - P[b + 3]);
  float d3 = (x - P[b]) * (x - P[b + 1]) * (x - P[b + 2]);
  w[0] = d0 * S[4 * b]; w[1] = d1 * S[4 * b + 1]; w[2] = d2 * S[4 * b + 2];
  w[3] = d3 * S[4 * b + 3];
}

// Num4D intensity in the mixed form: the slab and the Lagrange weights in
// FP32, the mu stencil formed once per profile column; the energy
// coordinate v3 = log10 E - log10 Z - log10 E_eff and its offset from the
// stencil base in FP64, so the weights see the FP32 rounding of an offset of
// a few grid spacings (~1e-9 absolute) rather than that of the coordinate
// (~3e-8, the same on every evaluation of a parallel: a systematic shift).
struct MuStencilF {
  int b2;
  float w2[4];
};
__device__ __forceinline__ MuStencilF mu_stencil_f(const Atmos4D &A, const AtmSmem &as, float mu,
                                                   bool clamp_mu) {
  float v2 = mu;
  const float mu_hi = as.fgmu[A.nmu - 1];
  if (v2 > mu_hi && clamp_mu) v2 = mu_hi;
  if (v2 < as.fgmu[0]) v2 = as.fgmu[0];
  MuStencilF m;
  m.b2 = stencil_base_f(as.fgmu, A.nmu, v2);
  lagrange_wf(as.fgmu, as.fsmu, m.b2, v2, m.w2);
  return m;
}
__device__ __forceinline__ float eval_num4d_f(const Atmos4D &A, const AtmSmem &as,
                                              const float *slab, const MuStencilF &m, double v3,
                                              float p3) {
  if (v3 < as.gE[0]) v3 = as.gE[0];
  if (v3 > as.gE[A.nE - 1]) v3 = as.gE[A.nE - 1];
  const int b3 = stencil_base_guided(as.gE, as.fgE, A.nE, v3);
  const float u = (float)(v3 - as.gE[b3]);
  const float *o = as.fgEo + 3 * b3;  // node offsets gE[b3 + i] - gE[b3], i = 1..3
  const float d0 = u, d1 = u - o[0], d2 = u - o[1], d3 = u - o[2];
  const float *S = as.fsE + 4 * b3;
  const float w3[4] = {d1 * d2 * d3 * S[0], d0 * d2 * d3 * S[1], d0 * d1 * d3 * S[2],
                       d0 * d1 * d2 * S[3]};
  float I = 0.0f;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const float *r = slab + (size_t)(m.b2 + k) * A.nE + b3;
    const float t = w3[0] * r[0] + w3[1] * r[1] + w3[2] * r[2] + w3[3] * r[3];
    I += m.w2[k] * t;
  }
  if (I < 0.0f) return 0.0f;
  return I * p3;
}

__device__ __forceinline__ float eval_bb_f(float E, float kT) {
  return E * E * E / expm1f(E / kT);
}

struct Layout {
  int N_L, EC, nmu, nE;
  size_t bytes;
};

// nmu, nE: Num4D grid sizes (0 when no mesh uses the numerical atmosphere)
__host__ __device__ inline Layout make_layout(int N_L, int N_P, int N_E, int nmu = 0,
                                              int nE = 0, int piece_bytes = 32, int N_R = 0) {
  Layout L;
  L.N_L = N_L;
  L.nmu = nmu;
  L.nE = nE;
  int ec = 8;
  while (ec < 32 && (long)N_P * (ec * 2 / kEPT) <= kThreads && ec * 2 <= N_E + kEPT) ec *= 2;
  while (ec > 8 && (size_t)ec * N_L * piece_bytes > 96 * 1024) ec /= 2;
  L.EC = ec;
  L.bytes = (size_t)5 * N_L * sizeof(double)      // phase, leafphase, Z, ABB, GEOM
            + (size_t)ec * N_L * piece_bytes       // coefficients
            + (size_t)(nmu + nE) * 5 * sizeof(double)  // Num4D grids + inverse denominators
            + (size_t)(nmu + nE) * 5 * sizeof(float)   // their FP32 copies (mixed form)
            + (size_t)3 * nE * sizeof(float)           // energy-grid node offsets (mixed)
            + (size_t)nE * sizeof(int)                 // slab column exponents (FP64 form)
            + (size_t)(5 * N_L + 4 * kMaxCellsF + kMaxEnergiesF) * sizeof(float)
            + (size_t)N_R * sizeof(double)  // staged deflection table
            + (size_t)(ec + N_L) * sizeof(double)  // lgE, lzs
            + (size_t)2 * N_L * sizeof(DF)         // ih, ih2
            + (size_t)(4 * N_L + 8 + ec) * sizeof(int) + 64;
  return L;
}

// bytes carve() takes with no coefficients and no atmosphere arrays (the
// Num4D pre-pass)
inline size_t geometry_bytes(int N_L, int N_R) {
  return (size_t)N_R * sizeof(double) + (size_t)8 * N_L * sizeof(double) + 16 /* alignment */ +
         (size_t)(4 * N_L + 8) * sizeof(int) + 16;
}

__device__ GeoSmem carve(char *base, int N_L, int EC, double **coef, int nmu = 0, int nE = 0,
                         AtmSmem *atm = nullptr, int piece_bytes = 32, int N_R = 0) {
  GeoSmem g;
  double *d = reinterpret_cast<double *>(base);
  g.rD = d; d += N_R;
  g.phase = d; d += N_L;
  g.leafphase = d; d += N_L;
  g.Z = d; d += N_L;
  g.ABB = d; d += N_L;
  g.GEOM = d; d += N_L;
  g.lzs = d; d += N_L;
  g.lgE = d; d += EC;
  g.ih = reinterpret_cast<DF *>(d); d += N_L;
  g.ih2 = reinterpret_cast<DF *>(d); d += N_L;
  d = reinterpret_cast<double *>((reinterpret_cast<uintptr_t>(d) + 15) & ~uintptr_t(15));
  *coef = d; d += (size_t)EC * N_L * piece_bytes / 8;
  if (atm) {
    atm->gmu = d; d += nmu;
    atm->gE = d; d += nE;
    atm->smu = d; d += (size_t)4 * nmu;
    atm->sE = d; d += (size_t)4 * nE;
    float *f = reinterpret_cast<float *>(d);
    atm->fgmu = f; f += nmu;
    atm->fgE = f; f += nE;
    atm->fsmu = f; f += (size_t)4 * nmu;
    atm->fsE = f; f += (size_t)4 * nE;
    atm->fgEo = f; f += (size_t)3 * nE;
    // the FP64 form's double-float energy-grid data reuse the mixed form's
    // FP32 arrays (fsmu .. fgEo: 4 nmu + 7 nE floats >= 6 nE + 1) and sE
    atm->dgEo = reinterpret_cast<DF *>((reinterpret_cast<uintptr_t>(atm->fsmu) + 7) &
                                       ~uintptr_t(7));
    atm->dsE = reinterpret_cast<DF *>(atm->sE);
    atm->fphase = f; f += N_L;
    atm->fphase_lo = f; f += N_L;
    atm->fcphi = f; f += kMaxCellsF;
    atm->fcphi_lo = f; f += kMaxCellsF;
    atm->fcarea = f; f += kMaxCellsF;
    atm->fcarea_lo = f; f += kMaxCellsF;
    atm->finvZ = f; f += N_L;
    atm->fabb = f; f += N_L;
    atm->fgeom = f; f += N_L;
    atm->fE = f; f += kMaxEnergiesF;
    atm->xe = reinterpret_cast<int *>(f); f += nE;
    d = reinterpret_cast<double *>((reinterpret_cast<uintptr_t>(f) + 15) & ~uintptr_t(15));
  }
  int *ip = reinterpret_cast<int *>(d);
  g.src = ip; ip += N_L;
  g.calc = ip; ip += N_L;
  g.term = ip; ip += N_L;
  g.clamp0 = ip; ip += N_L;
  g.flags = ip; ip += 8;
  g.sc_exp = ip;
  return g;
}

// ---------------------------------------------------------------------------
// Pre-pass for Num4D: per parallel, does it evaluate the atmosphere, and does
// its last evaluation leave the mu stencil at the top of the table?
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) num4d_prepass_kernel(IntegrateArgs a) {
  extern __shared__ __align__(16) char smem[];
  const int64_t row = blockIdx.x;
  const int m = a.row_member[row];
  const MemberDesc M = a.members[m];
  const int i = (int)(row - M.row_off);
  const int N_L = a.N_L;
  const int leaf_lim = (N_L % 2 == 0) ? N_L / 2 : (N_L + 1) / 2;
  double *coef;
  GeoSmem g = carve(smem, N_L, 0, &coef, 0, 0, nullptr, 32, a.N_R);
  __shared__ int s_J, s_any, s_top, s_jalt;
  RowCtx c;
  if (threadIdx.x == 0) { s_any = 0; s_top = 0; }
  if (!load_row(a, M, row, i, c, &s_J)) {
    if (threadIdx.x == 0) { a.row_has_eval[row] = 0; a.row_last_top[row] = 0; }
    return;
  }
  stage_deflection(c, g, &s_jalt);
  const double mu_max = a.atmos.mu[a.atmos.nmu - 1], mu_top3 = a.atmos.mu[a.atmos.nmu - 3];
  for (int I = 0; I < c.IO; I++) {
    for (int k = threadIdx.x; k < leaf_lim; k += blockDim.x)
      leaf_geometry(c, I, k, N_L, leaf_lim, a.leaves, g);
    __syncthreads();
    if (threadIdx.x == 0) {
      int top = s_top, any = s_any;
      state_machine(N_L, leaf_lim, a.leaves, g, true, mu_top3, mu_max, top, any);
      s_top = top;
      s_any = any;
    }
    __syncthreads();
    int stop = g.flags[0] | g.flags[1];
    __syncthreads();
    if (stop) break;
  }
  if (threadIdx.x == 0) {
    a.row_has_eval[row] = (uint8_t)s_any;
    a.row_last_top[row] = (uint8_t)s_top;
  }
}

// serial over the parallels of each mesh, in the reference's call order
__global__ void num4d_scan_kernel(IntegrateArgs a) {
  int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= a.n_members) return;
  const MemberDesc M = a.members[m];
  if (M.atm != 2 && M.atm != 4 && M.atm != 6) return;
  uint8_t carry = 0;
  for (int i = 0; i < M.S0; i++) {
    int64_t row = M.row_off + i;
    a.row_entry_top[row] = carry;
    if (a.row_has_eval[row]) carry = a.row_last_top[row];
  }
}

// ---------------------------------------------------------------------------
// Cell x phase sums (:571-598).  A task is one signal phase and kEPT energies
// of the current chunk; it walks the radiating cells of the parallel in
// azimuth order, so a cell's interval is found by stepping forward from the
// previous cell's (one or two knot comparisons) rather than by bisection, and
// each (cell, energy) costs the piece's Horner form plus one FMA.
// ---------------------------------------------------------------------------
constexpr int kWrapLimit = 1024;  // 2 pi shifts of a cell phase (a few suffice)

// the phase of cell j at a signal phase, wrapped into the knot range
// (:575-586), with phases as unevaluated float pairs (hi + lo) and error-free
// sums, so the offset t keeps ~1e-14 rad absolute accuracy instead of one
// FP32 ulp of the phase (~5e-7 rad)
struct CellPhaseF {
  const float *knot, *knot_lo;
  int N_L;
  float x_lo, x_hi, ph, ph_lo, tp, tp_lo;
  const float *cphi, *cphi_lo;  // cached pairs, or null
  const double *cphi_d;
  // interval and offset th + tl of cell j's phase
  __device__ __forceinline__ int offset(int j, int hint, float &th, float &tl) const {
    float cp, cp_lo;
    if (cphi) {
      cp = cphi[j];
      cp_lo = cphi_lo[j];
    } else {
      const double c = cphi_d[j];
      cp = (float)c;
      cp_lo = (float)(c - (double)cp);
    }
    float x, lo;
    two_sum(ph, cp, x, lo);
    lo += ph_lo + cp_lo;
    if (x > x_hi) {
      for (int w = 0; x > x_hi && w < kWrapLimit; w++) {
        float e;
        two_sum(x, -tp, x, e);
        lo += e - tp_lo;
      }
    } else if (x < x_lo) {
      for (int w = 0; x < x_lo && w < kWrapLimit; w++) {
        float e;
        two_sum(x, tp, x, e);
        lo += e + tp_lo;
      }
    }
    if (!(x >= x_lo && x <= x_hi)) return -1;
    int iv = hint;
    if (iv < 0 || knot[iv] > x) iv = locate(knot, N_L, x);
    else
      while (iv < N_L - 2 && knot[iv + 1] <= x) iv++;
    float e3;
    two_sum(x, -knot[iv], th, e3);
    tl = e3 + lo - knot_lo[iv];
    return iv;
  }
  __device__ __forceinline__ int operator()(int j, int hint, float &t) const {
    float th, tl;
    const int iv = offset(j, hint, th, tl);
    t = th + tl;
    return iv;
  }
  __device__ __forceinline__ int operator()(int j, int hint, DF &t) const {
    float th, tl;
    const int iv = offset(j, hint, th, tl);
    t = fast_two_sum(th, tl);
    return iv;
  }
};

struct AreaF {
  const float *Af;  // cached, or null
  const double *A;
  __device__ __forceinline__ float operator()(int j) const { return Af ? Af[j] : (float)A[j]; }
};
struct AreaDF {
  const float *Ah, *Al;  // cached pairs, or null
  const double *A;
  __device__ __forceinline__ DF operator()(int j) const {
    return Ah ? DF{Ah[j], Al[j]} : df_split(A[j]);
  }
};

// the reference adds an interpolant value when it is > 0 (:593-594)
__device__ __forceinline__ bool positive(float v) { return v > 0.0f; }

// sums over the radiating cells of one parallel at one signal phase for the
// energies pb .. pb+kEPT-1 of the chunk; false when a cell phase cannot be
// wrapped into the knot range (the reference's terminate)
template <typename WT, typename CP, typename AR>
__device__ __forceinline__ bool cell_phase_sums(const CP &cp, const AR &area, int S1,
                                                const int32_t *rad, const PieceT<WT> *co4,
                                                int N_L, int pb, int ne, WT (&acc)[kEPT]) {
  int hint = -1;
  for (int j = 0; j < S1; j++) {
    if (rad[j] != 1) continue;
    WT t;
    const int iv = cp(j, hint, t);
    if (iv < 0) return false;
    hint = iv;
    const WT A = area(j);
#pragma unroll
    for (int e = 0; e < kEPT; e++) {
      if (pb + e < ne) {
        const PieceT<WT> q = co4[(pb + e) * N_L + iv];
        const WT sv = q.y + t * (q.k1 + t * (q.k2 + t * q.k3));
        if (positive(sv)) acc[e] += A * sv;
      }
    }
  }
  return true;
}

// the FP64 path's form of cell_phase_sums, in double-float arithmetic on
// scaled pieces (the sign test is on the high part: h + l has the sign of h;
// with the elsewhere correction every value is added, :593-594)
template <typename CP, typename AR>
__device__ __forceinline__ bool cell_phase_sums_df(const CP &cp, const AR &area, int S1,
                                                   const int32_t *rad, const PieceDF *pc, int N_L,
                                                   int pb, int ne, bool add_all,
                                                   DF (&acc)[kEPT]) {
  int hint = -1;
  for (int j = 0; j < S1; j++) {
    if (rad[j] != 1) continue;
    DF t;
    const int iv = cp(j, hint, t);
    if (iv < 0) return false;
    hint = iv;
    const DF A = area(j);
    // every energy slot of the task is evaluated (slots past the chunk's
    // energies read pieces of the coefficient area that the caller ignores)
    // and the positive part is a select: no branch inside the cell, so the
    // kEPT independent double-float chains interleave
#pragma unroll
    for (int e = 0; e < kEPT; e++) {
      const PieceDF q = pc[(pb + e) * N_L + iv];
      const DF sv = df_fma(t, df_fma(t, df_fma(t, q.k3, q.k2), q.k1), q.y);
      const DF nx = df_fma(A, sv, acc[e]);
      const bool take = add_all || sv.h > 0.0f;
      acc[e].h = take ? nx.h : acc[e].h;
      acc[e].l = take ? nx.l : acc[e].l;
    }
  }
  return true;
}

// ---------------------------------------------------------------------------
// Power-sum form of the FP64 path's cell x phase sums.  At a signal phase k
// the cells of a parallel fall, in azimuth order, into runs of consecutive
// radiating cells whose wrapped phase lies in the same knot interval iv (a
// run ends where the interval changes).  Over a run every energy row
// evaluates the same cubic piece, so
//     sum_j A_j S_E(t_j) = y W0 + k1 W1 + k2 W2 + k3 W3,  Wp = sum_j A_j t_j^p,
// and the power sums Wp depend on the geometry only: they are formed once
// per (parallel, image) and reused by all N_E energies.  This holds where
// the reference adds every value (the elsewhere correction) or where the
// piece is positive on its whole interval; a piece that is <= 0 on its whole
// interval adds nothing.  A piece whose sign changes inside its interval is
// evaluated cell by cell over the run, with the reference's test (:593-594).
// The sign of a piece on [0, h] is bounded by its Bernstein coefficients
// (the curve lies in their convex hull), with a margin of 1e-5 of the
// piece's scale so that rounding cannot flip the classification.
//
// Run records live in global scratch, per chunk: for cell half c (the two
// halves of the parallel's cells are walked by different threads) and run r
// of phase k, record (c w_cap + r) N_P + k (consecutive phases adjacent, so a
// warp's tasks load them coalesced): two float4 with the float pairs of
// W0, W1 and W2, W3, and an int with the interval (bits 0-9), the first
// cell (bits 10-19) and the cell span (bits 20-29).
// ---------------------------------------------------------------------------
__host__ __device__ inline size_t integrate_wsum_bytes_dev(int N_P, int cap) {
  const size_t n = (size_t)2 * cap * N_P;
  return (n * (2 * sizeof(float4) + sizeof(int)) + 255) & ~size_t(255);
}

struct WRuns {
  float4 *wa, *wb;
  int *meta;
  int cap, N_P;
  __device__ __forceinline__ size_t rec(int half, int r, int k) const {
    return ((size_t)half * cap + r) * N_P + k;
  }
};

__device__ __forceinline__ WRuns wruns_of(unsigned char *base, int cap, int N_P) {
  const size_t n = (size_t)2 * cap * N_P;
  WRuns w;
  w.wa = reinterpret_cast<float4 *>(base);
  w.wb = w.wa + n;
  w.meta = reinterpret_cast<int *>(w.wb + n);
  w.cap = cap;
  w.N_P = N_P;
  return w;
}

// piece classes: 0 adds nothing, 1 power sums, 2 cell by cell
__device__ __forceinline__ uint8_t piece_class(const PieceDF &q, float h) {
  const float y = q.y.h, a1 = q.k1.h * h, a2 = q.k2.h * h * h, a3 = q.k3.h * h * h * h;
  const float scale = fabsf(y) + fabsf(a1) + fabsf(a2) + fabsf(a3);
  if (scale == 0.0f) return 0;
  const float b1 = y + a1 * (1.0f / 3.0f);
  const float b2 = y + a1 * (2.0f / 3.0f) + a2 * (1.0f / 3.0f);
  const float b3 = y + a1 + a2 + a3;
  const float lo = fminf(fminf(y, b1), fminf(b2, b3));
  const float hi = fmaxf(fmaxf(y, b1), fmaxf(b2, b3));
  const float margin = 1.0e-5f * scale;
  if (lo > margin) return 1;
  if (hi < -margin) return 0;
  return 2;
}

// the runs of signal phase k over cells [jb, je) of the parallel; returns
// the number of runs written, or -1 when a cell phase cannot be wrapped
// into the knot range (the reference's terminate)
template <typename CP, typename AR>
__device__ __forceinline__ int build_runs(const CP &cp, const AR &area, int jb, int je,
                                          const int32_t *rad, const WRuns &w, int half, int k) {
  int n = 0, cur = -1, j0 = 0, span = 0, hint = -1;
  const DF zero{0.0f, 0.0f};
  DF w0 = zero, w1 = zero, w2 = zero, w3 = zero;
  auto flush = [&]() {
    const size_t r = w.rec(half, n, k);
    w.wa[r] = make_float4(w0.h, w0.l, w1.h, w1.l);
    w.wb[r] = make_float4(w2.h, w2.l, w3.h, w3.l);
    w.meta[r] = cur | (j0 << 10) | (span << 20);
    n++;
  };
  for (int j = jb; j < je; j++) {
    if (rad[j] != 1) continue;
    DF t;
    const int iv = cp(j, hint, t);
    if (iv < 0) return -1;
    hint = iv;
    if (iv != cur) {
      if (cur >= 0) flush();
      cur = iv;
      j0 = j;
      w0 = w1 = w2 = w3 = zero;
    }
    const DF A = area(j);
    const DF At = df_mul(A, t), At2 = df_mul(At, t), At3 = df_mul(At2, t);
    w0 = df_add(w0, A);
    w1 = df_add(w1, At);
    w2 = df_add(w2, At2);
    w3 = df_add(w3, At3);
    span = j - j0 + 1;
  }
  if (cur >= 0) flush();
  return n;
}

// the run's cells one by one (a piece whose sign changes on its interval)
template <typename CP, typename AR>
__device__ __forceinline__ DF run_cells(const CP &cp, const AR &area, const int32_t *rad, int iv,
                                     int j0, int span, const PieceDF &q, DF acc) {
  for (int j = j0; j < j0 + span; j++) {
    if (rad[j] != 1) continue;
    DF t;
    if (cp(j, iv, t) != iv) continue;
    const DF sv = df_fma(t, df_fma(t, df_fma(t, q.k3, q.k2), q.k1), q.y);
    if (sv.h > 0.0f) acc = df_fma(area(j), sv, acc);
  }
  return acc;
}

// sums at signal phase k for the energies pb .. pb+kEPT-1 of the chunk from
// the power sums of the runs of one half of the parallel's cells.  The lanes of a warp take consecutive phases,
// so the r-th runs of neighbouring lanes lie in different intervals and
// carry different piece classes: every energy's power-sum term is formed on
// every lane and kept where the class is 1 (a select, no branch), and the
// runs whose piece changes sign are only noted here and walked cell by cell
// after the last run, so that one lane's cell walk does not hold up the
// others run after run.  The next run's record is loaded before the current
// one is used.
constexpr int kDeferRuns = 24;  // sign-changing (run, energy) items noted per task

template <typename CP, typename AR>
__device__ __forceinline__ void run_sums(const CP &cp, const AR &area, const int32_t *rad,
                                         const WRuns &w, const int *nruns, int k, int half,
                                         const PieceDF *pc, const uint8_t *cls, int N_L, int EC,
                                         int pb, DF (&acc)[kEPT]) {
  uint32_t defer[kDeferRuns];
  int nd = 0;
  const int n = nruns[half * w.N_P + k];
  float4 a4, b4;
  int meta = 0;
  if (n > 0) {
    const size_t ri = w.rec(half, 0, k);
    a4 = w.wa[ri];
    b4 = w.wb[ri];
    meta = w.meta[ri];
  }
  for (int r = 0; r < n; r++) {
    const DF W0{a4.x, a4.y}, W1{a4.z, a4.w}, W2{b4.x, b4.y}, W3{b4.z, b4.w};
    const int iv = meta & 1023;
    if (r + 1 < n) {
      const size_t ri = w.rec(half, r + 1, k);
      a4 = w.wa[ri];
      b4 = w.wb[ri];
      meta = w.meta[ri];
    }
    // slots past the chunk's energies have class 0
#pragma unroll
    for (int e = 0; e < kEPT; e++) {
      const uint8_t c = cls[iv * EC + pb + e];
      const PieceDF q = pc[(pb + e) * N_L + iv];
      float sh = acc[e].h, sl = acc[e].l;
      df_acc_mul(q.y, W0, sh, sl);
      df_acc_mul(q.k1, W1, sh, sl);
      df_acc_mul(q.k2, W2, sh, sl);
      df_acc_mul(q.k3, W3, sh, sl);
      if (c == 1) acc[e] = fast_two_sum(sh, sl);
      if (c == 2) {
        if (nd < kDeferRuns) {
          defer[nd++] = ((uint32_t)r << 4) | (uint32_t)e;
        } else {
          const int m = w.meta[w.rec(half, r, k)];
          acc[e] = df_add(acc[e], run_cells(cp, area, rad, iv, (m >> 10) & 1023,
                                            (m >> 20) & 1023, q, DF{0.0f, 0.0f}));
        }
      }
    }
  }
  for (int d = 0; d < nd; d++) {
    const uint32_t it = defer[d];
    const int r = (int)(it >> 4), ed = (int)(it & 15u);
    const int m = w.meta[w.rec(half, r, k)];
    const int iv = m & 1023;
    const DF add = run_cells(cp, area, rad, iv, (m >> 10) & 1023, (m >> 20) & 1023,
                             pc[(pb + ed) * N_L + iv], DF{0.0f, 0.0f});
#pragma unroll
    for (int e = 0; e < kEPT; e++)
      if (e == ed) acc[e] = df_add(acc[e], add);
  }
}

// ---------------------------------------------------------------------------
// beaming modification of the hot intensity I at energy E (the comoving
// energy the atmosphere sees) and emission cosine mu, hot_wrapper.pyx:153-199:
// 1: I (1 + abb E^cbb mu + bbb E^dbb mu^2); 2: the same with the analytical
// normalisation 0.5 / (0.5 + abb E^cbb / 3 + bbb E^dbb / 4); 3: normalised by
// the trapezoidal mu-integrals of I and of the modified I over nimu nodes
// mu = 1/nimu, 2/nimu, ... (the reference's accumulated sums), eval_mu(mu)
// giving the unmodified intensity there.  Negative results are 0.
// ---------------------------------------------------------------------------
template <typename EvalMu>
__device__ double beamed_intensity(int opt, const double *b, double E, double mu, double I_hot,
                                   const EvalMu &eval_mu) {
  const double fa = b[0] * pow(E, b[2]), fb = b[1] * pow(E, b[3]);
  double I = 0.0;
  if (opt == 1) {
    I = (1.0 + fa * mu + fb * (mu * mu)) * I_hot;
  } else if (opt == 2) {
    const double anorm = 0.5 / (0.5 + (1.0 / 3.0) * b[0] * pow(E, b[2]) +
                                (1.0 / 4.0) * b[1] * pow(E, b[3]));
    I = anorm * (1.0 + fa * mu + fb * (mu * mu)) * I_hot;
  } else if (opt == 3) {
    const double nimu = b[4];
    const long n = nimu > 0.0 ? (long)nimu : 0;
    double m = 0.0, nom = 0.0, den = 0.0;
    for (long k = 0; k < n; k++) {
      m = m + (1.0 / nimu);
      const double dmu = (k == 0 || (double)k == nimu - 1.0) ? (0.5 / nimu) : (1.0 / nimu);
      const double Ik = eval_mu(m);
      const double fk = 1.0 + fa * m + fb * (m * m);
      den = den + m * fk * Ik * dmu;
      nom = nom + m * Ik * dmu;
    }
    if (are_equal(den, 0.0)) I = 0.0;
    else I = (nom / den) * (1.0 + fa * mu + fb * (mu * mu)) * I_hot;
  } else {
    return I_hot;
  }
  return I < 0.0 ? 0.0 : I;
}

// ---------------------------------------------------------------------------
// main integrator kernel: one CTA per chunk of parallels of one mesh
// ---------------------------------------------------------------------------
// WT = double: the plain FP64 drop-in.  WT = float: the mixed-precision form
// (geometry, visibility and knots in FP64; atmosphere, Akima pieces and the
// cell x phase sums in FP32; per-chunk partials in FP64).
template <typename WT>
__global__ void __launch_bounds__(kThreads, 2) integrate_kernel(IntegrateArgs a) {
  constexpr bool kMixed = std::is_same<WT, float>::value;
  extern __shared__ __align__(16) char smem[];
  if ((int)blockIdx.x >= *a.chunk_count) return;
  const int chunk = a.chunk_order[blockIdx.x];
  const int64_t r0 = a.chunk_r0[chunk], r1 = a.chunk_r1[chunk];
  const int m = a.row_member[r0];
  const MemberDesc M = a.members[m];
  const int N_L = a.N_L, N_E = a.N_E, N_P = a.N_P;
  const int leaf_lim = (N_L % 2 == 0) ? N_L / 2 : (N_L + 1) / 2;
  // 2-D tables (atmos.I is [nmu][nE], no 10^(3 log T)): atm 4, Pol_Num2D's
  // I on (mu, log10 E') (hot_Num2D.pyx:187-400); atm 6, a split atmosphere
  // reduced once per call to (mu, E) with E' in electron rest energies
  // (integrator_for_azimuthal_invariance_split.pyx:270-275,457-476)
  const bool tab2 = (M.atm == 4 || M.atm == 6) && !kMixed;
  const bool erest = (M.atm == 6);
  const bool num4d = (M.atm == 2) || tab2;
  const int nmu = a.atmos.I ? a.atmos.nmu : 0, nEt = a.atmos.I ? a.atmos.nE : 0;
  const Layout L = make_layout(N_L, N_P, N_E, nmu, nEt, (int)sizeof(PieceT<WT>), a.N_R);
  const int EC = L.EC;
  double *coef;
  AtmSmem as{};
  GeoSmem g = carve(smem, N_L, EC, &coef, nmu, nEt, &as, (int)sizeof(PieceT<WT>), a.N_R);
  PieceT<WT> *co4 = reinterpret_cast<PieceT<WT> *>(coef);
  __shared__ int s_J, s_top, s_any, s_jalt;
  // a beaming modification's (abb, bbb, cbb, dbb, nimu) for the parallel
  __shared__ double s_beam[5];
  // power-sum form (FP64 path with scratch): run counts per (cell half,
  // signal phase) and the class of every piece of the chunk; the run
  // records live in one of a.w_slots scratch slots, taken for the CTA's
  // lifetime (at most 2 CTAs per SM are resident, the pool has more slots;
  // a CTA that finds none after a bounded search runs the per-cell form)
  __shared__ int s_wslot, s_next;
  bool use_w = !kMixed && a.wsum != nullptr;
  if (use_w) {
    if (threadIdx.x == 0) {
      int got = -1;
      for (int i = 0; i < 4 * a.w_slots && got < 0; i++) {
        const int sl = (int)((blockIdx.x + i) % a.w_slots);
        if (atomicCAS(&a.w_slot_busy[sl], 0, 1) == 0) got = sl;
      }
      s_wslot = got;
    }
    __syncthreads();
    use_w = s_wslot >= 0;
  }
  int *s_nruns = reinterpret_cast<int *>(g.sc_exp + EC);
  uint8_t *s_cls = reinterpret_cast<uint8_t *>(s_nruns + 2 * N_P);
  const WRuns wr = use_w ? wruns_of(a.wsum + (size_t)s_wslot *
                                                 integrate_wsum_bytes_dev(N_P, a.w_cap),
                                    a.w_cap, N_P)
                         : WRuns{};
  double *slab = nullptr;
  float *slabf = nullptr;
  if (num4d) {
    stage_table_grids(a.atmos, as, nmu, nEt);
    // the mixed form's FP32 interpolation data
    if (kMixed) {
      for (int t = threadIdx.x; t < min(N_E, kMaxEnergiesF); t += blockDim.x)
        as.fE[t] = (float)a.energies[t];
      for (int t = threadIdx.x; t < 4 * nmu; t += blockDim.x) as.fsmu[t] = (float)as.smu[t];
      for (int t = threadIdx.x; t < 4 * nEt; t += blockDim.x) as.fsE[t] = (float)as.sE[t];
      for (int t = threadIdx.x; t < 3 * nEt; t += blockDim.x) {
        const int b = t / 3, i = t - 3 * b + 1;
        as.fgEo[t] = b + i < nEt ? (float)(as.gE[b + i] - as.gE[b]) : 0.0f;
      }
    }
    slab = tab2 ? const_cast<double *>(a.atmos.I) : a.slab + (size_t)chunk * nmu * nEt;
    slabf = reinterpret_cast<float *>(slab);
    if (!kMixed && !tab2) {
      // the energy grid's node offsets and inverse denominators as
      // double-float pairs for eval_num4d_df (sE converted in place)
      for (int t = threadIdx.x; t < 3 * nEt; t += blockDim.x) {
        const int b = t / 3, i = t - 3 * b + 1;
        as.dgEo[t] = b + i < nEt ? df_split(as.gE[b + i] - as.gE[b]) : DF{0.0f, 0.0f};
      }
      for (int t = threadIdx.x; t < 4 * nEt; t += blockDim.x) {
        const double v = as.sE[t];
        as.dsE[t] = df_split(v);
      }
    }
    __syncthreads();
  }
  if (kMixed && !num4d) {
    for (int t = threadIdx.x; t < min(N_E, kMaxEnergiesF); t += blockDim.x)
      as.fE[t] = (float)a.energies[t];
    __syncthreads();
  }
  const double norm = num4d ? kErg / kHKeV : kErg * kPlanck;
  double *part = a.partial + (size_t)chunk * N_E * N_P;
  // the power sums' second cell half adds into its own partial
  double *part2 = a.partial2 ? a.partial2 + (size_t)chunk * N_E * N_P : nullptr;
  for (int t = threadIdx.x; t < N_E * N_P; t += blockDim.x) {
    part[t] = 0.0;
    if (part2) part2[t] = 0.0;
  }
  __syncthreads();
  const double mu_max = num4d ? a.atmos.mu[a.atmos.nmu - 1] : 0.0;
  const double mu_top3 = num4d ? a.atmos.mu[a.atmos.nmu - 3] : 0.0;
  const int groups = EC / kEPT;
  const int ntasks = N_P * groups;
  // algorithmic FLOPs per (parallel, image), the cost model of the
  // likelihood path: leaf work N_L (60 + N_E f_atm) and spline work
  // N_E (30 N_L + C N_P 14), f_atm 12 (blackbody) or 1350 (4-D table)
  double flops = 0.0;
  const double f_atm = num4d ? 1350.0 : 12.0;

  for (int64_t row = r0; row < r1; row++) {
    const int i = (int)(row - M.row_off);
    RowCtx c;
    if (!load_row(a, M, row, i, c, &s_J)) continue;
    stage_deflection(c, g, &s_jalt);
    if (threadIdx.x == 0) {
      s_top = num4d ? (int)a.row_entry_top[row] : 0;
      s_any = 0;
      // parameters 2-6 of the parallel's first radiating cell
      if (M.beam_opt > 0) {
        const double *vec = a.params + (M.cell_off + (int64_t)i * M.S1 + c.J) * a.n_params;
        for (int b = 0; b < 5; b++) s_beam[b] = vec[2 + b];
      }
    }
    __syncthreads();
    double E_eff = 0.0, p3 = 0.0;
    if (tab2) {
      p3 = 1.0;
    } else if (num4d) {
      // contract the (log T, log g) stencil of this parallel once:
      // slab[mu][logE] = sum_ij w_T[i] w_g[j] table[bT+i][bg+j][mu][logE]
      double vT = c.vec0, vg = c.vec1;
      if (vT < a.atmos.logT[0]) vT = a.atmos.logT[0];
      if (vT > a.atmos.logT[a.atmos.nT - 1]) vT = a.atmos.logT[a.atmos.nT - 1];
      if (vg < a.atmos.logg[0]) vg = a.atmos.logg[0];
      if (vg > a.atmos.logg[a.atmos.ng - 1]) vg = a.atmos.logg[a.atmos.ng - 1];
      const int bT = stencil_base(a.atmos.logT, a.atmos.nT, vT);
      const int bg = stencil_base(a.atmos.logg, a.atmos.ng, vg);
      double wT[4], wg[4];
      lagrange4(a.atmos.logT, bT, vT, wT);
      lagrange4(a.atmos.logg, bg, vg, wg);
      const size_t S1t = (size_t)nmu * nEt, S0t = (size_t)a.atmos.ng * S1t;
      if (kMixed && a.atmos.I32 != nullptr) {
        // FP32 contraction from the FP32 copy of the table
        const float *basef = a.atmos.I32 + bT * S0t + bg * S1t;
        float wTf[4], wgf[4];
#pragma unroll
        for (int ii = 0; ii < 4; ii++) {
          wTf[ii] = (float)wT[ii];
          wgf[ii] = (float)wg[ii];
        }
        for (int t = threadIdx.x; t < (int)S1t; t += blockDim.x) {
          float r = 0.0f;
#pragma unroll
          for (int ii = 0; ii < 4; ii++) {
            const float *q = basef + ii * S0t + t;
            float u = wgf[0] * __ldg(q) + wgf[1] * __ldg(q + S1t) + wgf[2] * __ldg(q + 2 * S1t) +
                      wgf[3] * __ldg(q + 3 * S1t);
            r += wTf[ii] * u;
          }
          slabf[t] = r;
        }
      } else {
        const double *base = a.atmos.I + bT * S0t + bg * S1t;
        double mx = 0.0;
        for (int t = threadIdx.x; t < (int)S1t; t += blockDim.x) {
          double r = 0.0;
#pragma unroll
          for (int ii = 0; ii < 4; ii++) {
            const double *q = base + ii * S0t + t;
            double u = wg[0] * __ldg(q) + wg[1] * __ldg(q + S1t) + wg[2] * __ldg(q + 2 * S1t) +
                       wg[3] * __ldg(q + 3 * S1t);
            r += wT[ii] * u;
          }
          if (kMixed) {
            slabf[t] = (float)r;
          } else {
            slab[t] = r;
            mx = fmax(mx, fabs(r));
          }
        }
        if (!kMixed) {
          // the FP64 form keeps the slab as double-float pairs, each energy
          // node's column (all mu) scaled by 2^-xe[e] (exact), xe the binary
          // exponent of its largest value, so that the pairs keep full
          // relative precision across the table's exponential tail
          for (int e = threadIdx.x; e < nEt; e += blockDim.x) as.xe[e] = kZeroExp;
          __syncthreads();
          for (int t = threadIdx.x; t < (int)S1t; t += blockDim.x)
            atomicMax(&as.xe[t % nEt], binary_exponent(slab[t]));
          __syncthreads();
          DF *slabd = reinterpret_cast<DF *>(slab);
          for (int t = threadIdx.x; t < (int)S1t; t += blockDim.x) {
            const double r = slab[t];
            slabd[t] = df_split(r * pow2_double(-as.xe[t % nEt]));
          }
        }
      }
      E_eff = (kKB / kKeV) * pow(10.0, c.vec0);
      p3 = pow(10.0, 3.0 * vT);
      __syncthreads();
    }
    // the FP64 form's double-float slab (energy columns scaled by 2^-xe)
    const DF *slabd = reinterpret_cast<const DF *>(slab);
    const double kT = (kKB / kKeV) * pow(10.0, c.vec0);
    const float kT_f = (float)kT;
    // mixed form: the FP32 roundings of the constant factors norm and
    // 10^(3 log T) are undone exactly on the parallel's FP64 partials
    const float p3f = (float)p3;
    const double fix = num4d ? (norm * p3) / ((double)(float)norm * (double)p3f)
                             : norm / (double)(float)norm;
    const double lg_Eeff = (num4d && !tab2) ? log10(E_eff) : 0.0;
    // the elsewhere correction's blackbody temperature at the parallel's
    // first radiating cell (:469-476)
    const bool corr = !kMixed && a.correction != nullptr;
    // the plain Num4D columns without beaming or correction keep their
    // intensities as double-float mantissas with exponents up to the row
    // scaling (uniform over the CTA: a chunk is one mesh's rows)
    const bool dfy = !kMixed && num4d && !tab2 && M.beam_opt == 0 && !corr;
    const double kT_c =
        corr ? (kKB / kKeV) *
                   pow(10.0, a.correction[(M.cell_off + (int64_t)i * M.S1 + c.J) * a.n_correction])
             : 0.0;
    const double *cellA = a.cellArea + M.cell_off + (int64_t)i * M.S1;
    const double *cellPhi = a.phi + M.cell_off + (int64_t)i * M.S1;
    const int32_t *rad = a.radiates + M.cell_off + (int64_t)i * M.S1;
    for (int I = 0; I < c.IO; I++) {
      for (int k = threadIdx.x; k < leaf_lim; k += blockDim.x)
        leaf_geometry(c, I, k, N_L, leaf_lim, a.leaves, g);
      __syncthreads();
      if (threadIdx.x == 0) {
        int top = s_top, any = s_any;
        state_machine(N_L, leaf_lim, a.leaves, g, num4d, mu_top3, mu_max, top, any);
        s_top = top;
        s_any = any;
      }
      __syncthreads();
      const int term = g.flags[0], invis = g.flags[1];
      if (term) {
        if (threadIdx.x == 0) {
          atomicExch(&a.member_status[m], (int)kPulseFail);
          if (use_w) atomicExch(&a.w_slot_busy[s_wslot], 0);
        }
        return;
      }
      if (invis) break;
      // phase knots, cell azimuths and areas as float pairs for the cell x
      // phase sums (both forms)
      for (int t = threadIdx.x; t < N_L; t += blockDim.x) {
        const float hi = (float)g.phase[t];
        as.fphase[t] = hi;
        as.fphase_lo[t] = (float)(g.phase[t] - (double)hi);
      }
      if (M.S1 <= kMaxCellsF) {
        for (int t = threadIdx.x; t < M.S1; t += blockDim.x) {
          const float hi = (float)cellPhi[t];
          as.fcphi[t] = hi;
          as.fcphi_lo[t] = (float)(cellPhi[t] - (double)hi);
          const float ah = (float)cellA[t];
          as.fcarea[t] = ah;
          as.fcarea_lo[t] = (float)(cellA[t] - (double)ah);
        }
      }
      if (!kMixed) {
        for (int t = threadIdx.x; t < N_L - 1; t += blockDim.x) {
          const double h = g.phase[t + 1] - g.phase[t];
          g.ih[t] = df_split(1.0 / h);
          g.ih2[t] = df_split(1.0 / (h * h));
        }
      }
      for (int t = threadIdx.x; t < N_L; t += blockDim.x) {
        const int sidx = g.src[t];
        if (sidx >= 0) {
          if (kMixed) {
            as.finvZ[sidx] = (float)(1.0 / g.Z[sidx]);
            as.fabb[sidx] = (float)g.ABB[sidx];
            as.fgeom[sidx] = (float)g.GEOM[sidx];
          }
          if (erest) g.lzs[sidx] = g.Z[sidx];
          else if (num4d) g.lzs[sidx] = log10(g.Z[sidx]) + lg_Eeff;
        }
      }
      __syncthreads();
      if (use_w) {
        // the runs of every signal phase, each half of the cells by its own
        // thread (energy independent: formed once per parallel and image)
        const int hc = (M.S1 + 1) / 2;
        const bool cached = M.S1 <= kMaxCellsF;
        const AreaDF ar{cached ? as.fcarea : nullptr, cached ? as.fcarea_lo : nullptr, cellA};
        for (int t = threadIdx.x; t < 2 * N_P; t += blockDim.x) {
          const int k = t % N_P, half = t / N_P;
          const double phd = a.phases[k];
          const float ph = (float)phd;
          const float tp = (float)kTwoPi;
          const CellPhaseF cp{as.fphase, as.fphase_lo, N_L, as.fphase[0], as.fphase[N_L - 1], ph,
                              (float)(phd - (double)ph), tp, (float)(kTwoPi - (double)tp),
                              cached ? as.fcphi : nullptr, cached ? as.fcphi_lo : nullptr,
                              cellPhi};
          int n = build_runs(cp, ar, half * hc, min(M.S1, (half + 1) * hc), rad, wr, half, k);
          if (n < 0) {
            atomicExch(&a.member_status[m], (int)kPulseFail);
            n = 0;
          }
          s_nruns[half * N_P + k] = n;
        }
        __syncthreads();
      }
      if (threadIdx.x == 0 && a.flop_counter) {
        int Cr = 0;
        for (int j = 0; j < M.S1; j++) Cr += (rad[j] == 1);
        flops += (double)N_L * (60.0 + N_E * f_atm) +
                 (double)N_E * (30.0 * N_L + (double)Cr * N_P * 14.0);
      }

      for (int e0 = 0; e0 < N_E; e0 += EC) {
        const int ne = min(EC, N_E - e0);
        if (num4d) {
          for (int t = threadIdx.x; t < ne; t += blockDim.x)
            g.lgE[t] = erest ? a.energies[e0 + t] : log10(a.energies[e0 + t]);
          __syncthreads();
        }
        // specific intensities of every profile column (:445-478).  With
        // N_L dividing the block size a thread keeps one column for all its
        // energies, so its mu stencil (FP64 form) is formed once.
        {
          int mu_col = -1;
          MuStencil ms{};
          MuStencilF msf{};
          MuStencilDF msd{};
          double col_factor = 0.0;  // norm 10^(3 log T) GEOM of the column
          DF cf_m{0.0f, 0.0f};      // col_factor = cf_m 2^cf_x (dfy form)
          int cf_x = 0;
          for (int t = threadIdx.x; t < ne * N_L; t += blockDim.x) {
            const int pl = t / N_L, col = t - pl * N_L;
            const int p = e0 + pl;
            const int s = g.src[col];
            WT y = WT(0);
            if (s >= 0) {
              if constexpr (kMixed) {
                float I_E;
                if (num4d) {
                  // atm 6: E' = E / Z in electron rest energies (:457-458)
                  const double v3 = erest ? (g.lgE[pl] / g.lzs[s]) * 0.001956951
                                          : g.lgE[pl] - g.lzs[s];
                  if (p == 0 && g.clamp0[s]) {
                    I_E = eval_num4d_f(a.atmos, as, slabf,
                                       mu_stencil_f(a.atmos, as, as.fabb[s], true), v3, p3f);
                  } else {
                    if (s != mu_col) {
                      msf = mu_stencil_f(a.atmos, as, as.fabb[s], false);
                      mu_col = s;
                    }
                    I_E = eval_num4d_f(a.atmos, as, slabf, msf, v3, p3f);
                  }
                } else {
                  const float Ef = p < kMaxEnergiesF ? as.fE[p] : (float)a.energies[p];
                  I_E = eval_bb_f(Ef * as.finvZ[s], kT_f);
                }
                y = (WT)((float)norm * I_E * as.fgeom[s]);
              } else {
                double I_E;
                if (num4d && !tab2) {
                  // the contracted 4-D table in double-float (eval_num4d_df);
                  // with beaming option 3 every call is followed by calls up
                  // to mu = 1, so no out-of-table mu is ever clamped
                  const double v3 = g.lgE[pl] - g.lzs[s];
                  if (s != mu_col) {
                    msd = mu_stencil_df(a.atmos, as, g.ABB[s], false);
                    col_factor = norm * p3 * g.GEOM[s];
                    if (dfy) {
                      MaxExponent mx;
                      mx.fold(col_factor);
                      cf_x = mx.exponent();
                      cf_m = df_split(scale_pow2(col_factor, -cf_x));
                    }
                    mu_col = s;
                  }
                  int xr;
                  DF I = (p == 0 && g.clamp0[s] && M.beam_opt != 3)
                             ? eval_num4d_dfx(a.atmos, as, slabd,
                                              mu_stencil_df(a.atmos, as, g.ABB[s], true), v3,
                                              xr)
                             : eval_num4d_dfx(a.atmos, as, slabd, msd, v3, xr);
                  if (I.h < 0.0f) I = DF{0.0f, 0.0f};
                  if (dfy) {
                    // y = I 2^xr col_factor kept as a double-float mantissa
                    // and an exponent (no round trip through FP64)
                    Piece &o = co4[pl * N_L + col];
                    *reinterpret_cast<DF *>(&o.y) = df_mul(I, cf_m);
                    *reinterpret_cast<int *>(&o.k1) = xr + cf_x;
                    continue;
                  }
                  I_E = df_value(I) * pow2_double(xr) * p3;
                } else if (num4d) {
                  // atm 6: E' = E / Z in electron rest energies (:457-458)
                  const double v3 = erest ? (g.lgE[pl] / g.lzs[s]) * 0.001956951
                                          : g.lgE[pl] - g.lzs[s];
                  // with beaming option 3 every call is followed by calls up
                  // to mu = 1, so no out-of-table mu is ever clamped
                  if (p == 0 && g.clamp0[s] && M.beam_opt != 3) {
                    I_E = eval_num4d_e(a.atmos, as, slab, mu_stencil(a.atmos, as, g.ABB[s], true),
                                       v3, p3);
                  } else {
                    if (s != mu_col) {
                      ms = mu_stencil(a.atmos, as, g.ABB[s], false);
                      mu_col = s;
                    }
                    I_E = eval_num4d_e(a.atmos, as, slab, ms, v3, p3);
                  }
                } else {
                  I_E = eval_bb(a.energies[p] / g.Z[s], kT);
                  // the burst blackbody's limb darkening (hot_BB_burst.pyx)
                  if (M.atm == 3) I_E = I_E * (0.421 + 0.868 * g.ABB[s]);
                }
                {
                  const double I_c =
                      corr ? eval_bb(a.energies[p] / g.Z[s], kT_c) * (kErg * kPlanck) : 0.0;
                  // with a beaming modification the raw intensity is kept
                  // here and modified in the pass below
                  y = (WT)(M.beam_opt > 0 ? I_E : (I_E * norm - I_c) * g.GEOM[s]);
                }
              }
            }
            co4[pl * N_L + col].y = y;
          }
        }
        if (!kMixed && M.beam_opt > 0) {
          // the beaming modification (hot_wrapper.pyx:153-199) of every
          // column intensity of the chunk, by the thread that formed it
          for (int t = threadIdx.x; t < ne * N_L; t += blockDim.x) {
            const int pl = t / N_L, col = t - pl * N_L;
            const int p = e0 + pl;
            const int s = g.src[col];
            if (s < 0) continue;
            const double I_raw = (double)co4[pl * N_L + col].y;
            double I_E;
            if (num4d) {
              const double v3 = erest ? (g.lgE[pl] / g.lzs[s]) * 0.001956951 : g.lgE[pl] - g.lzs[s];
              const double Ep = erest ? v3 : a.energies[p] / g.Z[s];
              I_E = beamed_intensity(M.beam_opt, s_beam, Ep, g.ABB[s], I_raw, [&](double mu_k) {
                if (tab2)
                  return eval_num4d_e(a.atmos, as, slab, mu_stencil(a.atmos, as, mu_k, false),
                                      v3, p3);
                double scale;
                const DF I = eval_num4d_df(a.atmos, as, slabd,
                                           mu_stencil_df(a.atmos, as, mu_k, false), v3, scale);
                return I.h < 0.0f ? 0.0 : df_value(I) * scale * p3;
              });
            } else {
              const double Ep = a.energies[p] / g.Z[s];
              const double I0 = eval_bb(Ep, kT);  // the blackbody has no mu dependence
              I_E = beamed_intensity(M.beam_opt, s_beam, Ep, g.ABB[s], I_raw,
                                     [&](double) { return I0; });
            }
            const double I_c =
                corr ? eval_bb(a.energies[p] / g.Z[s], kT_c) * (kErg * kPlanck) : 0.0;
            co4[pl * N_L + col].y = (WT)((I_E * norm - I_c) * g.GEOM[s]);
          }
        }
        __syncthreads();
        // Akima-periodic piece coefficients (:566-569): a thread builds kStrip
        // consecutive pieces of one energy row from a sliding window of the
        // five chords each piece needs, so each chord is formed once per
        // strip instead of five times
        const int n_iv = N_L - 1, strips = (n_iv + kStrip - 1) / kStrip;
        if constexpr (kMixed) {
          for (int t = threadIdx.x; t < ne * strips; t += blockDim.x) {
            const int pl = t / strips, i0 = (t - pl * strips) * kStrip;
            const int i1 = min(i0 + kStrip, n_iv);
            PieceT<WT> *yr = co4 + pl * N_L;
            auto chord = [&](int j) -> WT {
              const int q = periodic_chord(j, N_L);
              // knot spacings from the FP64 knots: adjacent knots closer
              // than an FP32 ulp stay distinct
              return (yr[q + 1].y - yr[q].y) / (WT)(g.phase[q + 1] - g.phase[q]);
            };
            WT m0 = chord(i0 - 2), m1 = chord(i0 - 1), m2 = chord(i0), m3 = chord(i0 + 1),
               m4 = chord(i0 + 2);
            for (int iv = i0; iv < i1; iv++) {
              if (iv > i0) {
                m0 = m1; m1 = m2; m2 = m3; m3 = m4;
                m4 = chord(iv + 2);
              }
              WT k1, k2, k3;
              const WT h = (WT)(g.phase[iv + 1] - g.phase[iv]);
              akima_piece(m0, m1, m2, m3, m4, h, k1, k2, k3);
              PieceT<WT> *o = yr + iv;
              o->k1 = k1;
              o->k2 = k2;
              o->k3 = k3;
            }
          }
          __syncthreads();
        } else {
          // scale each energy row by a power of two (exact) so that its
          // largest profile value lies in [0.5, 1): double-float values then
          // keep the row's full relative precision whatever its magnitude
          const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
          PieceDF *pc = reinterpret_cast<PieceDF *>(co4);
          if (dfy) {
            // values m 2^x (mantissa in the y slot, exponent in k1's): the
            // row's largest exponent from the bits, then each value times
            // 2^(x - that) in float arithmetic (exact)
            for (int pl = warp; pl < ne; pl += kThreads / 32) {
              MaxExponent mx;
              for (int col = lane; col < N_L; col += 32) {
                const Piece &o = co4[pl * N_L + col];
                const float h = reinterpret_cast<const DF *>(&o.y)->h;
                if (h != 0.0f && h == h) {
                  if (isinf(h)) mx.inf = true;
                  else mx.e = max(mx.e, *reinterpret_cast<const int *>(&o.k1) + float_exponent(h));
                }
              }
              mx.merge_warp();
              if (lane == 0) g.sc_exp[pl] = mx.exponent();
            }
            __syncthreads();
            for (int t = threadIdx.x; t < ne * N_L; t += blockDim.x) {
              const DF m = *reinterpret_cast<const DF *>(&co4[t].y);
              const int x = *reinterpret_cast<const int *>(&co4[t].k1);
              pc[t].y = m.h == 0.0f ? DF{0.0f, 0.0f} : df_times_pow2(m, x - g.sc_exp[t / N_L]);
            }
          } else {
            for (int pl = warp; pl < ne; pl += kThreads / 32) {
              MaxExponent mx;
              for (int col = lane; col < N_L; col += 32) mx.fold((double)co4[pl * N_L + col].y);
              mx.merge_warp();
              if (lane == 0) g.sc_exp[pl] = mx.exponent();
            }
            __syncthreads();
            for (int t = threadIdx.x; t < ne * N_L; t += blockDim.x) {
              const double v = (double)co4[t].y;
              pc[t].y = df_split(scale_pow2(v, -g.sc_exp[t / N_L]));
            }
          }
          __syncthreads();
          for (int t = threadIdx.x; t < ne * strips; t += blockDim.x) {
            const int pl = t / strips, i0 = (t - pl * strips) * kStrip;
            const int i1 = min(i0 + kStrip, n_iv);
            PieceDF *yr = pc + pl * N_L;
            auto chord = [&](int j) -> DF {
              const int q = periodic_chord(j, N_L);
              return df_mul(df_sub(yr[q + 1].y, yr[q].y), g.ih[q]);
            };
            DF m0 = chord(i0 - 2), m1 = chord(i0 - 1), m2 = chord(i0), m3 = chord(i0 + 1),
               m4 = chord(i0 + 2);
            for (int iv = i0; iv < i1; iv++) {
              if (iv > i0) {
                m0 = m1; m1 = m2; m2 = m3; m3 = m4;
                m4 = chord(iv + 2);
              }
              DF k1, k2, k3;
              akima_piece_df(m0, m1, m2, m3, m4, g.ih[iv], g.ih2[iv], k1, k2, k3);
              yr[iv].k1 = k1;
              yr[iv].k2 = k2;
              yr[iv].k3 = k3;
            }
          }
          __syncthreads();
          // the class of every piece for the power sums, [N_L][EC] (0
          // beyond the chunk's energies); every nonzero value is added with
          // the elsewhere correction (:593-594)
          if (use_w) for (int t = threadIdx.x; t < EC * N_L; t += blockDim.x) {
            const int iv = t / EC, pl = t - iv * EC;
            uint8_t cl = 0;
            if (pl < ne && iv < N_L - 1) {
              const PieceDF &q = pc[pl * N_L + iv];
              cl = piece_class(q, as.fphase[iv + 1] - as.fphase[iv]);
              if (corr && cl == 0 &&
                  (q.y.h != 0.0f || q.k1.h != 0.0f || q.k2.h != 0.0f || q.k3.h != 0.0f))
                cl = 1;
              if (corr) cl = cl ? 1 : 0;
            }
            s_cls[t] = cl;
          }
          if (threadIdx.x == 0) s_next = blockDim.x;
          if (use_w) __syncthreads();
        }
        // cell x phase accumulation (:571-598).  The power-sum form splits
        // each task into its two cell halves (units u < ntasks: half 0,
        // u >= ntasks: half 1, adding into part2); a warp takes its first 32
        // consecutive units by index and further blocks of 32 from a shared
        // counter, so the uneven run counts of the phases even out over the
        // CTA while a warp's lanes keep consecutive phases
        const int nunits = use_w ? 2 * ntasks : ntasks;
        const int lane = threadIdx.x & 31;
        for (int u = threadIdx.x; u - lane < nunits;
             u = use_w ? __shfl_sync(0xffffffffu, lane == 0 ? atomicAdd(&s_next, 32) : 0, 0) + lane
                       : u + (int)blockDim.x) {
          if (u >= nunits) continue;
          const int half = u >= ntasks ? 1 : 0;
          const int task = u - half * ntasks;
          const int k = task % N_P, grp = task / N_P;
          const int pb = grp * kEPT;
          if (pb >= ne) continue;
          const double phd = a.phases[k];
          const float ph = (float)phd;
          const float tp = (float)kTwoPi;
          const bool cached = M.S1 <= kMaxCellsF;
          const CellPhaseF cp{as.fphase, as.fphase_lo, N_L, as.fphase[0], as.fphase[N_L - 1], ph,
                              (float)(phd - (double)ph), tp, (float)(kTwoPi - (double)tp),
                              cached ? as.fcphi : nullptr, cached ? as.fcphi_lo : nullptr,
                              cellPhi};
          if constexpr (kMixed) {
            WT acc[kEPT];
#pragma unroll
            for (int e = 0; e < kEPT; e++) acc[e] = WT(0);
            const AreaF ar{cached ? as.fcarea : nullptr, cellA};
            if (!cell_phase_sums<WT>(cp, ar, M.S1, rad, co4, N_L, pb, ne, acc)) {
              atomicExch(&a.member_status[m], (int)kPulseFail);
              continue;
            }
#pragma unroll
            for (int e = 0; e < kEPT; e++)
              if (pb + e < ne) part[(size_t)(e0 + pb + e) * N_P + k] += (double)acc[e] * fix;
          } else {
            DF acc[kEPT];
#pragma unroll
            for (int e = 0; e < kEPT; e++) acc[e] = DF{0.0f, 0.0f};
            const AreaDF ar{cached ? as.fcarea : nullptr, cached ? as.fcarea_lo : nullptr, cellA};
            if (use_w) {
              run_sums(cp, ar, rad, wr, s_nruns, k, half,
                       reinterpret_cast<const PieceDF *>(co4), s_cls, N_L, EC, pb, acc);
            } else if (!cell_phase_sums_df(cp, ar, M.S1, rad,
                                           reinterpret_cast<const PieceDF *>(co4), N_L, pb, ne,
                                           corr, acc)) {
              atomicExch(&a.member_status[m], (int)kPulseFail);
              continue;
            }
            double *dst = half ? part2 : part;
#pragma unroll
            for (int e = 0; e < kEPT; e++)
              if (pb + e < ne)
                dst[(size_t)(e0 + pb + e) * N_P + k] +=
                    scale_pow2(df_value(acc[e]), g.sc_exp[pb + e]);
          }
        }
        __syncthreads();
      }
    }
  }
  if (use_w) {
    __syncthreads();
    if (threadIdx.x == 0) atomicExch(&a.w_slot_busy[s_wslot], 0);
  }
  if (threadIdx.x == 0 && a.flop_counter && flops > 0.0) atomicAdd(a.flop_counter, flops);
}

// ---------------------------------------------------------------------------
// Stokes I, Q, U (integratorIQU_for_azimuthal_invariance.pyx:68-743) for the
// blackbody (Q = 0) and burst blackbody (hot_BB_burst.pyx) atmospheres: one
// CTA per parallel.  Per chunk of energies the I, Q and U profiles of the
// leaves are scaled, splined (Akima periodic) and summed over cells x phases
// in double-float exactly as the FP64 integrator does for I; Q and U are
// added wherever I is (:646-650).
// ---------------------------------------------------------------------------
constexpr int kStokesPiece = 3 * (int)sizeof(PieceDF);

template <typename CP, typename AR>
__device__ __forceinline__ bool cell_phase_sums_stokes(const CP &cp, const AR &area, int S1,
                                                       const int32_t *rad, const PieceDF *pI,
                                                       const PieceDF *pQ, const PieceDF *pU,
                                                       int N_L, int pb, int ne, bool add_all,
                                                       DF (&aI)[kEPT], DF (&aQ)[kEPT],
                                                       DF (&aU)[kEPT]) {
  int hint = -1;
  for (int j = 0; j < S1; j++) {
    if (rad[j] != 1) continue;
    DF t;
    const int iv = cp(j, hint, t);
    if (iv < 0) return false;
    hint = iv;
    const DF A = area(j);
#pragma unroll
    for (int e = 0; e < kEPT; e++) {
      if (pb + e < ne) {
        const int o = (pb + e) * N_L + iv;
        const PieceDF q = pI[o];
        const DF sv = df_fma(t, df_fma(t, df_fma(t, q.k3, q.k2), q.k1), q.y);
        if (sv.h > 0.0f || add_all) {
          aI[e] = df_fma(A, sv, aI[e]);
          const PieceDF qq = pQ[o], qu = pU[o];
          aQ[e] = df_fma(A, df_fma(t, df_fma(t, df_fma(t, qq.k3, qq.k2), qq.k1), qq.y), aQ[e]);
          aU[e] = df_fma(A, df_fma(t, df_fma(t, df_fma(t, qu.k3, qu.k2), qu.k1), qu.y), aU[e]);
        }
      }
    }
  }
  return true;
}

size_t stokes_smem(int N_L, int N_P, int N_E, int N_R, int nmu, int nE) {
  const Layout L = make_layout(N_L, N_P, N_E, nmu, nE, kStokesPiece, N_R);
  return L.bytes + (size_t)2 * N_L * sizeof(double) + (size_t)2 * L.EC * sizeof(int) + 64;
}

__global__ void __launch_bounds__(kThreads, 1) stokes_kernel(IntegrateArgs a) {
  extern __shared__ __align__(16) char smem[];
  const int64_t row = blockIdx.x;
  const int m = a.row_member[row];
  const MemberDesc M = a.members[m];
  const int i = (int)(row - M.row_off);
  const int N_L = a.N_L, N_E = a.N_E, N_P = a.N_P;
  const int leaf_lim = (N_L % 2 == 0) ? N_L / 2 : (N_L + 1) / 2;
  // 2-D table atmospheres: atm 4 (Pol_Num2D, I and Q on (mu, log10 E'),
  // hot_Num2D.pyx:187-400) and atm 6 (split I and Q reduced to (mu, E), E'
  // in electron rest energies,
  // integratorIQU_for_azimuthal_invariance_split.pyx:310-322,515-530)
  const bool tab2 = (M.atm == 4 || M.atm == 6);
  const bool erest = (M.atm == 6);
  const int nmu = a.atmos.I ? a.atmos.nmu : 0, nEt = a.atmos.I ? a.atmos.nE : 0;
  const Layout L = make_layout(N_L, N_P, N_E, nmu, nEt, kStokesPiece, a.N_R);
  const int EC = L.EC;
  double *coef;
  AtmSmem as{};
  GeoSmem g = carve(smem, N_L, EC, &coef, nmu, nEt, &as, kStokesPiece, a.N_R);
  double *xd = reinterpret_cast<double *>(
      (reinterpret_cast<uintptr_t>(g.sc_exp + EC) + 15) & ~uintptr_t(15));
  g.c2chi = xd;
  g.s2chi = xd + N_L;
  int *scQ = reinterpret_cast<int *>(xd + 2 * N_L), *scU = scQ + EC;
  Piece *coI = reinterpret_cast<Piece *>(coef);
  Piece *coQ = coI + (size_t)EC * N_L, *coU = coQ + (size_t)EC * N_L;
  __shared__ int s_J, s_jalt, s_top, s_any;
  double *part = a.partial + (size_t)row * 3 * N_E * N_P;
  RowCtx c;
  if (!load_row(a, M, row, i, c, &s_J)) return;
  stage_deflection(c, g, &s_jalt);
  if (tab2) stage_table_grids(a.atmos, as, nmu, nEt);
  if (threadIdx.x == 0) {
    s_top = tab2 ? (int)a.row_entry_top[row] : 0;
    s_any = 0;
  }
  __syncthreads();
  const double mu_max = tab2 ? a.atmos.mu[nmu - 1] : 0.0;
  const double mu_top3 = tab2 ? a.atmos.mu[nmu - 3] : 0.0;
  const bool burst = (M.atm == 3);
  // hot_BB_burst.pyx, hot_Num2D.pyx:359-367, hot_Num5D_split.pyx:538-563
  const double norm = tab2 ? kErg / kHKeV : kErg * kPlanck;
  const double kT = (kKB / kKeV) * pow(10.0, c.vec0);
  const bool corr = a.correction != nullptr;
  const double kT_c =
      corr ? (kKB / kKeV) *
                 pow(10.0, a.correction[(M.cell_off + (int64_t)i * M.S1 + c.J) * a.n_correction])
           : 0.0;
  const double *cellA = a.cellArea + M.cell_off + (int64_t)i * M.S1;
  const double *cellPhi = a.phi + M.cell_off + (int64_t)i * M.S1;
  const int32_t *rad = a.radiates + M.cell_off + (int64_t)i * M.S1;
  const int n_iv = N_L - 1, strips = (n_iv + kStrip - 1) / kStrip;
  for (int I = 0; I < c.IO; I++) {
    for (int k = threadIdx.x; k < leaf_lim; k += blockDim.x)
      leaf_geometry(c, I, k, N_L, leaf_lim, a.leaves, g);
    __syncthreads();
    if (threadIdx.x == 0) {
      int top = s_top, any = s_any;
      state_machine(N_L, leaf_lim, a.leaves, g, tab2, mu_top3, mu_max, top, any);
      s_top = top;
      s_any = any;
    }
    __syncthreads();
    if (g.flags[0]) {
      if (threadIdx.x == 0) atomicExch(&a.member_status[m], (int)kPulseFail);
      return;
    }
    if (g.flags[1]) break;
    for (int t = threadIdx.x; t < N_L; t += blockDim.x) {
      const float hi = (float)g.phase[t];
      as.fphase[t] = hi;
      as.fphase_lo[t] = (float)(g.phase[t] - (double)hi);
    }
    if (M.S1 <= kMaxCellsF) {
      for (int t = threadIdx.x; t < M.S1; t += blockDim.x) {
        const float hi = (float)cellPhi[t];
        as.fcphi[t] = hi;
        as.fcphi_lo[t] = (float)(cellPhi[t] - (double)hi);
        const float ah = (float)cellA[t];
        as.fcarea[t] = ah;
        as.fcarea_lo[t] = (float)(cellA[t] - (double)ah);
      }
    }
    for (int t = threadIdx.x; t < N_L - 1; t += blockDim.x) {
      const double h = g.phase[t + 1] - g.phase[t];
      g.ih[t] = df_split(1.0 / h);
      g.ih2[t] = df_split(1.0 / (h * h));
    }
    if (tab2) {
      for (int t = threadIdx.x; t < N_L; t += blockDim.x) {
        const int sidx = g.src[t];
        if (sidx >= 0) g.lzs[sidx] = erest ? g.Z[sidx] : log10(g.Z[sidx]);
      }
    }
    __syncthreads();
    for (int e0 = 0; e0 < N_E; e0 += EC) {
      const int ne = min(EC, N_E - e0);
      if (tab2) {
        for (int t = threadIdx.x; t < ne; t += blockDim.x)
          g.lgE[t] = erest ? a.energies[e0 + t] : log10(a.energies[e0 + t]);
        __syncthreads();
      }
      // I, Q cos 2chi and Q sin 2chi of every profile column (:468-497)
      int mu_col = -1;
      MuStencil ms{};
      for (int t = threadIdx.x; t < ne * N_L; t += blockDim.x) {
        const int pl = t / N_L, col = t - pl * N_L;
        const int p = e0 + pl;
        const int s = g.src[col];
        double yI = 0.0, yQ = 0.0, yU = 0.0;
        if (s >= 0) {
          const double Ep = a.energies[p] / g.Z[s];
          const double abb = g.ABB[s];
          double I_E, Q_E = 0.0;
          if (tab2) {
            // the walk's mu clamp applies to a leaf's first energy only
            const double v3 = erest ? (g.lgE[pl] / g.lzs[s]) * 0.001956951
                                    : g.lgE[pl] - g.lzs[s];
            MuStencil m1;
            if (p == 0 && g.clamp0[s]) {
              m1 = mu_stencil(a.atmos, as, abb, true);
            } else {
              if (s != mu_col) {
                ms = mu_stencil(a.atmos, as, abb, false);
                mu_col = s;
              }
              m1 = ms;
            }
            I_E = eval_num4d_e(a.atmos, as, a.atmos.I, m1, v3, 1.0);
            if (a.table_q) Q_E = eval_table_raw(a.atmos, as, a.table_q, m1, v3);
          } else {
            I_E = eval_bb(Ep, kT);
            if (burst) {
              I_E = I_E * (0.421 + 0.868 * abb);
              Q_E = (0.1171 * (abb - 1.) / (1. + 3.582 * abb)) * I_E;
            }
          }
          const double I_c = corr ? eval_bb(Ep, kT_c) * (kErg * kPlanck) : 0.0;
          yI = (I_E * norm - I_c) * g.GEOM[s];
          yQ = ((Q_E * g.c2chi[s]) * norm) * g.GEOM[s];
          yU = ((Q_E * g.s2chi[s]) * norm) * g.GEOM[s];
        }
        coI[pl * N_L + col].y = yI;
        coQ[pl * N_L + col].y = yQ;
        coU[pl * N_L + col].y = yU;
      }
      __syncthreads();
      // an exact power-of-two scale per (component, energy row)
      const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
      for (int r = warp; r < 3 * ne; r += kThreads / 32) {
        const int comp = r / ne, pl = r - comp * ne;
        const Piece *co = comp == 0 ? coI : (comp == 1 ? coQ : coU);
        double mx = 0.0;
        for (int col = lane; col < N_L; col += 32) mx = fmax(mx, fabs(co[pl * N_L + col].y));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        int ex = 0;
        if (mx > 0.0 && mx <= 1.7976931348623157e308) frexp(mx, &ex);
        if (lane == 0) (comp == 0 ? g.sc_exp : (comp == 1 ? scQ : scU))[pl] = ex;
      }
      __syncthreads();
      for (int t = threadIdx.x; t < 3 * ne * N_L; t += blockDim.x) {
        const int comp = t / (ne * N_L), u = t - comp * ne * N_L;
        Piece *co = comp == 0 ? coI : (comp == 1 ? coQ : coU);
        const int *sc = comp == 0 ? g.sc_exp : (comp == 1 ? scQ : scU);
        const double v = co[u].y;
        reinterpret_cast<PieceDF *>(co)[u].y = df_split(ldexp(v, -sc[u / N_L]));
      }
      __syncthreads();
      for (int t = threadIdx.x; t < 3 * ne * strips; t += blockDim.x) {
        const int comp = t / (ne * strips), u = t - comp * ne * strips;
        const int pl = u / strips, i0 = (u - pl * strips) * kStrip;
        const int i1 = min(i0 + kStrip, n_iv);
        PieceDF *yr = reinterpret_cast<PieceDF *>(comp == 0 ? coI : (comp == 1 ? coQ : coU)) +
                      pl * N_L;
        auto chord = [&](int j) -> DF {
          const int q = periodic_chord(j, N_L);
          return df_mul(df_sub(yr[q + 1].y, yr[q].y), g.ih[q]);
        };
        DF m0 = chord(i0 - 2), m1 = chord(i0 - 1), m2 = chord(i0), m3 = chord(i0 + 1),
           m4 = chord(i0 + 2);
        for (int iv = i0; iv < i1; iv++) {
          if (iv > i0) {
            m0 = m1; m1 = m2; m2 = m3; m3 = m4;
            m4 = chord(iv + 2);
          }
          DF k1, k2, k3;
          akima_piece_df(m0, m1, m2, m3, m4, g.ih[iv], g.ih2[iv], k1, k2, k3);
          yr[iv].k1 = k1;
          yr[iv].k2 = k2;
          yr[iv].k3 = k3;
        }
      }
      __syncthreads();
      // cell x phase accumulation (:612-650)
      const int ntasks = N_P * ((ne + kEPT - 1) / kEPT);
      for (int task = threadIdx.x; task < ntasks; task += blockDim.x) {
        const int k = task % N_P, pb = (task / N_P) * kEPT;
        const double phd = a.phases[k];
        const float ph = (float)phd;
        const float tp = (float)kTwoPi;
        const bool cached = M.S1 <= kMaxCellsF;
        const CellPhaseF cp{as.fphase, as.fphase_lo, N_L, as.fphase[0], as.fphase[N_L - 1], ph,
                            (float)(phd - (double)ph), tp, (float)(kTwoPi - (double)tp),
                            cached ? as.fcphi : nullptr, cached ? as.fcphi_lo : nullptr,
                            cellPhi};
        const AreaDF ar{cached ? as.fcarea : nullptr, cached ? as.fcarea_lo : nullptr, cellA};
        DF aI[kEPT], aQ[kEPT], aU[kEPT];
#pragma unroll
        for (int e = 0; e < kEPT; e++) aI[e] = aQ[e] = aU[e] = DF{0.0f, 0.0f};
        if (!cell_phase_sums_stokes(cp, ar, M.S1, rad, reinterpret_cast<const PieceDF *>(coI),
                                    reinterpret_cast<const PieceDF *>(coQ),
                                    reinterpret_cast<const PieceDF *>(coU), N_L, pb, ne, corr, aI,
                                    aQ, aU)) {
          atomicExch(&a.member_status[m], (int)kPulseFail);
          continue;
        }
#pragma unroll
        for (int e = 0; e < kEPT; e++) {
          if (pb + e < ne) {
            const int p = e0 + pb + e;
            part[(size_t)p * N_P + k] += ldexp(df_value(aI[e]), g.sc_exp[pb + e]);
            part[(size_t)(N_E + p) * N_P + k] += ldexp(df_value(aQ[e]), scQ[pb + e]);
            part[(size_t)(2 * N_E + p) * N_P + k] += ldexp(df_value(aU[e]), scU[pb + e]);
          }
        }
      }
      __syncthreads();
    }
  }
}

// the parallels' Stokes partials of each member in order, / (E keV) (:715-725)
__global__ void reduce_stokes_kernel(IntegrateArgs a) {
  const int m = blockIdx.y, comp = blockIdx.z;
  const MemberDesc M = a.members[m];
  const int n = a.N_E * a.N_P;
  double *out = comp == 0 ? a.flux : (comp == 1 ? a.flux_q : a.flux_u);
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int r = 0; r < M.S0; r++)
      s += a.partial[((size_t)(M.row_off + r) * 3 + comp) * n + t];
    const int p = t / a.N_P;
    out[M.flux_off + t] = s / (a.energies[p] * kKeV);
  }
}

// ---------------------------------------------------------------------------
// The split atmosphere's (mu, E) table at the first cell's (t_e, t_bb, tau)
// (integrator_for_azimuthal_invariance_split.pyx:270-275 calls
// hot_Num5D_split.pyx:267-481 once per (mu, E) node, mu outer, from a fresh
// evaluator).  The cached walk's state at each call is known in closed form:
// on t_e, t_bb, tau the first call moves the base node from 0 (clamping a
// query beyond the top of the grid on that call only) and later calls leave
// it; a query on the node mu_k or E_k has base node min(max(k - 2, 0), n - 4).
// On those two dimensions only the weight of the node itself is nonzero, so
// the 64 remaining terms are summed in the reference's order with its
// products (numerators, then inverse denominators, multiplied dimension by
// dimension) and without contraction, which reproduces its rounding.  One
// thread per (mu, E) node.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void walk_factors(const double *P, int b, double x, double D[4],
                                             double S[4]) {
  D[0] = x - P[b + 1]; D[0] *= x - P[b + 2]; D[0] *= x - P[b + 3];
  D[1] = x - P[b];     D[1] *= x - P[b + 2]; D[1] *= x - P[b + 3];
  D[2] = x - P[b];     D[2] *= x - P[b + 1]; D[2] *= x - P[b + 3];
  D[3] = x - P[b];     D[3] *= x - P[b + 1]; D[3] *= x - P[b + 2];
  S[0] = 1.0 / (P[b] - P[b + 1]);     S[0] /= P[b] - P[b + 2];     S[0] /= P[b] - P[b + 3];
  S[1] = 1.0 / (P[b + 1] - P[b]);     S[1] /= P[b + 1] - P[b + 2]; S[1] /= P[b + 1] - P[b + 3];
  S[2] = 1.0 / (P[b + 2] - P[b]);     S[2] /= P[b + 2] - P[b + 1]; S[2] /= P[b + 2] - P[b + 3];
  S[3] = 1.0 / (P[b + 3] - P[b]);     S[3] /= P[b + 3] - P[b + 1]; S[3] /= P[b + 3] - P[b + 2];
}

__global__ void split_reduce_kernel(SplitArgs a) {
  const int n3 = a.n[3], n4 = a.n[4];
  // the first call's walk on t_e, t_bb, tau from base node 0
  __shared__ int b[3];
  __shared__ double vfirst[3];
  if (threadIdx.x < 3) {
    const int d = threadIdx.x, n = a.n[d];
    const double *P = a.grid[d];
    double v = a.vec[d];
    int bn = 0;
    if (v > P[2] && n != 4) {
      for (int it = 0; it < n && v > P[bn + 2]; it++) {
        if (bn < n - 4) {
          bn++;
        } else {
          if (v >= P[n - 1]) v = P[n - 1];
          break;
        }
      }
    }
    b[d] = bn;
    vfirst[d] = v;
  }
  __syncthreads();
  const size_t s3 = (size_t)n4, s2 = (size_t)n3 * n4, s1 = (size_t)a.n[2] * s2,
               s0 = (size_t)a.n[1] * s1;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n3 * n4; t += gridDim.x * blockDim.x) {
    const int i = t / n4, j = t - i * n4;
    double D[3][4], S[3][4];
#pragma unroll
    for (int d = 0; d < 3; d++) walk_factors(a.grid[d], b[d], t == 0 ? vfirst[d] : a.vec[d], D[d], S[d]);
    const int b3 = min(max(i - 2, 0), n3 - 4), b4 = min(max(j - 2, 0), n4 - 4);
    double D3[4], S3[4], D4[4], S4[4];
    walk_factors(a.grid[3], b3, a.grid[3][i], D3, S3);
    walk_factors(a.grid[4], b4, a.grid[4][j], D4, S4);
    const double d3 = D3[i - b3], sp3 = S3[i - b3], d4 = D4[j - b4], sp4 = S4[j - b4];
    const double *T = a.I + (size_t)i * s3 + j;
    double I = 0.0;
    for (int k0 = 0; k0 < 4; k0++)
      for (int k1 = 0; k1 < 4; k1++)
        for (int k2 = 0; k2 < 4; k2++) {
          double dp = D[0][k0];
          dp = __dmul_rn(dp, D[1][k1]); dp = __dmul_rn(dp, D[2][k2]);
          dp = __dmul_rn(dp, d3); dp = __dmul_rn(dp, d4);
          double sp = S[0][k0];
          sp = __dmul_rn(sp, S[1][k1]); sp = __dmul_rn(sp, S[2][k2]);
          sp = __dmul_rn(sp, sp3); sp = __dmul_rn(sp, sp4);
          const double v = T[(size_t)(b[0] + k0) * s0 + (size_t)(b[1] + k1) * s1 +
                             (size_t)(b[2] + k2) * s2];
          I = __dadd_rn(I, __dmul_rn(__dmul_rn(dp, sp), v));
        }
    a.out[t] = I;
  }
}

// ---------------------------------------------------------------------------
// Work plan.  A parallel's cost is dominated by its images: each image
// repeats the profile columns, the splines and the cell x phase sums, and a
// star near the photon sphere (R -> 1.5 r_s) has rays deflected by several
// pi, so its parallels carry up to ~8 images against the usual 1-2.  The
// image count per parallel, ceil(max deflection / pi) (or the mesh's image
// order limit), is known only after the ray tables are built on the device,
// so the chunks are planned there:
//   cost(parallel) = images x (kCostImage + radiating cells) + kCostRow
// in units of one radiating cell's sums over one image (the fixed per-image
// work -- columns, splines, leaf geometry -- measured at about 28 cells, the
// per-parallel slab contraction at about 6), or 1 for a parallel with no
// radiating cell.  The consecutive parallels of each mesh are cut greedily
// into chunks of about total / target_chunks (a chunk closes before the
// parallel that would take it past the target), which bounds the count by
// 2 target_chunks + members.  The CTAs take the chunks heaviest first
// (a counting sort on floor(log2 cost)), so the few heavy chunks start in
// the first wave instead of forming the tail.  Chunk boundaries depend only
// on the costs, so every result is independent of the order in which the
// CTAs run.
// ---------------------------------------------------------------------------
constexpr float kCostImage = 28.0f;
constexpr float kCostRow = 6.0f;
constexpr int kPlanThreads = 1024;

__global__ void row_cost_kernel(IntegrateArgs a) {
  const int lane = threadIdx.x & 31;
  const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (row >= a.n_rows) return;
  const MemberDesc M = a.members[a.row_member[row]];
  const int64_t i = row - M.row_off;
  const int32_t *rad = a.radiates + M.cell_off + i * M.S1;
  int cr = 0;
  for (int j = lane; j < M.S1; j += 32) cr += (rad[j] == 1);
  for (int o = 16; o > 0; o >>= 1) cr += __shfl_xor_sync(0xffffffffu, cr, o);
  if (lane == 0) {
    float c = 1.0f;
    if (cr > 0) {
      const double md = a.maxDeflection[row];
      int io = M.image_order_limit > 0 ? M.image_order_limit
                                       : (md > 0.0 ? (int)ceil(md / kPi) : 1);
      io = max(1, min(io, 64));
      c = (float)io * (kCostImage + (float)cr) + kCostRow;
    }
    a.row_cost[row] = c;
  }
}

// chunks of mesh m for a target cost: count (write == false) or write them
// from index c0; returns the count
__device__ int plan_mesh(const IntegrateArgs &a, int m, double target, bool write, int c0) {
  const MemberDesc M = a.members[m];
  int n = 0;
  double acc = 0.0;
  int64_t start = M.row_off;
  for (int64_t s = 0; s < M.S0; s++) {
    const int64_t row = M.row_off + s;
    const double c = a.row_cost[row];
    if (acc > 0.0 && acc + c > target) {
      if (write) {
        a.chunk_r0[c0 + n] = start;
        a.chunk_r1[c0 + n] = row;
        a.chunk_cost[c0 + n] = (float)acc;
      }
      n++;
      acc = 0.0;
      start = row;
    }
    acc += c;
  }
  if (M.S0 > 0) {
    if (write) {
      a.chunk_r0[c0 + n] = start;
      a.chunk_r1[c0 + n] = M.row_off + M.S0;
      a.chunk_cost[c0 + n] = (float)acc;
    }
    n++;
  }
  return n;
}

// exclusive scan of per-thread values over the block; returns the total
__device__ int block_exclusive_scan(int v, int *s_buf, int &excl) {
  const int t = threadIdx.x;
  s_buf[t] = v;
  __syncthreads();
  for (int o = 1; o < kPlanThreads; o <<= 1) {
    const int x = t >= o ? s_buf[t - o] : 0;
    __syncthreads();
    s_buf[t] += x;
    __syncthreads();
  }
  excl = s_buf[t] - v;
  const int total = s_buf[kPlanThreads - 1];
  __syncthreads();
  return total;
}

// one CTA of kPlanThreads threads
__global__ void __launch_bounds__(kPlanThreads) plan_chunks_kernel(IntegrateArgs a) {
  __shared__ double s_sum[kPlanThreads];
  __shared__ int s_scan[kPlanThreads];
  __shared__ int s_hist[64], s_cur[64];
  const int t = threadIdx.x;
  // total cost (fixed summation order)
  double sum = 0.0;
  for (int64_t r = t; r < a.n_rows; r += kPlanThreads) sum += a.row_cost[r];
  s_sum[t] = sum;
  __syncthreads();
  for (int o = kPlanThreads / 2; o > 0; o >>= 1) {
    if (t < o) s_sum[t] += s_sum[t + o];
    __syncthreads();
  }
  double target = fmax(1.0, s_sum[0] / (double)max(1, a.target_chunks));
  // meshes [m0, m1) of this thread
  const int per = (a.n_members + kPlanThreads - 1) / kPlanThreads;
  const int m0 = min(a.n_members, t * per), m1 = min(a.n_members, m0 + per);
  int excl = 0, total = 0;
  for (int pass = 0; pass < 2; pass++) {
    int cnt = 0;
    for (int m = m0; m < m1; m++) cnt += plan_mesh(a, m, target, false, 0);
    total = block_exclusive_scan(cnt, s_scan, excl);
    if (total <= a.max_chunks) break;
    // the bound cannot be exceeded in exact arithmetic; should rounding ever
    // do it, one chunk per mesh fits
    target = 1.0e300;
  }
  int c = excl;
  for (int m = m0; m < m1; m++) {
    a.chunk_first[m] = c;
    c += plan_mesh(a, m, target, true, c);
  }
  if (t == 0) {
    a.chunk_first[a.n_members] = total;
    *a.chunk_count = total;
  }
  // heaviest first: counting sort on floor(log2 cost), descending
  if (t < 64) s_hist[t] = 0;
  __syncthreads();
  for (int k = t; k < total; k += kPlanThreads) {
    int e = 0;
    frexpf(a.chunk_cost[k], &e);
    atomicAdd(&s_hist[min(63, max(0, e))], 1);
  }
  __syncthreads();
  if (t == 0) {
    int run = 0;
    for (int b = 63; b >= 0; b--) {
      s_cur[b] = run;
      run += s_hist[b];
    }
  }
  __syncthreads();
  for (int k = t; k < total; k += kPlanThreads) {
    int e = 0;
    frexpf(a.chunk_cost[k], &e);
    a.chunk_order[atomicAdd(&s_cur[min(63, max(0, e))], 1)] = k;
  }
}

// ordered reduction of the chunk partials and the 1/(E keV) factor (:605-612)
__global__ void reduce_flux_kernel(IntegrateArgs a) {
  const int m = blockIdx.y;
  const MemberDesc M = a.members[m];
  const int n = a.N_E * a.N_P;
  const int c0 = a.chunk_first[m], c1 = a.chunk_first[m + 1];
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int c = c0; c < c1; c++)
      s += a.partial2 ? a.partial[(size_t)c * n + t] + a.partial2[(size_t)c * n + t]
                      : a.partial[(size_t)c * n + t];
    const int p = t / a.N_P;
    a.flux[M.flux_off + t] = s / (a.energies[p] * kKeV);
  }
}

}  // namespace

// each parallel's entry state of a table atmosphere's mu walk: the
// geometry pre-pass, then the per-mesh scan in call order
static void launch_table_state(const IntegrateArgs &a, cudaStream_t st) {
  const size_t pre_smem = geometry_bytes(a.N_L, a.N_R);
  static bool pre_attr = false;
  if (!pre_attr) {
    cudaFuncSetAttribute(num4d_prepass_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         200 * 1024);
    pre_attr = true;
  }
  num4d_prepass_kernel<<<(unsigned)a.n_rows, 128, pre_smem, st>>>(a);
  num4d_scan_kernel<<<(a.n_members + 127) / 128, 128, 0, st>>>(a);
}

size_t integrate_wsum_bytes(int N_P, int max_cells, int *w_cap) {
  const int cap = (max_cells + 1) / 2;
  if (w_cap) *w_cap = cap;
  return integrate_wsum_bytes_dev(N_P, cap);
}

void launch_integrate(const IntegrateArgs &a, cudaStream_t st) {
  if (a.n_members <= 0) return;
  const int pb = a.mixed ? (int)sizeof(PieceT<float>) : (int)sizeof(PieceT<double>);
  Layout L = a.atmos.I ? make_layout(a.N_L, a.N_P, a.N_E, a.atmos.nmu, a.atmos.nE, pb, a.N_R)
                       : make_layout(a.N_L, a.N_P, a.N_E, 0, 0, pb, a.N_R);
  // run counts [2][N_P] and piece classes [EC][N_L] after the layout
  const size_t bytes = L.bytes + (size_t)2 * a.N_P * sizeof(int) + (size_t)L.EC * a.N_L + 16;
  // the work plan from the parallels' costs (needs the ray tables)
  if (a.n_rows > 0) row_cost_kernel<<<(unsigned)((a.n_rows * 32 + 255) / 256), 256, 0, st>>>(a);
  plan_chunks_kernel<<<1, kPlanThreads, 0, st>>>(a);
  // the attribute is per device: set it on every launch (cheap)
  if (a.atmos.I != nullptr) launch_table_state(a, st);
  if (a.mixed) {
    cudaFuncSetAttribute(integrate_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         200 * 1024);
    integrate_kernel<float><<<a.max_chunks, kThreads, bytes, st>>>(a);
  } else {
    cudaFuncSetAttribute(integrate_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         200 * 1024);
    integrate_kernel<double><<<a.max_chunks, kThreads, bytes, st>>>(a);
  }
  dim3 grid((a.N_E * a.N_P + 255) / 256, a.n_members);
  reduce_flux_kernel<<<grid, 256, 0, st>>>(a);
}


void launch_split_reduce(const SplitArgs &a, cudaStream_t st) {
  const int n = a.n[3] * a.n[4];
  split_reduce_kernel<<<(n + 255) / 256, 256, 0, st>>>(a);
}

size_t stokes_smem_bytes(int N_L, int N_P, int N_E, int N_R, int nmu, int nE) {
  return stokes_smem(N_L, N_P, N_E, N_R, nmu, nE);
}

size_t stokes_partial_doubles(const IntegrateArgs &a) {
  return (size_t)a.n_rows * 3 * a.N_E * a.N_P;
}

int launch_stokes(const IntegrateArgs &a, cudaStream_t st) {
  if (a.n_members <= 0) return 0;
  const int nmu = a.atmos.I ? a.atmos.nmu : 0, nE = a.atmos.I ? a.atmos.nE : 0;
  const size_t smem = stokes_smem(a.N_L, a.N_P, a.N_E, a.N_R, nmu, nE);
  if (smem > 227 * 1024) return -2;
  if (a.atmos.I != nullptr) launch_table_state(a, st);
  if (cudaFuncSetAttribute(stokes_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess)
    return -5;
  stokes_kernel<<<(unsigned)a.n_rows, kThreads, smem, st>>>(a);
  const int n = a.N_E * a.N_P;
  dim3 grid((n + 255) / 256, a.n_members, 3);
  reduce_stokes_kernel<<<grid, 256, 0, st>>>(a);
  return cudaGetLastError() == cudaSuccess ? 0 : -5;
}

}  // namespace xg
