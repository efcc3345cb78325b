// elsewhere.cu -- the photosphere elsewhere: the time-invariant integrator
// over a closed cell mesh, replacing
// xpsi/cellmesh/integrator_for_time_invariance.pyx:59-338 with the blackbody
// (hot_BB.pyx:54-98) and numerical 4-D (hot_Num4D.pyx:248-461) atmospheres
// that elsewhere_wrapper.pyx:22-96 dispatches to.
//
// Work decomposition (one CTA per parallel of one closed mesh):
//   1. the parallel's ray tables are staged in shared memory and the first
//      ray deflected beyond pi/2 is found (:197-213);
//   2. one thread per cell: for every image up to the image order, the
//      deflection, cos alpha and d cos alpha / d psi from the Steffen tables,
//      the Doppler factor and mu (:215-296) -> per visible image the triple
//      (Z, mu eta, geometric factor), kept in shared memory in the
//      reference's call order (cell, then image);
//   3. one thread per energy walks the triples in that order and sums
//      I(E / Z, mu eta) x geometric factor (:298-307), so each parallel's sum
//      is formed in a fixed order;
//   4. a second kernel adds the parallels in order and applies
//      cellArea x norm / (E keV) (:318-323).
//
// Num4D call history.  The reference evaluator keeps its stencil base node
// between calls and clamps a coordinate outside the table only on the call
// that moves the node (hot_Num4D.pyx:300-351).  Given the previous call's
// coordinates, the base node and the clamp of the next call follow exactly;
// step 3 visits the evaluations in the reference's single-thread call order
// and carries the previous call's coordinates along (the first call of a
// parallel takes them from the last visible image of the parallels before
// it, recomputed in step 2b).
#include "common.cuh"
#include "kernels.h"
#include "num4d_walk.cuh"

namespace xg {

namespace {

constexpr int kElseThreads = 128;

struct ElseRow {
  const double *D, *CA;  // ray tables of the parallel (deflection, cos alpha)
  int N_R, jalt;         // rays; first ray with deflection > pi/2
  double Grav_z, cos_gamma, sin_gamma, cos_th, sin_th, th_over_pi, beta, Lorentz, maxDefl;
};

__device__ ElseRow make_row(const ElsewhereArgs &a, int64_t row, double omega,
                            const double *D, const double *CA, int jalt) {
  ElseRow r;
  r.D = D;
  r.CA = CA;
  r.N_R = a.N_R;
  r.jalt = jalt;
  r.Grav_z = sqrt(1.0 - a.u[row]);
  r.cos_gamma = a.cos_gamma[row];
  r.sin_gamma = sqrt(1.0 - r.cos_gamma * r.cos_gamma);
  const double th = a.theta0[row];
  r.cos_th = cos(th);
  r.sin_th = sin(th);
  r.th_over_pi = th / kPi;
  r.beta = a.radius[row] * omega * r.sin_th / (kC * r.Grav_z);
  r.Lorentz = sqrt(1.0 - r.beta * r.beta);
  r.maxDefl = a.maxDeflection[row];
  return r;
}

// the visible images of one cell at azimuth ph (:215-296): writes up to IO
// triples (Z, mu eta, geometric factor) and returns how many, or -1 when a
// deflection falls outside the ray table (the reference's terminate)
__device__ int cell_images(const ElseRow &r, double cos_i, double sin_i, double incl, double ph,
                           int IO, double *Z, double *ABB, double *GEOM, int stride) {
  const double c_psi0 = cos_i * r.cos_th + sin_i * r.sin_th * cos(ph);
  const double psi0 = acos(c_psi0);
  MainX mx{r.D};
  ArrY my{r.CA};
  AltX ax{r.D, r.jalt};
  AltY ay{r.CA, r.jalt};
  const double alt_xmin = cos(r.D[r.jalt]);
  int n = 0;
  for (int I = 0; I < IO; I++) {
    double cos_psi = c_psi0;
    double psi = image_deflection(I, psi0);
    double sin_psi = sin(psi);
    if (!are_equal(psi, 0.0) && are_equal(sin_psi, 0.0)) {  // :231-244
      const double _i = (cos_i >= 0.0) ? incl + incl * 1.0e-6 : incl - incl * 1.0e-6;
      cos_psi = cos(_i) * r.cos_th + sin(_i) * r.sin_th * cos(ph);
      psi = image_deflection(I, acos(cos_psi));
      sin_psi = sin(psi);
    }
    if (psi > r.maxDefl) break;
    if (psi < r.D[0] || psi > r.D[r.N_R - 1]) return -1;
    const bool use_alt = psi <= kHalfPi && cos_psi >= alt_xmin;
    double cos_a, deriv;
    if (use_alt) steffen_eval(ax, ay, r.jalt + 1, cos_psi, &cos_a, &deriv);
    else steffen_eval(mx, my, r.N_R, psi, &cos_a, &deriv);
    const double sin_alpha = sqrt(1.0 - cos_a * cos_a);
    double mu = cos_a * r.cos_gamma;
    if (!are_equal(psi, 0.0)) {
      const double cos_delta = (cos_i - r.cos_th * cos_psi) / (r.sin_th * sin_psi);
      if (r.th_over_pi < 0.5) mu = mu + sin_alpha * r.sin_gamma * cos_delta;
      else mu = mu - sin_alpha * r.sin_gamma * cos_delta;
    }
    if (!(mu > 0.0)) continue;
    double eta;
    if (!are_equal(sin_psi, 0.0)) {
      const double cos_xi = sin_alpha * sin_i * sin(ph) / sin_psi;
      eta = r.Lorentz / (1.0 + r.beta * cos_xi);
    } else {
      eta = r.Lorentz;
    }
    if (!use_alt) deriv = exp(log(fabs(deriv)) - log(fabs(sin_psi)));
    Z[n * stride] = eta * r.Grav_z;
    ABB[n * stride] = mu * eta;
    GEOM[n * stride] = mu * fabs(deriv) * r.Grav_z * eta * eta * eta;
    n++;
  }
  return n;
}

// first ray of a table with deflection > pi/2 (the reference's unbounded
// `while deflection[j] <= pi/2` scan, stopped at the last ray).  The first
// ray is radial (deflection 0), so the answer is >= 1 for every table the
// ray tracer makes; it is held there for any other input, so that the
// reversed table always has two knots.
__device__ int first_beyond_half_pi(const double *D, int N_R, int *s_j) {
  if (threadIdx.x == 0) *s_j = N_R - 1;
  __syncthreads();
  for (int t = threadIdx.x; t < N_R; t += blockDim.x)
    if (D[t] > kHalfPi) atomicMin(s_j, t);
  __syncthreads();
  const int j = *s_j < 1 ? 1 : *s_j;
  __syncthreads();
  return j;
}

__global__ void __launch_bounds__(kElseThreads) elsewhere_row_kernel(ElsewhereArgs a) {
  const int64_t row = blockIdx.x;
  const int m = a.row_mesh[row];
  const ElseMeshDesc M = a.meshes[m];
  const int S = M.S, N_R = a.N_R, N_E = a.N_E;
  const int i_loc = (int)(row - M.row_off);
  const int cap = a.max_images;
  const bool num4d = M.atm_ext == 2;
  extern __shared__ double sm[];
  double *sD = sm, *sCA = sD + N_R;
  double *eZ = sCA + N_R, *eA = eZ + (size_t)a.max_S * cap, *eG = eA + (size_t)a.max_S * cap;
  double *cT = eG + (size_t)a.max_S * cap, *cg = cT + a.max_S;  // per cell: log T (or kT), log g
  int *cnt = reinterpret_cast<int *>(cg + a.max_S);
  __shared__ int s_jalt, s_term, s_key;
  __shared__ double s_prev[4];

  const double *Dg = a.deflection + row * N_R, *CAg = a.cos_alpha + row * N_R;
  for (int t = threadIdx.x; t < N_R; t += blockDim.x) {
    sD[t] = Dg[t];
    sCA[t] = CAg[t];
  }
  if (threadIdx.x == 0) s_term = 0;
  __syncthreads();
  const int jalt = first_beyond_half_pi(sD, N_R, &s_jalt);
  const ElseRow r = make_row(a, row, M.omega, sD, sCA, jalt);
  const int IO = M.image_order_limit > 0 ? M.image_order_limit : (int)ceil(r.maxDefl / kPi);
  double *fout = a.row_flux + row * N_E;
  if (IO > cap) {  // more images than the launch holds: reported, not computed
    if (threadIdx.x == 0) a.status[m] = kBadInput;
    for (int e = threadIdx.x; e < N_E; e += blockDim.x) fout[e] = 0.0;
    return;
  }
  const double cos_i = cos(M.inclination), sin_i = sin(M.inclination);
  const int64_t c0 = M.cell_off + (int64_t)i_loc * S;
  for (int j = threadIdx.x; j < S; j += blockDim.x) {
    const int n = cell_images(r, cos_i, sin_i, M.inclination, a.phi[c0 + j], IO, eZ + j,
                              eA + j, eG + j, a.max_S);
    if (n < 0) s_term = 1;
    cnt[j] = n < 0 ? 0 : n;
    const double *vec = a.params + (c0 + j) * a.n_params;
    cT[j] = num4d ? vec[0] : (kKB / kKeV) * pow(10.0, vec[0]);
    cg[j] = num4d ? vec[1] : 0.0;
  }
  __syncthreads();
  if (s_term) {
    if (threadIdx.x == 0) a.status[m] = kPulseFail;
    for (int e = threadIdx.x; e < N_E; e += blockDim.x) fout[e] = 0.0;
    return;
  }

  // 2b. Num4D: the coordinates of the last evaluation before this parallel
  // (the last visible image of the nearest earlier parallel that has one)
  if (num4d) {
    if (threadIdx.x == 0) {
      s_prev[0] = s_prev[1] = s_prev[2] = s_prev[3] = -INFINITY;  // a fresh walk (base 0)
    }
    for (int rr = i_loc - 1; rr >= 0; rr--) {
      const int64_t prow = M.row_off + rr;
      const double *pD = a.deflection + prow * N_R, *pCA = a.cos_alpha + prow * N_R;
      if (threadIdx.x == 0) s_key = -1;
      const int pj = first_beyond_half_pi(pD, N_R, &s_jalt);
      const ElseRow pr = make_row(a, prow, M.omega, pD, pCA, pj);
      const int pIO = M.image_order_limit > 0 ? M.image_order_limit
                                              : (int)ceil(pr.maxDefl / kPi);
      const int64_t pc0 = M.cell_off + (int64_t)rr * S;
      double z[16], ab[16], ge[16];
      for (int j = threadIdx.x; j < S; j += blockDim.x) {
        const int n = pIO <= 16 ? cell_images(pr, cos_i, sin_i, M.inclination, a.phi[pc0 + j],
                                              pIO, z, ab, ge, 1)
                                : 0;
        if (n > 0) atomicMax(&s_key, j * 16 + n - 1);
      }
      __syncthreads();
      const int key = s_key;
      if (key >= 0 && threadIdx.x == 0) {
        const int j = key / 16, k = key % 16;
        const int n = cell_images(pr, cos_i, sin_i, M.inclination, a.phi[pc0 + j], pIO, z, ab,
                                  ge, 1);
        (void)n;
        const double *vec = a.params + (pc0 + j) * a.n_params;
        const double E_eff = (kKB / kKeV) * pow(10.0, vec[0]);
        s_prev[0] = vec[0];
        s_prev[1] = vec[1];
        s_prev[2] = ab[k];
        s_prev[3] = log10((a.energies[N_E - 1] / z[k]) / E_eff);
      }
      __syncthreads();
      if (key >= 0) break;
    }
    __syncthreads();
  }

  // 3. one thread per energy, the triples in call order (:298-307)
  for (int e = threadIdx.x; e < N_E; e += blockDim.x) {
    const double E = a.energies[e];
    double acc = 0.0;
    if (!num4d) {
      for (int j = 0; j < S; j++) {
        const int n = cnt[j];
        const double kT = cT[j];
        for (int k = 0; k < n; k++) {
          const int s = k * a.max_S + j;
          acc += eval_bb(E / eZ[s], kT) * eG[s];
        }
      }
    } else {
      const double Eprev = e > 0 ? a.energies[e - 1] : a.energies[N_E - 1];
      double vp[4] = {s_prev[0], s_prev[1], s_prev[2], s_prev[3]};
      for (int j = 0; j < S; j++) {
        const int n = cnt[j];
        const double v0 = cT[j], v1 = cg[j];
        const double E_eff = (kKB / kKeV) * pow(10.0, v0);
        for (int k = 0; k < n; k++) {
          const int s = k * a.max_S + j;
          const double Z = eZ[s], ab = eA[s];
          const double v3 = log10((E / Z) / E_eff);
          if (e > 0) {  // the previous call: this image at the previous energy
            vp[0] = v0; vp[1] = v1; vp[2] = ab;
            vp[3] = log10((Eprev / Z) / E_eff);
          }
          acc += num4d_walk(a.atmos, vp, v0, v1, ab, v3) * eG[s];
          if (e == 0) {  // the next image's previous call: this one at the last energy
            vp[0] = v0; vp[1] = v1; vp[2] = ab;
            vp[3] = log10((Eprev / Z) / E_eff);
          }
        }
      }
    }
    fout[e] = acc;
  }
}

// :312-323: the parallels in order, times cellArea x norm / (E keV); with a
// signal given, the spectrum is also added to every phase column of that
// mesh's signal [N_E][signal_N_P] (Photosphere.py:588-592)
__global__ void elsewhere_finish_kernel(ElsewhereArgs a) {
  const int m = blockIdx.x;
  const ElseMeshDesc M = a.meshes[m];
  const double norm = (M.atm_ext == 2) ? kErg / kHKeV : kErg * kPlanck;
  for (int e = threadIdx.x; e < a.N_E; e += blockDim.x) {
    double s = 0.0;
    for (int i = 0; i < M.S; i++) s += a.row_flux[(int64_t)(M.row_off + i) * a.N_E + e];
    const double f = s * (M.cellArea * norm / (a.energies[e] * kKeV));
    a.flux[(int64_t)m * a.N_E + e] = f;
    if (a.signal != nullptr && a.status[m] == 0) {
      double *row = a.signal + (int64_t)m * a.signal_stride + (int64_t)e * a.signal_N_P;
      for (int p = 0; p < a.signal_N_P; p++) row[p] += f;
    }
  }
}

}  // namespace

size_t elsewhere_smem_bytes(int N_R, int max_S, int max_images) {
  return (size_t)(2 * N_R + 3 * (size_t)max_S * max_images + 2 * max_S) * sizeof(double) +
         (size_t)max_S * sizeof(int);
}

int launch_elsewhere(const ElsewhereArgs &a, cudaStream_t st) {
  if (a.n_rows <= 0 || a.n_meshes <= 0) return 0;
  const size_t smem = elsewhere_smem_bytes(a.N_R, a.max_S, a.max_images);
  if (smem > 227 * 1024) return -2;
  if (cudaFuncSetAttribute(elsewhere_row_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess)
    return -5;
  elsewhere_row_kernel<<<(unsigned)a.n_rows, kElseThreads, smem, st>>>(a);
  elsewhere_finish_kernel<<<a.n_meshes, 128, 0, st>>>(a);
  return cudaGetLastError() == cudaSuccess ? 0 : -5;
}

}  // namespace xg
