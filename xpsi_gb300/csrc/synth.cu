// synth.cu -- data synthesis on the GPU: expected counts per (channel, phase
// bin) and their Poisson realisations, replacing
//   xpsi/tools/compute_expected_counts.pyx:66-197 (compute_expected_counts),
//   xpsi/tools/phase_integrator.pyx:23-121 (phase_integrator) and the draws of
//   xpsi/tools/synthesise.pyx:35-276 (synthesise_exposure,
//   synthesise_given_total_count_number), and the Gaussian likelihoods of
//   xpsi/likelihoods/_gaussian_likelihood_given_background_IQU.pyx and
//   _gaussian_likelihood_QnUn.pyx.
//
// Phase-bin integrals: one warp per (signal, channel) row, lanes over the
// bins, each bin the exact integral of the Akima-periodic interpolant of the
// row over the phase-shifted bin (wrapped into [0, 1)), with the reference's
// positive-part rules.
//
// Gaussian likelihoods of polarimetry: one warp per data set, the terms
// summed row by row in column order.
//
// Poisson draws: element i of a launch with key `seed` draws from the
// counter-based generator Philox4x32-10 (Salmon, Moraes, Dror and Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC'11) at counter
// (offset + i, attempt), so a draw depends only on (seed, offset + i) and not
// on how elements are batched.  Means below 10 are inverted by sequential
// search of the cumulative distribution; larger means use the transformed
// rejection with squeeze of Hormann ("The transformed rejection method for
// generating Poisson random variables", Insurance: Mathematics and Economics
// 12, 1993), PTRS.  Every loop is bounded.  The realisations follow the
// Poisson law as GSL's gsl_ran_poisson does; they are not GSL's stream.
#include <algorithm>

#include "common.cuh"
#include "kernels.h"

namespace xg {

namespace {

constexpr int kSynWarps = 4;

// ---------------------------------------------------------------- Philox
struct U4 {
  uint32_t x, y, z, w;
};

__device__ __forceinline__ U4 philox_round(U4 c, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t hi0 = __umulhi(M0, c.x), lo0 = M0 * c.x;
  const uint32_t hi1 = __umulhi(M1, c.z), lo1 = M1 * c.z;
  return U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
}

__device__ __forceinline__ U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; r++) {
    c = philox_round(c, k0, k1);
    k0 += W0;
    k1 += W1;
  }
  return c;
}

// uniform doubles in [0, 1) with 53 random bits, two per generator call
struct UniformStream {
  uint64_t elem;
  uint32_t k0, k1, n;
  double spare;
  bool have;
  __device__ double next() {
    if (have) {
      have = false;
      return spare;
    }
    const U4 r = philox4x32_10(U4{(uint32_t)elem, (uint32_t)(elem >> 32), n, 0x5eed5eedu}, k0, k1);
    n++;
    const double s = 1.0 / 9007199254740992.0;  // 2^-53
    const double a = (double)(((uint64_t)(r.x >> 5) << 26) | (r.y >> 6)) * s;
    spare = (double)(((uint64_t)(r.z >> 5) << 26) | (r.w >> 6)) * s;
    have = true;
    return a;
  }
};

__device__ double poisson_draw(double mu, UniformStream &u, int *fail) {
  if (!(mu > 0.0)) return (mu == 0.0) ? 0.0 : nan("");
  if (mu < 10.0) {
    // inversion: the smallest k with F(k) >= U
    const double U = u.next();
    double p = exp(-mu), F = p;
    int k = 0;
    while (U > F && k < 1000) {
      k++;
      p *= mu / (double)k;
      F += p;
    }
    return (double)k;
  }
  // PTRS (Hormann 1993): transformed rejection with squeeze
  const double slam = sqrt(mu), loglam = log(mu);
  const double b = 0.931 + 2.53 * slam;
  const double a = -0.059 + 0.02483 * b;
  const double invalpha = 1.1239 + 1.1328 / (b - 3.4);
  const double vr = 0.9277 - 3.6224 / (b - 2.0);
  for (int attempt = 0; attempt < 10000; attempt++) {
    const double U = u.next() - 0.5;
    const double V = u.next();
    const double us = 0.5 - fabs(U);
    const double k = floor((2.0 * a / us + b) * U + mu + 0.43);
    if (us >= 0.07 && V <= vr) return k;
    if (k < 0.0 || (us < 0.013 && V > us)) continue;
    if (log(V) + log(invalpha) - log(a / (us * us) + b) <= -mu + k * loglam - lgamma(k + 1.0))
      return k;
  }
  *fail = 1;
  return floor(mu + 0.5);
}

__global__ void poisson_kernel(int64_t n, const double *mean, double *out, uint64_t seed,
                               uint64_t offset, int32_t *fail) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    UniformStream u{offset + (uint64_t)i, (uint32_t)seed, (uint32_t)(seed >> 32), 0u, 0.0, false};
    int f = 0;
    out[i] = poisson_draw(mean[i], u, &f);
    if (f) atomicExch(fail, 1);
  }
}

// ------------------------------------------------- phase-bin integrals
// one bin of one component (compute_expected_counts.pyx:127-162 with
// `exact_cycle` false; phase_integrator.pyx:93-115 with it true, where a full
// cycle is recognised by exact equality and the first branch assigns)
__device__ __forceinline__ double bin_integral(const double *ph, const double *y, int n, double a,
                                               double b, bool neg, bool exact_cycle) {
  const bool full = exact_cycle ? (b - a == 1.0) : are_equal(b - a, 1.0);
  if (full) {
    a = 0.0;
    b = 1.0;
  } else {
    a -= floor(a);
    b -= floor(b);
  }
  double s = 0.0;
  if (a < b) {
    const double v = akima_periodic_integral(ph, y, n, a, b);
    if (v > 0.0 || neg) s += v;
  } else {
    double v = akima_periodic_integral(ph, y, n, a, 1.0);
    if (v > 0.0 || neg) s += v;
    v = akima_periodic_integral(ph, y, n, 0.0, b);
    if (v > 0.0 || neg) s += v;
  }
  return s;
}

// expected counts of one (set, channel) row: exposure x (sum over components
// of the star rate, clamped at zero, + background rate)
__global__ void __launch_bounds__(32 * kSynWarps) expected_counts_kernel(ExpectedArgs a) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = (int64_t)blockIdx.x * kSynWarps + (threadIdx.x >> 5);
  if (gw >= (int64_t)a.n_sets * a.K) return;
  const int s = (int)(gw / a.K), ch = (int)(gw - (int64_t)s * a.K);
  for (int j = lane; j < a.B; j += 32) {
    double st = 0.0;
    for (int h = 0; h < a.H; h++) {
      const CompDesc c = a.comps[(int64_t)s * a.H + h];
      const double *row = c.signal + (int64_t)ch * c.ld;
      if (c.n > 1) {
        st += bin_integral(c.phases, row, c.n, a.phase_edges[j] + c.shift,
                           a.phase_edges[j + 1] + c.shift, a.allow_negative[h] == 1, false);
      } else if (j == 0) {
        st = row[0];  // :161-162
      }
    }
    if (st < 0.0) st = 0.0;  // :164-166
    const double bg = a.background ? a.background[(int64_t)ch * a.B + j] : 0.0;
    double e = st + bg;
    e *= a.exposure;
    a.out[((int64_t)s * a.K + ch) * a.B + j] = e;
  }
}

// phase_integrator.pyx:23-121 for rows of one signal
__global__ void __launch_bounds__(32 * kSynWarps) phase_integrator_kernel(PhaseIntArgs a) {
  const int lane = threadIdx.x & 31;
  const int64_t row = (int64_t)blockIdx.x * kSynWarps + (threadIdx.x >> 5);
  if (row >= a.rows) return;
  const double *y = a.signal + row * a.n_phases;
  for (int j = lane; j < a.B; j += 32) {
    double v = bin_integral(a.signal_phases, y, a.n_phases, a.phase_edges[j] + a.shift,
                            a.phase_edges[j + 1] + a.shift, a.allow_negative, true);
    v *= a.exposure;
    a.out[row * a.B + j] = v;
  }
}

// Gaussian log-likelihood of one data set (the polarimetry likelihoods,
// _gaussian_likelihood_given_background_IQU.pyx:70-78 and
// _gaussian_likelihood_QnUn.pyx:31-36): -sum over (row, column) of
// (model - data)^2 / (2 sigma^2) + log(2 pi sigma^2) / 2.  One warp per data
// set: lane r sums rows r, r+32, ... in column order, the lanes' sums are
// added in row order by lane 0.
__global__ void gaussian_kernel(int n_sets, int rows, int cols, const double *model,
                                int64_t model_set_stride, int64_t model_row_stride,
                                const double *data, const double *errors, double *loglike) {
  const int lane = threadIdx.x & 31;
  const int set = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (set >= n_sets) return;
  const double *mdl = model + set * model_set_stride;
  double rowsum[8];
  double part = 0.0;
  int nr = 0;
  for (int i = lane; i < rows; i += 32) {
    double s = 0.0;
    for (int j = 0; j < cols; j++) {
      const double sig2 = pow(errors[(int64_t)i * cols + j], 2.0);
      const double norm = 0.5 * log(2.0 * kPi * sig2);
      const double d = mdl[(int64_t)i * model_row_stride + j] - data[(int64_t)i * cols + j];
      s += d * d / (2.0 * sig2) + norm;
    }
    if (nr < 8) rowsum[nr] = s;
    else part += s;
    nr++;
  }
  // rows in order: row i lives in lane i % 32, slot i / 32
  __shared__ double red[8][32 * 8];
  const int w = threadIdx.x >> 5;
  for (int k = 0; k < 8; k++) red[w][k * 32 + lane] = (k < nr && k < 8) ? rowsum[k] : 0.0;
  __syncwarp();
  const double extra = part;
  double tot_extra = extra;
  for (int o = 16; o > 0; o >>= 1) tot_extra += __shfl_xor_sync(0xffffffffu, tot_extra, o);
  if (lane == 0) {
    double L = 0.0;
    const int first = min(rows, 8 * 32);
    for (int i = 0; i < first; i++) L -= red[w][(i / 32) * 32 + (i % 32)];
    L -= tot_extra;
    loglike[set] = L;
  }
}

// one warp per (set, channel): lanes over the phase bins, the terms
// reduced by a fixed butterfly
__global__ void __launch_bounds__(32 * kSynWarps) poisson_channel_kernel(PoissonArgs a) {
  const int lane = threadIdx.x & 31;
  const int64_t w = (int64_t)blockIdx.x * kSynWarps + (threadIdx.x >> 5);
  if (w >= (int64_t)a.n_sets * a.K) return;
  const int i = (int)(w % a.K);
  const double *E = a.expected + w * a.B;
  const double *d = a.counts + (int64_t)i * a.B;
  double s = 0.0;
  int pen = 0;
  for (int j = lane; j < a.B; j += 32) {
    const double e = E[j], c = d[j];
    if (e > 0.0) s += c * log(e) - e;
    else if (!(c == 0.0 && e == 0.0)) pen++;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_xor_sync(0xffffffffu, s, o);
    pen += __shfl_xor_sync(0xffffffffu, pen, o);
  }
  if (lane == 0) {
    a.chan_ll[w] = s;
    a.chan_pen[w] = pen;
  }
}

// per set: the channels in order (constant term, then the channel's sum)
__global__ void poisson_finish_kernel(PoissonArgs a) {
  const int set = blockIdx.x * blockDim.x + threadIdx.x;
  if (set >= a.n_sets) return;
  double L = 0.0;
  int pen = 0;
  for (int i = 0; i < a.K; i++) {
    if (a.precomp) L += a.precomp[i];
    L += a.chan_ll[(int64_t)set * a.K + i];
    pen += a.chan_pen[(int64_t)set * a.K + i];
  }
  a.loglike[set] = L;
  a.n_penalty[set] = pen;
}

}  // namespace

void launch_poisson_loglike(const PoissonArgs &a, cudaStream_t st) {
  const int64_t warps = (int64_t)a.n_sets * a.K;
  if (warps <= 0) return;
  poisson_channel_kernel<<<(unsigned)((warps + kSynWarps - 1) / kSynWarps), 32 * kSynWarps, 0,
                           st>>>(a);
  poisson_finish_kernel<<<(a.n_sets + 127) / 128, 128, 0, st>>>(a);
}

void launch_gaussian(int n_sets, int rows, int cols, const double *model,
                     int64_t model_set_stride, int64_t model_row_stride, const double *data,
                     const double *errors, double *loglike, cudaStream_t st) {
  if (n_sets <= 0) return;
  gaussian_kernel<<<(n_sets + 3) / 4, 128, 0, st>>>(n_sets, rows, cols, model, model_set_stride,
                                                     model_row_stride, data, errors, loglike);
}

void launch_expected_counts(const ExpectedArgs &a, cudaStream_t st) {
  const int64_t warps = (int64_t)a.n_sets * a.K;
  if (warps <= 0) return;
  expected_counts_kernel<<<(unsigned)((warps + kSynWarps - 1) / kSynWarps), 32 * kSynWarps, 0,
                           st>>>(a);
}

void launch_phase_integrator(const PhaseIntArgs &a, cudaStream_t st) {
  if (a.rows <= 0) return;
  phase_integrator_kernel<<<(unsigned)((a.rows + kSynWarps - 1) / kSynWarps), 32 * kSynWarps, 0,
                            st>>>(a);
}

// phase_interpolator.pyx:25-95: the Akima-periodic interpolant of each row
// at new_phases + shift wrapped into [0, 1), kept when positive unless
// allow_negative; a warp per row, lanes over the new phases
__global__ void __launch_bounds__(32 * kSynWarps) phase_interp_kernel(InterpArgs a) {
  const int lane = threadIdx.x & 31;
  const int64_t row = (int64_t)blockIdx.x * kSynWarps + (threadIdx.x >> 5);
  if (row >= a.rows) return;
  const int n = a.n;
  const double *x = a.grid, *y = a.signal + row * n;
  for (int j = lane; j < a.n_new; j += 32) {
    double p = a.new_x[j] + a.shift;
    p -= floor(p);
    double v;
    if (p < x[0] || p > x[n - 1]) {
      v = nan("");  // outside the interpolant's domain
    } else {
      const int i = locate(x, n, p);
      auto chord = [&](int k) -> double {
        const int q = periodic_chord(k, n);
        return (y[q + 1] - y[q]) / (x[q + 1] - x[q]);
      };
      double k1, k2, k3;
      akima_piece(chord(i - 2), chord(i - 1), chord(i), chord(i + 1), chord(i + 2),
                  x[i + 1] - x[i], k1, k2, k3);
      const double u = p - x[i];
      v = y[i] + u * (k1 + u * (k2 + u * k3));
    }
    a.out[row * a.n_new + j] = (v > 0.0 || a.allow_negative) ? v : 0.0;
  }
}

struct ColumnY {
  const double *s;
  int64_t stride;
  bool lg;
  __device__ double operator()(int k) const {
    const double v = s[(int64_t)k * stride];
    return lg ? log10(v) : v;
  }
};

// energy_interpolator.pyx:27-113: each column of signal[N_E][n_cols]
// splined (Steffen) in log10 E -- in log10 of the signal when the column is
// positive throughout -- at the new energies, zero above the last energy;
// out[n_new][n_cols] as the reference returns it (:125).  A warp per column.
__global__ void __launch_bounds__(32 * kSynWarps) energy_interp_kernel(InterpArgs a) {
  const int lane = threadIdx.x & 31;
  const int64_t col = (int64_t)blockIdx.x * kSynWarps + (threadIdx.x >> 5);
  if (col >= a.rows) return;
  const int n = a.n;
  const double *x = a.grid;
  bool pos = true;
  for (int k = lane; k < n; k += 32) pos = pos && (a.signal[(int64_t)k * a.rows + col] > 0.0);
  const bool lg = __all_sync(0xffffffffu, pos);
  const ColumnY Y{a.signal + col, a.rows, lg};
  const double x_max = x[n - 1];
  for (int j = lane; j < a.n_new; j += 32) {
    const double e = a.new_x[j];
    double v = 0.0;
    if (!(e > x_max)) {
      if (e < x[0]) {
        v = nan("");  // below the grid: outside the interpolant's domain
      } else {
        const int i = locate(x, n, e);
        const Cubic c = steffen_piece(ArrY{x}, Y, n, i);
        v = cubic_eval(c, e);
        if (lg) v = pow(10.0, v);
      }
    }
    a.out[(int64_t)j * a.rows + col] = v;
  }
}

void launch_phase_interpolator(const InterpArgs &a, cudaStream_t st) {
  if (a.rows <= 0 || a.n_new <= 0) return;
  phase_interp_kernel<<<(unsigned)((a.rows + kSynWarps - 1) / kSynWarps), 32 * kSynWarps, 0,
                        st>>>(a);
}

void launch_energy_interpolator(const InterpArgs &a, cudaStream_t st) {
  if (a.rows <= 0 || a.n_new <= 0) return;
  energy_interp_kernel<<<(unsigned)((a.rows + kSynWarps - 1) / kSynWarps), 32 * kSynWarps, 0,
                         st>>>(a);
}

void launch_poisson(int64_t n, const double *mean, double *out, uint64_t seed, uint64_t offset,
                    int32_t *fail, cudaStream_t st) {
  if (n <= 0) return;
  const int64_t blocks = std::min<int64_t>((n + 255) / 256, 152 * 16);
  poisson_kernel<<<(unsigned)blocks, 256, 0, st>>>(n, mean, out, seed, offset, fail);
}

}  // namespace xg
