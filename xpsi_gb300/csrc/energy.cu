// energy.cu -- K4: integration of the specific-flux signal over instrument
// input-energy intervals, replacing xpsi/tools/energy_integrator.pyx:27-114.
//
// One CTA per (signal, block of kCols phase columns).  The integrand
// E S(E) ln 10 of the block's columns and its chords in log10 E are staged in
// shared memory once; then one thread per (interval, column) output forms
// the Akima pieces (periodic ends, as the reference uses, :54) of the
// intervals it covers from the staged chords and integrates them exactly,
// clipped at the highest energy (:91-103).
#include "common.cuh"
#include "kernels.h"

namespace xg {
namespace {

constexpr int kCols = 16;      // phase columns per CTA
constexpr int kEThreads = 256;

__global__ void __launch_bounds__(kEThreads) energy_kernel(EnergyArgs a) {
  extern __shared__ double sm[];
  const int N_E = a.N_E, N_P = a.N_P, ne = a.n_edges;
  double *logE = sm;                   // [N_E]
  double *wE = logE + N_E;             // [N_E] 10^logE
  double *edges = wE + N_E;            // [ne]
  double *Y = edges + ne;              // [N_E][kCols] integrand
  double *CH = Y + (size_t)N_E * kCols;  // [N_E - 1][kCols] chords
  __shared__ int s_stop;
  const int s = blockIdx.y;
  const int k0 = blockIdx.x * kCols;
  const double *sig = a.signal + a.in_off[s];
  double *out = a.out + a.out_off[s];
  const double div = a.scale_per ? a.scale_per[s] : 1.0;
  const double ln10 = log(10.0);
  for (int t = threadIdx.x; t < N_E; t += blockDim.x) {
    logE[t] = a.logE[t];
    wE[t] = pow(10.0, a.logE[t]);
  }
  for (int t = threadIdx.x; t < ne; t += blockDim.x) edges[t] = a.logEdges[t];
  if (threadIdx.x == 0) s_stop = ne - 1;
  __syncthreads();
  const double maxE = logE[N_E - 1];
  // the reference stops after the first interval that reaches past the
  // highest energy (:103); later intervals keep their initial zero
  for (int j = threadIdx.x; j + 1 < ne; j += blockDim.x)
    if (edges[j + 1] > maxE) atomicMin(&s_stop, j + 1);
  // y_j = 10^logE_j * (signal_j / d^2) * ln 10, evaluated in the reference's order
  for (int t = threadIdx.x; t < N_E * kCols; t += blockDim.x) {
    const int j = t / kCols, c = t - j * kCols, k = k0 + c;
    double v = 0.0;
    if (k < N_P) {
      v = sig[(size_t)j * N_P + k];
      if (a.scale_per) v = v / div;
    }
    Y[t] = wE[j] * v * ln10;
  }
  __syncthreads();
  for (int t = threadIdx.x; t < (N_E - 1) * kCols; t += blockDim.x) {
    const int q = t / kCols, c = t - q * kCols;
    CH[t] = (Y[(q + 1) * kCols + c] - Y[q * kCols + c]) / (logE[q + 1] - logE[q]);
  }
  __syncthreads();
  const int stop = s_stop;
  for (int t = threadIdx.x; t < (ne - 1) * kCols; t += blockDim.x) {
    const int j = t / kCols, c = t - j * kCols, k = k0 + c;
    if (k >= N_P) continue;
    double val;
    if (j >= stop) {
      val = 0.0;
    } else {
      const double lo = edges[j];
      const double hi = edges[j + 1] > maxE ? maxE : edges[j + 1];
      if (lo > hi || lo < logE[0] || hi > maxE) {
        val = nan("");
      } else if (lo == hi) {
        val = 0.0;
      } else {
        auto chord = [&](int i) -> double { return CH[periodic_chord(i, N_E) * kCols + c]; };
        const int ia = locate(logE, N_E, lo), ib = locate(logE, N_E, hi);
        double acc = 0.0;
        for (int i = ia; i <= ib; i++) {
          const double h = logE[i + 1] - logE[i];
          double k1, k2, k3;
          akima_piece(chord(i - 2), chord(i - 1), chord(i), chord(i + 1), chord(i + 2), h, k1,
                      k2, k3);
          const double u = (i == ia) ? lo - logE[i] : 0.0;
          const double w = (i == ib) ? hi - logE[i] : h;
          acc += piece_integral(Y[i * kCols + c], k1, k2, k3, u, w);
        }
        val = acc;
      }
    }
    if (a.accumulate) {
      if (j < stop) out[(size_t)j * N_P + k] += val;
    } else {
      out[(size_t)j * N_P + k] = val;
    }
  }
}

}  // namespace

void launch_energy(const EnergyArgs &a, cudaStream_t st) {
  if (a.n_signals <= 0) return;
  dim3 grid((a.N_P + kCols - 1) / kCols, a.n_signals);
  const size_t smem =
      (size_t)(2 * a.N_E + a.n_edges + (size_t)(2 * a.N_E - 1) * kCols) * sizeof(double);
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(energy_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    attr = true;
  }
  energy_kernel<<<grid, kEThreads, smem, st>>>(a);
}

}  // namespace xg
