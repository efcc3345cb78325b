// energy.cu -- K4: integration of the specific-flux signal over instrument
// input-energy intervals, replacing xpsi/tools/energy_integrator.pyx:27-114.
//
// One thread per (signal, phase column).  The integrand E S(E) ln 10 is
// splined in log10 E with the phase interpolant (Akima, periodic ends, as the
// reference uses, :54); each interval's integral is the exact integral of the
// cubic pieces it covers, clipped at the highest energy (:91-103).  Piece
// coefficients are formed on the fly from the five neighbouring chords, so a
// column needs no scratch beyond registers.
#include "common.cuh"
#include "kernels.h"

namespace xg {
namespace {

__global__ void __launch_bounds__(128) energy_kernel(EnergyArgs a) {
  extern __shared__ double sm[];
  const int N_E = a.N_E, N_P = a.N_P, ne = a.n_edges;
  double *logE = sm;             // [N_E]
  double *wE = sm + N_E;         // [N_E] 10^logE * ln 10 factors
  double *edges = sm + 2 * N_E;  // [ne]
  for (int t = threadIdx.x; t < N_E; t += blockDim.x) {
    logE[t] = a.logE[t];
    wE[t] = pow(10.0, a.logE[t]);
  }
  for (int t = threadIdx.x; t < ne; t += blockDim.x) edges[t] = a.logEdges[t];
  __syncthreads();
  const int s = blockIdx.y;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= N_P) return;
  const double *sig = a.signal + a.in_off[s];
  double *out = a.out + a.out_off[s];
  const double div = a.scale_per ? a.scale_per[s] : 1.0;
  const double ln10 = log(10.0);
  const double maxE = logE[N_E - 1];
  // y_j = 10^logE_j * (signal_j / d^2) * ln 10, evaluated in the reference's order
  auto y = [&](int j) -> double {
    double v = sig[(size_t)j * N_P + k];
    if (a.scale_per) v = v / div;
    return wE[j] * v * ln10;
  };
  auto chord = [&](int j) -> double {
    int q = periodic_chord(j, N_E);
    return (y(q + 1) - y(q)) / (logE[q + 1] - logE[q]);
  };
  for (int j = 0; j + 1 < ne; j++) {
    double lo = edges[j];
    double hi = edges[j + 1] > maxE ? maxE : edges[j + 1];
    double val;
    if (lo > hi || lo < logE[0] || hi > maxE) {
      val = nan("");
    } else if (lo == hi) {
      val = 0.0;
    } else {
      int ia = locate(logE, N_E, lo), ib = locate(logE, N_E, hi);
      double acc = 0.0;
      for (int i = ia; i <= ib; i++) {
        double h = logE[i + 1] - logE[i];
        double k1, k2, k3;
        akima_piece(chord(i - 2), chord(i - 1), chord(i), chord(i + 1), chord(i + 2), h, k1, k2,
                    k3);
        double u = (i == ia) ? lo - logE[i] : 0.0;
        double w = (i == ib) ? hi - logE[i] : h;
        acc += piece_integral(y(i), k1, k2, k3, u, w);
      }
      val = acc;
    }
    if (a.accumulate) out[(size_t)j * N_P + k] += val;
    else out[(size_t)j * N_P + k] = val;
    if (edges[j + 1] > maxE) break;
  }
}

}  // namespace

void launch_energy(const EnergyArgs &a, cudaStream_t st) {
  if (a.n_signals <= 0) return;
  dim3 grid((a.N_P + 127) / 128, a.n_signals);
  size_t smem = (size_t)(2 * a.N_E + a.n_edges) * sizeof(double);
  energy_kernel<<<grid, 128, smem, st>>>(a);
}

}  // namespace xg
