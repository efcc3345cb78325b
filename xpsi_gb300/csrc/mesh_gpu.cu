// mesh_gpu.cu -- K0: the hot-region cell meshes of a batch, built on the GPU
// from the steps of mesh_math.h (xpsi/cellmesh/mesh.pyx:23-417,
// polar_mesh.pyx:23-430, mesh_tools.pyx:18-890) and written straight into
// the packed per-row and per-cell arrays the rays and integrator kernels read
// (the packing of xpsi/HotRegion.py:774-1017 / Likelihood.py:297-432 that
// the host path does in numpy).
//
// Three launches over all meshes of the batch:
//   1. the 1000-point table of area(colat..lims[1]) per mesh, one thread per
//      entry (1000 independent adaptive quadratures);
//   2. per mesh: the cell area and the S - 1 parallels (one thread, the
//      reference's running sum), then one thread per parallel for its
//      centre colatitude, radius, gravity, tilt and the packed row values;
//   3. one thread per cell: the corner / centre membership tests and, for a
//      cell cut by a region boundary, its area quadrature.
// Each thread's quadrature keeps its interval list (128 intervals) in local
// memory; the host builder's limit of 4000 gives bitwise the same meshes
// (the boundary integrals converge in far fewer intervals).
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "../../include/xpsi_gb300.h"
#include "mesh_math.h"

namespace xg {
namespace {

using namespace xgm;
using DWork = WorkT<128>;
constexpr double kC = 2.99792458e8;

struct MeshJob {
  MeshPlan pl;
  Star s;
  int64_t row_off, cell_off;
  double r_s, R_over_rs, lag_scale, omit_azimuth, logT;
  int antiphased;
};

__global__ void __launch_bounds__(128) mesh_table_kernel(const MeshJob *jobs, double *tab) {
  const int m = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kAreaTab) return;
  const MeshJob &J = jobs[m];
  DWork w;
  tab[(size_t)m * kAreaTab + i] =
      integrateArea(mesh_table_colat(J.pl, i), J.pl.lims[1], J.s, 0, w);
}

// per mesh: parallels, then the rows.  row_tmp[row] = (lower, upper, colatC,
// effective gravity); mesh_tmp[m] = (cellArea, eta)
__global__ void __launch_bounds__(128) mesh_rows_kernel(const MeshJob *jobs, const double *tab,
                                                        xgpu_mesh_batch_out o, double *row_tmp,
                                                        double *mesh_tmp) {
  extern __shared__ double sm[];
  double *colat = sm, *par = sm + kAreaTab;
  const int m = blockIdx.x;
  const MeshJob &J = jobs[m];
  const size_t S = J.pl.S;
  const double *T = tab + (size_t)m * kAreaTab;
  for (int i = threadIdx.x; i < kAreaTab; i += blockDim.x) colat[i] = mesh_table_colat(J.pl, i);
  __syncthreads();
  __shared__ double s_eta;
  if (threadIdx.x == 0) {
    double cellArea, eta;
    mesh_cell_area(J.pl, T[kAreaTab - 1], cellArea, eta);
    mesh_parallels(J.pl, colat, T, eta, par);
    s_eta = eta;
    mesh_tmp[2 * m] = cellArea;
    mesh_tmp[2 * m + 1] = eta;
  }
  __syncthreads();
  const double eta = s_eta;
  for (size_t i = threadIdx.x; i < S; i += blockDim.x) {
    double lower, upper;
    mesh_row_bounds(J.pl, par, i, lower, upper);
    DWork w;
    const RowOut r = mesh_row(J.s, lower, upper, eta, w);
    const int64_t row = J.row_off + (int64_t)i;
    row_tmp[4 * row] = lower;
    row_tmp[4 * row + 1] = upper;
    row_tmp[4 * row + 2] = r.colat;
    row_tmp[4 * row + 3] = r.effGrav;
    // packed row values, as the host packing forms them
    const double u = J.r_s / r.r;
    o.u[row] = u;
    o.r_s[row] = J.r_s;
    o.maxAlpha[row] = r.maxAlpha;
    o.radius[row] = r.r;
    o.cos_gamma[row] = r.cos_gamma;
    o.theta0[row] = J.pl.invert ? PI - r.colat : r.colat;
    double C = (1.0 / u - J.R_over_rs);
    C += log((1.0 / u - 1.0) / (J.R_over_rs - 1.0));
    C *= J.r_s / kC;
    o.lag_C[row] = C;
    o.lag_scale[row] = J.lag_scale;
    o.row_mesh[row] = m;
  }
}

// one thread per cell of the batch (cells of mesh m at [cell_off, cell_off + S^2))
__global__ void __launch_bounds__(128) mesh_cells_kernel(const MeshJob *jobs, int n_mesh,
                                                         int64_t n_cells, xgpu_mesh_batch_out o,
                                                         const double *row_tmp,
                                                         const double *mesh_tmp) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n_cells) return;
  int lo = 0, hi = n_mesh - 1;
  while (lo < hi) {  // last mesh whose cell_off <= c
    const int mid = (lo + hi + 1) >> 1;
    if (jobs[mid].cell_off <= c) lo = mid; else hi = mid - 1;
  }
  const int m = lo;
  const MeshJob &J = jobs[m];
  const size_t S = J.pl.S;
  const int64_t k = c - J.cell_off;
  const size_t i = (size_t)(k / (int64_t)S), j = (size_t)(k - (int64_t)i * (int64_t)S);
  const int64_t row = J.row_off + (int64_t)i;
  // azimuth (shifted by the omitted region's azimuth, half a turn when
  // antiphased) and the atmosphere parameters of the cell
  double ph = mesh_phi(J.pl, j) - J.omit_azimuth;
  if (J.antiphased) ph = ph + PI;
  o.phi[c] = ph;
  o.params[2 * c] = J.logT;
  o.params[2 * c + 1] = row_tmp[4 * row + 3];
  const size_t j_max = J.pl.j_max;
  if (j < j_max) {
    DWork w;
    const double A = mesh_cell(J.pl, J.s, i, j, row_tmp[4 * row], row_tmp[4 * row + 1],
                               row_tmp[4 * row + 2], mesh_tmp[2 * m], w);
    o.cellArea[c] = A;
    o.radiates[c] = A > 0.0 ? 1 : 0;
    if (J.pl.sym) {
      const int64_t cm = J.cell_off + (int64_t)(i * S + (S - 1 - j));
      o.cellArea[cm] = A;
      o.radiates[cm] = A > 0.0 ? 1 : 0;
    }
  } else if (!J.pl.sym || j < S - j_max) {
    // columns no mirror reaches keep area 0
    o.cellArea[c] = 0.0;
    o.radiates[c] = 0;
  }
}

}  // namespace
}  // namespace xg

extern "C" int xgpu_mesh_batch(int n, const xgpu_mesh_member *members, int64_t n_rows,
                               int64_t n_cells, const xgpu_mesh_batch_out *out, void *stream) {
  using namespace xg;
  if (n <= 0) return 0;
  if (members == nullptr || out == nullptr) return -2;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  std::vector<MeshJob> jobs((size_t)n);
  size_t S_max = 2;
  int64_t rows = 0, cells = 0;
  for (int m = 0; m < n; m++) {
    const xgpu_mesh_member &q = members[m];
    if (q.S < 2) return -2;
    MeshJob &J = jobs[(size_t)m];
    mesh_plan(q.polar != 0, q.num_cells, q.S, q.cede_radius, q.cede_colatitude, q.super_radius,
              q.super_colatitude, q.super_azimuth, J.pl);
    J.s = Star{q.R_eq, q.epsilon, q.zeta, 0.0, q.star_shape_ind};
    J.row_off = q.row_off;
    J.cell_off = q.cell_off;
    J.r_s = q.r_s;
    J.R_over_rs = q.R_eq / q.r_s;
    J.lag_scale = q.lag_scale;
    J.omit_azimuth = q.omit_azimuth;
    J.antiphased = q.antiphased;
    J.logT = q.logT;
    if (q.row_off != rows || q.cell_off != cells) return -2;  // packed in member order
    rows += (int64_t)q.S;
    cells += (int64_t)(q.S * q.S);
    S_max = std::max(S_max, q.S);
  }
  if (rows != n_rows || cells != n_cells) return -2;
  MeshJob *d_jobs = nullptr;
  double *tab = nullptr, *row_tmp = nullptr, *mesh_tmp = nullptr;
  if (cudaMallocAsync(&d_jobs, sizeof(MeshJob) * (size_t)n, st) != cudaSuccess) return -5;
  if (cudaMallocAsync(&tab, sizeof(double) * (size_t)n * kAreaTab, st) != cudaSuccess ||
      cudaMallocAsync(&row_tmp, sizeof(double) * 4 * (size_t)n_rows, st) != cudaSuccess ||
      cudaMallocAsync(&mesh_tmp, sizeof(double) * 2 * (size_t)n, st) != cudaSuccess) {
    cudaFreeAsync(d_jobs, st);
    return -5;
  }
  cudaMemcpyAsync(d_jobs, jobs.data(), sizeof(MeshJob) * (size_t)n, cudaMemcpyHostToDevice, st);
  mesh_table_kernel<<<dim3((kAreaTab + 127) / 128, (unsigned)n), 128, 0, st>>>(d_jobs, tab);
  const size_t smem = sizeof(double) * (kAreaTab + S_max);
  mesh_rows_kernel<<<(unsigned)n, 128, smem, st>>>(d_jobs, tab, *out, row_tmp, mesh_tmp);
  mesh_cells_kernel<<<(unsigned)((n_cells + 127) / 128), 128, 0, st>>>(d_jobs, n, n_cells, *out,
                                                                         row_tmp, mesh_tmp);
  // (a copy from pageable memory has been staged when cudaMemcpyAsync
  // returns, so the host jobs may go out of scope)
  const cudaError_t e = cudaGetLastError();
  cudaFreeAsync(d_jobs, st);
  cudaFreeAsync(tab, st);
  cudaFreeAsync(row_tmp, st);
  cudaFreeAsync(mesh_tmp, st);
  return e == cudaSuccess ? 0 : -5;
}
