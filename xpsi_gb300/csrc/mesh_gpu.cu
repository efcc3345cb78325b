// mesh_gpu.cu -- K0: the hot-region cell meshes of a batch, built on the GPU
// from the steps of mesh_math.h (xpsi/cellmesh/mesh.pyx:23-417,
// polar_mesh.pyx:23-430, mesh_tools.pyx:18-890) and written straight into
// the packed per-row and per-cell arrays the rays and integrator kernels read
// (the packing of xpsi/HotRegion.py:774-1017 / Likelihood.py:297-432 that
// the host path does in numpy).
//
// Four launches over all meshes of the batch:
//   1. the 1000-point table of area(colat..lims[1]) per mesh, one thread per
//      entry (1000 independent adaptive quadratures);
//   2. per mesh: the cell area and the S - 1 parallels (one thread, the
//      reference's running sum), then one thread per parallel for its
//      centre colatitude, radius, gravity, tilt and the packed row values;
//   3. one thread per cell: the corner / centre membership tests; cells
//      wholly inside or outside get their area at once, cells cut by a
//      region boundary (~1 %) are queued;
//   4. one group of 16 lanes per queued cell, taken from a shared counter:
//      its area quadrature, group-cooperative (the 21 or 42 Gauss-Kronrod
//      nodes of a step over the lanes, the rule's sums reduced lane-parallel,
//      the interval list in shared memory) -- the same adaptive scheme the
//      host builder runs serially.
// The per-thread quadratures of steps 1-2 keep their interval list (128
// intervals) in local memory; the host builder's limit of 4000 gives bitwise
// the same meshes (these integrals converge in far fewer intervals).
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

// ---------------------------------------------------------------------------
// Group-cooperative form of the quadrature of mesh_math.h (qag21, dyadic,
// integrate): a group of kGrp = 16 lanes (half a warp) integrates one cell.
// Lane l of the group evaluates nodes l, l + 16 and l + 32 of the step's one
// or two 21-point panels, so the 42 nodes of a bisection step take three
// passes (88 % of the lane slots; one cell per warp took two passes of 32,
// 66 %).  Sums are xor-butterfly reductions within the group, identical in
// each of its lanes, so the control flow is group-uniform; the two groups of
// a warp run independently (group masks on every shuffle and sync).
// ---------------------------------------------------------------------------
constexpr int kGrp = 16;
constexpr int kWarpList = 128;
struct WarpList {
  double al[kWarpList], bl[kWarpList], rl[kWarpList], el[kWarpList];
};
struct Grp {
  int l;          // lane within the group
  unsigned mask;  // the group's lanes
};

__device__ __forceinline__ double gsum(const Grp &g, double v) {
#pragma unroll
  for (int o = kGrp / 2; o > 0; o >>= 1) v += __shfl_xor_sync(g.mask, v, o);
  return v;
}

struct WPanel {
  double res, err, rabs, rasc;
};

__device__ __forceinline__ int k21_slot(int n) { return n < 10 ? n : (n == 10 ? 10 : n - 11); }
__device__ __forceinline__ double k21_node(double a, double b, int n) {
  const double c = 0.5 * (a + b), h = 0.5 * (b - a);
  if (n < 10) return c - h * XG_K21_X[n];
  if (n == 10) return c;
  return c + h * XG_K21_X[n - 11];
}
__device__ __forceinline__ WPanel k21_finish(double rk, double rg, double ra, double rc,
                                             double a, double b) {
  const double h = 0.5 * (b - a), ah = fabs(h);
  WPanel P;
  P.res = rk * h;
  ra *= ah;
  rc *= ah;
  double e = fabs((rk - rg) * h);
  if (rc != 0.0 && e != 0.0) {
    const double x = 200.0 * e / rc, sc = x * sqrt(x);  // x^1.5 without pow
    e = sc < 1.0 ? rc * sc : rc;
  }
  const double eps = 2.220446049250313e-16, dmin = 2.2250738585072014e-308;
  if (ra > dmin / (50.0 * eps)) e = (e < 50.0 * eps * ra) ? 50.0 * eps * ra : e;
  P.err = e;
  P.rabs = ra;
  P.rasc = rc;
  return P;
}

template <typename F>
__device__ void grp_k21(const F &f, const Grp &g, double a1, double b1, double a2, double b2,
                        bool two, WPanel &P1, WPanel &P2) {
  const int total = two ? 42 : 21;
  double fv[3];
  double rk1 = 0.0, rg1 = 0.0, ra1 = 0.0, rk2 = 0.0, rg2 = 0.0, ra2 = 0.0;
#pragma unroll
  for (int p = 0; p < 3; p++) {
    const int n = g.l + p * kGrp;
    fv[p] = 0.0;
    if (n < total) {
      const bool first = n < 21;
      const int m = first ? n : n - 21;
      const double v = f(first ? k21_node(a1, b1, m) : k21_node(a2, b2, m));
      fv[p] = v;
      const int s = k21_slot(m);
      const double wk = XG_K21_WK[s], wg = XG_K21_WG[s];
      if (first) { rk1 += wk * v; rg1 += wg * v; ra1 += wk * fabs(v); }
      else { rk2 += wk * v; rg2 += wg * v; ra2 += wk * fabs(v); }
    }
  }
  rk1 = gsum(g, rk1); rg1 = gsum(g, rg1); ra1 = gsum(g, ra1);
  if (two) { rk2 = gsum(g, rk2); rg2 = gsum(g, rg2); ra2 = gsum(g, ra2); }
  const double mean1 = 0.5 * rk1, mean2 = 0.5 * rk2;
  double rc1 = 0.0, rc2 = 0.0;
#pragma unroll
  for (int p = 0; p < 3; p++) {
    const int n = g.l + p * kGrp;
    if (n < total) {
      if (n < 21) rc1 += XG_K21_WK[k21_slot(n)] * fabs(fv[p] - mean1);
      else rc2 += XG_K21_WK[k21_slot(n - 21)] * fabs(fv[p] - mean2);
    }
  }
  P1 = k21_finish(rk1, rg1, ra1, gsum(g, rc1), a1, b1);
  if (two) P2 = k21_finish(rk2, rg2, ra2, gsum(g, rc2), a2, b2);
}

template <typename F>
__device__ double grp_qag21(const F &f, double a, double b, double epsabs, double er,
                            WarpList &L, const Grp &g) {
  const double eps = 2.220446049250313e-16, dmin = 2.2250738585072014e-308;
  WPanel P0, Pu;
  grp_k21(f, g, a, b, 0.0, 0.0, false, P0, Pu);
  const double r0 = P0.res, e0 = P0.err;
  double tol = (epsabs < er * fabs(r0)) ? er * fabs(r0) : epsabs;
  if ((e0 <= 50.0 * eps * P0.rabs && e0 > tol) || (e0 <= tol && e0 != P0.rasc) || e0 == 0.0)
    return r0;
  __syncwarp(g.mask);
  if (g.l == 0) { L.al[0] = a; L.bl[0] = b; L.rl[0] = r0; L.el[0] = e0; }
  __syncwarp(g.mask);
  int size = 1, iter = 1, k = 0, rnd1 = 0, rnd2 = 0, fail = 0;
  double area = r0, errsum = e0;
  do {
    const double ai = L.al[k], bi = L.bl[k], ri = L.rl[k], ei = L.el[k];
    const double a1 = ai, b1 = 0.5 * (ai + bi), a2 = b1, b2 = bi;
    WPanel P1, P2;
    grp_k21(f, g, a1, b1, a2, b2, true, P1, P2);
    const double r1 = P1.res, e1 = P1.err, r2 = P2.res, e2 = P2.err;
    const double r12 = r1 + r2, e12 = e1 + e2;
    errsum += e12 - ei;
    area += r12 - ri;
    if (P1.rasc != e1 && P2.rasc != e2) {
      if (fabs(ri - r12) <= 1.0e-5 * fabs(r12) && e12 >= 0.99 * ei) rnd1++;
      if (iter >= 10 && e12 > ei) rnd2++;
    }
    tol = (epsabs < er * fabs(area)) ? er * fabs(area) : epsabs;
    if (errsum > tol) {
      if (rnd1 >= 6 || rnd2 >= 20) fail = 2;
      const double edge = (1.0 + 100.0 * eps) * (fabs(a2) + 1000.0 * dmin);
      if (fabs(a1) <= edge && fabs(b2) <= edge) fail = 3;
    }
    const int nw = size++;
    __syncwarp(g.mask);
    if (g.l == 0) {
      if (e2 > e1) {
        L.al[k] = a2; L.bl[k] = b2; L.rl[k] = r2; L.el[k] = e2;
        L.al[nw] = a1; L.bl[nw] = b1; L.rl[nw] = r1; L.el[nw] = e1;
      } else {
        L.al[k] = a1; L.bl[k] = b1; L.rl[k] = r1; L.el[k] = e1;
        L.al[nw] = a2; L.bl[nw] = b2; L.rl[nw] = r2; L.el[nw] = e2;
      }
    }
    __syncwarp(g.mask);
    // the interval of largest error, compared by bit pattern: the errors are
    // non-negative, so their patterns order as 64-bit integers like the
    // values (the integer pipe instead of FP64 compares; the first of equal
    // errors wins, as before)
    k = 0;
    long long ek = __double_as_longlong(L.el[0]);
    for (int i = 1; i < size; i++) {
      const long long e = __double_as_longlong(L.el[i]);
      if (e > ek) { ek = e; k = i; }
    }
    iter++;
  } while (iter < kWarpList && !fail && errsum > tol);
  double sum = 0.0;
  for (int i = 0; i < size; i++) sum += L.rl[i];
  __syncwarp(g.mask);
  return sum;
}

template <typename F>
__device__ double grp_dyadic(const F &f, double lo, double hi, bool toward_lo, double er,
                             WarpList &L, const Grp &g) {
  const double Lw = hi - lo;
  double sum = 0.0;
  int seen = 0, quiet = 0;
  for (int k = 0; k < 2100; k++) {
    const double s1 = ldexp(Lw, -(k + 1)), s0 = ldexp(Lw, -k);
    const double p0 = toward_lo ? lo + s1 : hi - s0;
    const double p1 = toward_lo ? lo + s0 : hi - s1;
    if (!(p0 < p1) || (toward_lo ? p0 <= lo : p1 >= hi)) break;
    const double r = grp_qag21(f, p0, p1, 0.0, er, L, g);
    sum += r;
    if (r != 0.0) seen = 1;
    if (seen && fabs(r) <= 1.0e-17 * fabs(sum)) {
      if (++quiet >= 4) break;
    } else {
      quiet = 0;
    }
  }
  return sum;
}

template <typename F>
__device__ double grp_integrate(const F &f, double a, double b, double epsabs, double epsrel,
                                WarpList &L, const Grp &g) {
  double sign = 1.0;
  if (b < a) { const double t = a; a = b; b = t; sign = -1.0; }
  if (a == b) return 0.0;
  double er = (1.0e-13 < epsrel) ? 1.0e-13 : epsrel;
  if (epsabs <= 0.0 && er < 50.0 * 2.220446049250313e-16) er = 50.0 * 2.220446049250313e-16;
  double r = grp_qag21(f, a, b, epsabs, er, L, g);
  if (r == 0.0) {
    const double fa = f(a), fb = f(b);
    if (fa != 0.0 || fb != 0.0) {
      const double m = 0.5 * (a + b);
      const double rl = fa != 0.0 ? grp_dyadic(f, a, m, true, er, L, g)
                                  : grp_qag21(f, a, m, 0.0, er, L, g);
      const double rr = fb != 0.0 ? grp_dyadic(f, m, b, false, er, L, g)
                                  : grp_qag21(f, m, b, 0.0, er, L, g);
      r = rl + rr;
    }
  }
  return sign * r;
}

__device__ __forceinline__ int mesh_of_cell(const MeshJob *jobs, int n_mesh, int64_t c) {
  int lo = 0, hi = n_mesh - 1;
  while (lo < hi) {  // last mesh whose cell_off <= c
    const int mid = (lo + hi + 1) >> 1;
    if (jobs[mid].cell_off <= c) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ void put_area(const MeshJob &J, xgpu_mesh_batch_out &o, int64_t c,
                                         size_t i, size_t j, double A) {
  const size_t S = J.pl.S;
  o.cellArea[c] = A;
  o.radiates[c] = A > 0.0 ? 1 : 0;
  if (J.pl.sym) {
    const int64_t cm = J.cell_off + (int64_t)(i * S + (S - 1 - j));
    o.cellArea[cm] = A;
    o.radiates[cm] = A > 0.0 ? 1 : 0;
  }
}

// one thread per cell of the batch (cells of mesh m at [cell_off, cell_off + S^2))
__global__ void __launch_bounds__(128) mesh_cells_kernel(const MeshJob *jobs, int n_mesh,
                                                         int64_t n_cells, xgpu_mesh_batch_out o,
                                                         const double *row_tmp,
                                                         const double *mesh_tmp,
                                                         int64_t *queue, unsigned *n_queue) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n_cells) return;
  const int m = mesh_of_cell(jobs, n_mesh, c);
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
    double leftmost, rightmost;
    const int kind = mesh_cell_kind(J.pl, i, j, row_tmp[4 * row], row_tmp[4 * row + 1],
                                    row_tmp[4 * row + 2], leftmost, rightmost);
    if (kind == 2) queue[atomicAdd(n_queue, 1u)] = c;
    else put_area(J, o, c, i, j, kind == 1 ? mesh_tmp[2 * m] : 0.0);
  } else if (!J.pl.sym || j < S - j_max) {
    // columns no mirror reaches keep area 0
    o.cellArea[c] = 0.0;
    o.radiates[c] = 0;
  }
}

// one group of 16 lanes per queued cell: the area quadrature of a cell cut
// by a boundary.  The groups take the next queued cell from a shared counter
// (n_queue[1]) when they finish one, as the cells' costs differ by 5x or
// more (10-50 bisection steps); each cell's result is independent of which
// group integrates it.
constexpr int kBoundaryWarps = 4;
__global__ void __launch_bounds__(32 * kBoundaryWarps, 4) mesh_boundary_kernel(
    const MeshJob *jobs, int n_mesh, xgpu_mesh_batch_out o, const double *row_tmp,
    const int64_t *queue, unsigned *n_queue) {
  __shared__ WarpList lists[2 * kBoundaryWarps];
  const int lane = threadIdx.x & 31, half = lane / kGrp;
  const int grp = (threadIdx.x >> 5) * 2 + half;
  const Grp gp{lane - half * kGrp, 0xFFFFu << (kGrp * half)};
  WarpList &L = lists[grp];
  const unsigned n = n_queue[0];
  for (;;) {
    unsigned q = 0;
    if (gp.l == 0) q = atomicAdd(&n_queue[1], 1u);
    q = __shfl_sync(gp.mask, q, half * kGrp);
    if (q >= n) break;
    const int64_t c = queue[q];
    const int m = mesh_of_cell(jobs, n_mesh, c);
    const MeshJob &J = jobs[m];
    const size_t S = J.pl.S;
    const int64_t k = c - J.cell_off;
    const size_t i = (size_t)(k / (int64_t)S), j = (size_t)(k - (int64_t)i * (int64_t)S);
    const int64_t row = J.row_off + (int64_t)i;
    const double lower = row_tmp[4 * row], upper = row_tmp[4 * row + 1];
    double pa, pb;
    mesh_cell_kind(J.pl, i, j, lower, upper, row_tmp[4 * row + 2], pa, pb);
    const Region g = mesh_region(J.pl);
    const CellIntegrand f{J.s, g, pa, pb};
    double integral = grp_integrate(f, lower, upper, 0.0, 1.0e-8, L, gp);
    if (are_equal(integral, 0.0)) {
      double tmin, tmax;
      if (cell_fallback_interval(lower, upper, pa, pb, g, tmin, tmax))
        integral = grp_integrate(f, tmin, tmax, 0.0, 1.0e-8, L, gp);
    }
    if (gp.l == 0) put_area(J, o, c, i, j, J.s.R_eq * J.s.R_eq * integral);
    __syncwarp(gp.mask);
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
  int64_t *queue = nullptr;
  unsigned *n_queue = nullptr;
  if (cudaMallocAsync(&d_jobs, sizeof(MeshJob) * (size_t)n, st) != cudaSuccess) return -5;
  if (cudaMallocAsync(&tab, sizeof(double) * (size_t)n * kAreaTab, st) != cudaSuccess ||
      cudaMallocAsync(&row_tmp, sizeof(double) * 4 * (size_t)n_rows, st) != cudaSuccess ||
      cudaMallocAsync(&mesh_tmp, sizeof(double) * 2 * (size_t)n, st) != cudaSuccess ||
      cudaMallocAsync(&queue, sizeof(int64_t) * (size_t)n_cells, st) != cudaSuccess ||
      cudaMallocAsync(&n_queue, 2 * sizeof(unsigned), st) != cudaSuccess) {
    cudaFreeAsync(d_jobs, st);
    return -5;
  }
  // (a copy from pageable memory has been staged when cudaMemcpyAsync
  // returns, so the host jobs may go out of scope)
  cudaMemcpyAsync(d_jobs, jobs.data(), sizeof(MeshJob) * (size_t)n, cudaMemcpyHostToDevice, st);
  cudaMemsetAsync(n_queue, 0, 2 * sizeof(unsigned), st);  // queue length, next cell
  mesh_table_kernel<<<dim3((kAreaTab + 127) / 128, (unsigned)n), 128, 0, st>>>(d_jobs, tab);
  const size_t smem = sizeof(double) * (kAreaTab + S_max);
  mesh_rows_kernel<<<(unsigned)n, 128, smem, st>>>(d_jobs, tab, *out, row_tmp, mesh_tmp);
  mesh_cells_kernel<<<(unsigned)((n_cells + 127) / 128), 128, 0, st>>>(
      d_jobs, n, n_cells, *out, row_tmp, mesh_tmp, queue, n_queue);
  mesh_boundary_kernel<<<152 * 8, 32 * kBoundaryWarps, 0, st>>>(d_jobs, n, *out, row_tmp, queue,
                                                                 n_queue);
  const cudaError_t e = cudaGetLastError();
  cudaFreeAsync(d_jobs, st);
  cudaFreeAsync(tab, st);
  cudaFreeAsync(row_tmp, st);
  cudaFreeAsync(mesh_tmp, st);
  cudaFreeAsync(queue, st);
  cudaFreeAsync(n_queue, st);
  return e == cudaSuccess ? 0 : -5;
}
