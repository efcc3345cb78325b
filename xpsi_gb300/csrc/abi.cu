// abi.cu -- the C ABI (include/xpsi_gb300.h): host staging for the drop-in
// entry points and argument plumbing for the batched ones.  Device scratch
// comes from the stream-ordered allocator (cudaMallocAsync), so a drop-in
// call costs one H2D burst, the kernels and one D2H burst.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <cstdlib>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/xpsi_gb300.h"
#include "kernels.h"

namespace {

thread_local std::string g_err;

int fail(const char *what, cudaError_t e) {
  g_err = std::string(what) + ": " + cudaGetErrorString(e);
  return -1;
}
int fail_msg(const std::string &m) {
  g_err = m;
  return -2;
}

#define CK(x)                              \
  do {                                     \
    cudaError_t e_ = (x);                  \
    if (e_ != cudaSuccess) return fail(#x, e_); \
  } while (0)

// one library stream per device for the drop-in calls
std::mutex g_mu;
cudaStream_t g_stream[64] = {};

int lib_stream(cudaStream_t *st) {
  int dev = 0;
  CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail_msg("device index out of range");
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_stream[dev]) CK(cudaStreamCreateWithFlags(&g_stream[dev], cudaStreamNonBlocking));
  *st = g_stream[dev];
  return 0;
}

// keep freed stream-ordered memory in the device pool between calls
void keep_pool(void) {
  static bool done[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64 || done[dev]) return;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
    uint64_t thr = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  done[dev] = true;
}

// stream-ordered device buffer
struct Dev {
  void *p = nullptr;
  cudaStream_t st = nullptr;
  ~Dev() {
    if (p) cudaFreeAsync(p, st);
  }
  template <typename T>
  T *as() const { return static_cast<T *>(p); }
};

int dalloc(Dev &d, size_t bytes, cudaStream_t st) {
  keep_pool();
  d.st = st;
  if (bytes == 0) bytes = 16;
  CK(cudaMallocAsync(&d.p, bytes, st));
  return 0;
}

template <typename T>
int upload(Dev &d, const T *h, size_t n, cudaStream_t st) {
  int r = dalloc(d, n * sizeof(T), st);
  if (r) return r;
  if (n) CK(cudaMemcpyAsync(d.p, h, n * sizeof(T), cudaMemcpyHostToDevice, st));
  return 0;
}

// Device copy of the most recent Num4D table passed to the drop-in layer, one
// per device, keyed by the table's host pointers, sizes and a strided sample
// of its contents.  The key cannot see every in-place edit of the host table
// or a new table allocated at a freed one's address with the same sample:
// callers that change a table in place call xgpu_atmos_cache_invalidate().
struct AtmosCache {
  const double *host_I = nullptr;
  size_t nT = 0, ng = 0, nmu = 0, nE = 0;
  uint64_t sample = 0;
  void *buf = nullptr;
  xg::Atmos4D view{};
};
AtmosCache g_atmos[64];

uint64_t sample_table(const xgpu_atmos4d *A) {
  size_t n = A->nT * A->ng * A->nmu * A->nE;
  uint64_t h = 1469598103934665603ull;
  auto mix = [&](const double *p, size_t m, size_t stride) {
    for (size_t i = 0; i < m; i += stride) {
      uint64_t b;
      std::memcpy(&b, p + i, 8);
      h = (h ^ b) * 1099511628211ull;
    }
  };
  mix(A->intensity, n, std::max<size_t>(1, n / 65536));
  mix(A->logT, A->nT, 1);
  mix(A->logg, A->ng, 1);
  mix(A->mu, A->nmu, 1);
  mix(A->logE, A->nE, 1);
  return h;
}

// frees device `dev`'s cached table; the caller holds g_mu and has made
// `dev` current.  Every stream of the device may still read the buffer (the
// drop-in stream, or a caller's), so the whole device is synchronised first.
int atmos_release(int dev) {
  AtmosCache &c = g_atmos[dev];
  if (!c.buf) return 0;
  CK(cudaDeviceSynchronize());
  CK(cudaFree(c.buf));
  c = AtmosCache{};
  return 0;
}

int atmos_device(const xgpu_atmos4d *A, cudaStream_t st, xg::Atmos4D *out) {
  if (A->nT < 4 || A->ng < 4 || A->nmu < 4 || A->nE < 4)
    return fail_msg("Num4D grids need at least 4 nodes per dimension");
  int dev = 0;
  CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail_msg("device index out of range");
  uint64_t smp = sample_table(A);
  std::lock_guard<std::mutex> lk(g_mu);
  AtmosCache &c = g_atmos[dev];
  if (c.buf && c.host_I == A->intensity && c.nT == A->nT && c.ng == A->ng &&
      c.nmu == A->nmu && c.nE == A->nE && c.sample == smp) {
    *out = c.view;
    return 0;
  }
  int rc = atmos_release(dev);
  if (rc) return rc;
  size_t nI = A->nT * A->ng * A->nmu * A->nE;
  size_t tot = A->nT + A->ng + A->nmu + A->nE + nI;
  CK(cudaMalloc(&c.buf, tot * sizeof(double)));
  double *b = static_cast<double *>(c.buf);
  double *pT = b, *pg = pT + A->nT, *pm = pg + A->ng, *pE = pm + A->nmu, *pI = pE + A->nE;
  CK(cudaMemcpyAsync(pT, A->logT, A->nT * 8, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(pg, A->logg, A->ng * 8, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(pm, A->mu, A->nmu * 8, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(pE, A->logE, A->nE * 8, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(pI, A->intensity, nI * 8, cudaMemcpyHostToDevice, st));
  c.host_I = A->intensity;
  c.nT = A->nT; c.ng = A->ng; c.nmu = A->nmu; c.nE = A->nE;
  c.sample = smp;
  c.view = xg::Atmos4D{pT, pg, pm, pE, pI, (int)A->nT, (int)A->ng, (int)A->nmu,
                       (int)A->nE, nullptr};
  *out = c.view;
  return 0;
}

static_assert(sizeof(xgpu_mesh) == sizeof(xg::MemberDesc), "mesh descriptor layout");

}  // namespace

extern "C" {

int xgpu_abi_version(void) { return XGPU_ABI_VERSION; }
const char *xgpu_last_error(void) { return g_err.c_str(); }

int xgpu_atmos_cache_invalidate(void) {
  int dev = 0;
  CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail_msg("device index out of range");
  std::lock_guard<std::mutex> lk(g_mu);
  return atmos_release(dev);
}

// ------------------------------------------------------------------ batched
int xgpu_rays_batch(int64_t n_rows, int N_R, const double *u, const double *r_s,
                    double *maxAlpha, double *deflection, double *cos_alpha, double *lag,
                    double *maxDeflection, int32_t *row_status, const double *lag_C,
                    const double *lag_scale, void *stream) {
  if (N_R < 3) return fail_msg("num_rays must be at least 3");
  if (n_rows > INT32_MAX) return fail_msg("too many rows in one launch");
  xg::RaysArgs a{(int)n_rows, N_R, u, r_s, maxAlpha, deflection, cos_alpha, lag,
                 maxDeflection, row_status, lag_C, lag_scale};
  xg::launch_rays(a, static_cast<cudaStream_t>(stream));
  CK(cudaGetLastError());
  return 0;
}

namespace {
int integrate_batch_impl(int n_meshes, const xgpu_mesh *meshes, int64_t n_rows, int N_R,
                         int N_E, int N_L, int N_P, const xgpu_integrate_batch_data *d,
                         int target_ctas, void *stream, int mixed, int table2d = 0);
}

int xgpu_integrate_batch(int n_meshes, const xgpu_mesh *meshes, int64_t n_rows, int N_R,
                         int N_E, int N_L, int N_P, const xgpu_integrate_batch_data *d,
                         int target_ctas, void *stream) {
  return integrate_batch_impl(n_meshes, meshes, n_rows, N_R, N_E, N_L, N_P, d, target_ctas,
                              stream, 0);
}

int xgpu_integrate_batch_mixed(int n_meshes, const xgpu_mesh *meshes, int64_t n_rows, int N_R,
                               int N_E, int N_L, int N_P, const xgpu_integrate_batch_data *d,
                               int target_ctas, void *stream) {
  return integrate_batch_impl(n_meshes, meshes, n_rows, N_R, N_E, N_L, N_P, d, target_ctas,
                              stream, 1);
}

}  // extern "C"

namespace {
// XGPU_CELL_SUMS=runs selects the power-sum form of the FP64 integrator's
// cell x phase sums instead of the per-cell form (the same sums, another
// order of summation)
bool wsum_enabled() {
  static const bool on = [] {
    const char *e = std::getenv("XGPU_CELL_SUMS");
    return e && std::string(e) == "runs";
  }();
  return on;
}

int integrate_batch_impl(int n_meshes, const xgpu_mesh *meshes, int64_t n_rows, int N_R,
                         int N_E, int N_L, int N_P, const xgpu_integrate_batch_data *d,
                         int target_ctas, void *stream, int mixed, int table2d) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (n_meshes <= 0) return 0;
  if (N_L < 5) return fail_msg("num_leaves must be at least 5 (Akima spline)");
  if (N_R < 3) return fail_msg("num_rays must be at least 3");
  for (int m = 0; m < n_meshes; m++) {
    if (meshes[m].atm_ext == 2 && d->atmos.intensity == nullptr)
      return fail_msg("a Num4D mesh needs the atmosphere table");
    const int ext = meshes[m].atm_ext;
    if ((ext == 4 || ext == 6) && (!table2d || mixed))
      return fail_msg("2-D table atmospheres (atm_ext 4, 6) are reached through the drop-in "
                      "integrators only");
    if (table2d && ext != 4 && ext != 6)
      return fail_msg("a 2-D table call takes atm_ext 4 or 6 only");
    if (ext == 3 && mixed) return fail_msg("the mixed integrator takes atm_ext 1 or 2");
    if (ext != 1 && ext != 2 && ext != 3 && ext != 4 && ext != 6)
      return fail_msg("atm_ext must be 1 (BB) or 2 (Num4D)");
  }
  for (int m = 0; m < n_meshes; m++) {
    const int b = meshes[m].beam_opt;
    if (b < 0 || b > 3) return fail_msg("beam_opt must be 0, 1, 2 or 3");
    if (b > 0 && mixed) return fail_msg("the mixed integrator takes beam_opt 0 only");
    if (b > 0 && d->n_params < 7)
      return fail_msg("beaming options read (abb, bbb, cbb, dbb, nimu) from parameters 2-6 of "
                      "the cell vectors: n_params must be at least 7");
    if (b == 3 && meshes[m].atm_ext != 1 && meshes[m].atm_ext != 2)
      return fail_msg("beam_opt 3 (numerical renormalisation) takes atm_ext 1 or 2");
  }
  if (d->correction != nullptr && mixed)
    return fail_msg("the elsewhere correction is computed by the FP64 integrator only");
  if (d->correction != nullptr && d->n_correction < 1)
    return fail_msg("correction vectors need at least 1 parameter per cell");
  if (target_ctas <= 0) target_ctas = 8 * 152;
  // the chunks are planned on the device from the parallels' costs (image
  // counts are known only after the ray tables): about 4 per CTA slot of
  // the target, at most 2 target + members and at most one per parallel
  // (integrator.cu)
  const int64_t target_chunks = 4 * (int64_t)target_ctas;
  const int64_t max_chunks = std::min<int64_t>(2 * target_chunks + n_meshes, n_rows) + 16;
  if (max_chunks > (int64_t)INT32_MAX / 2) return fail_msg("too many meshes in one call");
  const int n_chunks = (int)max_chunks;
  Dev dm, dr0, dr1, dfirst, dorder, dcount, drowcost, dchunkcost, dpart, dstate;
  int rc;
  if ((rc = upload(dm, reinterpret_cast<const xg::MemberDesc *>(meshes), n_meshes, st))) return rc;
  if ((rc = dalloc(dr0, (size_t)n_chunks * sizeof(int64_t), st)) ||
      (rc = dalloc(dr1, (size_t)n_chunks * sizeof(int64_t), st)) ||
      (rc = dalloc(dfirst, (size_t)(n_meshes + 1) * sizeof(int32_t), st)) ||
      (rc = dalloc(dorder, (size_t)n_chunks * sizeof(int32_t), st)) ||
      (rc = dalloc(dcount, sizeof(int32_t), st)) ||
      (rc = dalloc(drowcost, (size_t)std::max<int64_t>(1, n_rows) * sizeof(float), st)) ||
      (rc = dalloc(dchunkcost, (size_t)n_chunks * sizeof(float), st)))
    return rc;
  // each chunk's CTA zeroes its own partial before accumulating
  size_t part_n = (size_t)n_chunks * N_E * N_P;
  if ((rc = dalloc(dpart, part_n * sizeof(double), st))) return rc;
  if ((rc = dalloc(dstate, (size_t)3 * n_rows + 16, st))) return rc;
  Dev dslab;
  if (d->atmos.intensity != nullptr && !table2d &&
      (rc = dalloc(dslab, (size_t)n_chunks * d->atmos.nmu * d->atmos.nE * sizeof(double), st)))
    return rc;
  CK(cudaMemsetAsync(d->mesh_status, 0, n_meshes * sizeof(int32_t), st));
  // run records of the FP64 form's power sums (parallels of up to 1023
  // cells and 1024 leaves; beyond that the per-cell form runs)
  Dev dwsum;
  int w_cap = 0;
  int max_cells = 0;
  for (int m = 0; m < n_meshes; m++) max_cells = std::max(max_cells, (int)meshes[m].S1);
  const bool use_w = !mixed && max_cells <= 1023 && N_L <= 1024 && wsum_enabled();
  // a slot per CTA that can be resident (at most 2 per SM), twice over
  int w_slots = 0;
  Dev dwbusy, dpart2;
  if (use_w) {
    int dev = 0, sms = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    w_slots = 4 * std::max(1, sms);
    const size_t w_chunk = xg::integrate_wsum_bytes(N_P, max_cells, &w_cap);
    if ((rc = dalloc(dwsum, (size_t)w_slots * w_chunk, st)) ||
        (rc = dalloc(dwbusy, (size_t)w_slots * sizeof(int32_t), st)) ||
        (rc = dalloc(dpart2, part_n * sizeof(double), st)))
      return rc;
    CK(cudaMemsetAsync(dwbusy.p, 0, (size_t)w_slots * sizeof(int32_t), st));
  }

  xg::IntegrateArgs a{};
  a.n_members = n_meshes;
  a.n_rows = n_rows;
  a.members = dm.as<xg::MemberDesc>();
  a.row_member = d->row_mesh;
  a.radius = d->radius; a.u = d->u; a.cos_gamma = d->cos_gamma; a.theta0 = d->theta0;
  a.maxDeflection = d->maxDeflection;
  a.deflection = d->deflection; a.cos_alpha = d->cos_alpha; a.lag = d->lag;
  a.N_R = N_R;
  a.cellArea = d->cellArea; a.phi = d->phi; a.params = d->params; a.n_params = d->n_params;
  a.radiates = d->radiates;
  a.correction = d->correction;
  a.n_correction = d->n_correction;
  a.N_E = N_E; a.N_L = N_L; a.N_P = N_P;
  a.energies = d->energies; a.leaves = d->leaves; a.phases = d->phases;
  a.atmos = xg::Atmos4D{d->atmos.logT, d->atmos.logg, d->atmos.mu, d->atmos.logE,
                        d->atmos.intensity, (int)d->atmos.nT, (int)d->atmos.ng,
                        (int)d->atmos.nmu, (int)d->atmos.nE, d->atmos.intensity_f32};
  a.max_chunks = n_chunks;
  a.target_chunks = (int)target_chunks;
  a.chunk_r0 = dr0.as<int64_t>();
  a.chunk_r1 = dr1.as<int64_t>();
  a.partial = dpart.as<double>();
  a.chunk_first = dfirst.as<int32_t>();
  a.chunk_order = dorder.as<int32_t>();
  a.chunk_count = dcount.as<int32_t>();
  a.row_cost = drowcost.as<float>();
  a.chunk_cost = dchunkcost.as<float>();
  uint8_t *sb = dstate.as<uint8_t>();
  a.row_has_eval = sb; a.row_last_top = sb + n_rows; a.row_entry_top = sb + 2 * n_rows;
  a.member_status = d->mesh_status;
  a.flux = d->flux;
  a.flop_counter = d->flop_counter;
  a.slab = d->atmos.intensity != nullptr && !table2d ? dslab.as<double>() : nullptr;
  a.wsum = use_w ? dwsum.as<unsigned char>() : nullptr;
  a.w_cap = w_cap;
  a.w_slots = w_slots;
  a.w_slot_busy = use_w ? dwbusy.as<int32_t>() : nullptr;
  a.partial2 = use_w ? dpart2.as<double>() : nullptr;
  a.mixed = mixed;
  xg::launch_integrate(a, st);
  CK(cudaGetLastError());
  return 0;
}
}  // namespace

extern "C" {

int xgpu_energy_batch(int n_signals, int N_E, int N_P, int n_edges, const double *signal,
                      const int64_t *in_off, const double *log10_energies,
                      const double *log10_edges, const double *d_sq, double *out,
                      const int64_t *out_off, int accumulate, void *stream) {
  if (N_E < 5) return fail_msg("at least 5 energies are needed (Akima spline)");
  xg::EnergyArgs a{n_signals, N_E, N_P, n_edges, signal, in_off, log10_energies,
                   log10_edges, 1.0, d_sq, out, out_off, accumulate};
  xg::launch_energy(a, static_cast<cudaStream_t>(stream));
  CK(cudaGetLastError());
  return 0;
}

int xgpu_fold_batch(int batch, int K, int q, int N, const double *matrix, int ld,
                    const double *in, double *out, void *stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  xg::FoldArgs a{batch, K, q, N, matrix, ld, in, out};
  Dev scratch;
  int rc = dalloc(scratch, xg::fold_scratch_bytes(a), st);
  if (rc) return rc;
  xg::launch_fold(a, scratch.p, st);
  CK(cudaGetLastError());
  return 0;
}

int xgpu_fold_batch_tc(int batch, int K, int q, int N, const double *matrix, int ld,
                       const double *in, double *out, int32_t *status, void *stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  xg::FoldArgs a{batch, K, q, N, matrix, ld, in, out, status};
  Dev scratch;
  int rc = dalloc(scratch, xg::fold_tc_scratch_bytes(a), st);
  if (rc) return rc;
  rc = xg::launch_fold_tc(a, scratch.p, st);
  if (rc == -5) return fail_msg("could not set the tensor-core fold's shared-memory size");
  if (rc) return fail_msg("tensor-map encoding failed for the tensor-core fold");
  CK(cudaGetLastError());
  return 0;
}

int xgpu_fold_tc_timeout_selftest(int32_t *status_out) {
  cudaStream_t st;
  int rc;
  if ((rc = lib_stream(&st))) return rc;
  const int K = 8, q = 8, N = 8;
  xg::FoldArgs a{1, K, q, N, nullptr, q, nullptr, nullptr, nullptr};
  Dev dout, dst, scratch;
  if ((rc = dalloc(dout, (size_t)K * N * 8, st)) || (rc = dalloc(dst, 4, st)) ||
      (rc = dalloc(scratch, xg::fold_tc_scratch_bytes(a), st)))
    return rc;
  CK(cudaMemsetAsync(scratch.p, 0, xg::fold_tc_scratch_bytes(a), st));
  CK(cudaMemsetAsync(dst.p, 0, 4, st));
  a.out = dout.as<double>();
  a.status = dst.as<int32_t>();
  rc = xg::launch_fold_tc_timeout_selftest(a, scratch.p, st);
  if (rc) return fail_msg("could not launch the tensor-core fold's timeout self-test");
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(status_out, dst.p, 4, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return 0;
}

double xgpu_peak_probe(int fp64, int blocks, int threads, int iters, void *out,
                       void *stream) {
  return xg::launch_peak_probe(fp64, blocks, threads, iters, out,
                               static_cast<cudaStream_t>(stream));
}

int xgpu_likelihood_batch(const xgpu_likelihood_batch_data *d, void *stream) {
  if (d->B > 64) return fail_msg("at most 64 phase bins per channel");
  if (d->N_P < 5) return fail_msg("at least 5 signal phases are needed (Akima spline)");
  xg::LikeArgs a{};
  a.n_vec = d->n_vec; a.K = d->K; a.B = d->B; a.H = d->H; a.N_P = d->N_P;
  a.exposure = d->exposure; a.epsabs = d->epsabs; a.epsrel = d->epsrel;
  a.epsilon = d->epsilon; a.sigmas = d->sigmas; a.llzero = d->llzero; a.slim = d->slim;
  a.phase_edges = d->phase_edges; a.comp_phases = d->comp_phases; a.counts = d->counts;
  a.precomp = d->precomp; a.support = d->support; a.background = d->background;
  a.signals = d->signals; a.shifts = d->shifts; a.allow_negative = d->allow_negative;
  a.chan_ll = d->chan_ll; a.chan_flag = d->chan_flag; a.star = d->star;
  a.mcl_bg = d->mcl_bg; a.mcl_bg_s = d->mcl_bg_support; a.loglike = d->loglike;
  a.status = d->status;
  xg::launch_likelihood(a, static_cast<cudaStream_t>(stream));
  CK(cudaGetLastError());
  return 0;
}

// ------------------------------------------------------------------ drop-in
int xgpu_compute_rays(size_t N_u, double r_s, const double *r_s_over_R, double *maxAlpha,
                      size_t N_R, double *deflection, double *cos_alpha, double *lag,
                      double *maxDeflection) {
  cudaStream_t st;
  int rc;
  if ((rc = lib_stream(&st))) return rc;
  if (N_u == 0) return 0;
  std::vector<double> rs(N_u, r_s);
  Dev du, drs, dma, dD, dCA, dL, dMD, dstat;
  size_t tab = N_u * N_R;
  if ((rc = upload(du, r_s_over_R, N_u, st))) return rc;
  if ((rc = upload(drs, rs.data(), N_u, st))) return rc;
  if ((rc = upload(dma, maxAlpha, N_u, st))) return rc;
  if ((rc = dalloc(dD, tab * 8, st)) || (rc = dalloc(dCA, tab * 8, st)) ||
      (rc = dalloc(dL, tab * 8, st)) || (rc = dalloc(dMD, N_u * 8, st)) ||
      (rc = dalloc(dstat, N_u * 4, st)))
    return rc;
  rc = xgpu_rays_batch((int64_t)N_u, (int)N_R, du.as<double>(), drs.as<double>(),
                       dma.as<double>(), dD.as<double>(), dCA.as<double>(), dL.as<double>(),
                       dMD.as<double>(), dstat.as<int32_t>(), nullptr, nullptr, st);
  if (rc) return rc;
  std::vector<int32_t> stat(N_u);
  CK(cudaMemcpyAsync(maxAlpha, dma.p, N_u * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(deflection, dD.p, tab * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(cos_alpha, dCA.p, tab * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(lag, dL.p, tab * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(maxDeflection, dMD.p, N_u * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(stat.data(), dstat.p, N_u * 4, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  for (size_t i = 0; i < N_u; i++)
    if (stat[i] != 0) return 1;
  return 0;
}

}  // extern "C"

namespace {
// a 2-D table atmosphere on the device: grids (mu, E coordinate) and the
// I table [nmu][nE] of `I`, and the Q table of `Q` (on the same grids) when Q
// is given; one allocation held by `buf`
int table2d_device(cudaStream_t st, const xgpu_atmos4d *I, const xgpu_atmos4d *Q, Dev &buf,
                   xg::Atmos4D *out, const double **q_out) {
  if (!I->mu || !I->logE || !I->intensity) return fail_msg("the 2-D table is incomplete");
  if (I->nmu < 4 || I->nE < 4) return fail_msg("2-D table grids need at least 4 nodes");
  if (Q) {
    if (!Q->intensity) return fail_msg("the Q table is missing");
    if (Q->nmu != I->nmu || Q->nE != I->nE) return fail_msg("I and Q tables on different grids");
    for (size_t k = 0; k < I->nmu; k++)
      if (Q->mu[k] != I->mu[k]) return fail_msg("I and Q tables on different grids");
    for (size_t k = 0; k < I->nE; k++)
      if (Q->logE[k] != I->logE[k]) return fail_msg("I and Q tables on different grids");
  }
  const size_t nt = I->nmu * I->nE;
  int rc;
  if ((rc = dalloc(buf, (I->nmu + I->nE + (Q ? 2 : 1) * nt) * 8, st))) return rc;
  double *b = buf.as<double>();
  CK(cudaMemcpyAsync(b, I->mu, I->nmu * 8, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(b + I->nmu, I->logE, I->nE * 8, cudaMemcpyHostToDevice, st));
  double *tI = b + I->nmu + I->nE;
  CK(cudaMemcpyAsync(tI, I->intensity, nt * 8, cudaMemcpyHostToDevice, st));
  if (Q) CK(cudaMemcpyAsync(tI + nt, Q->intensity, nt * 8, cudaMemcpyHostToDevice, st));
  *out = xg::Atmos4D{};
  out->mu = b;
  out->logE = b + I->nmu;
  out->I = tI;
  out->nmu = (int)I->nmu;
  out->nE = (int)I->nE;
  if (q_out) *q_out = Q ? tI + nt : nullptr;
  return 0;
}

// a split atmosphere uploaded and reduced on the device to its (mu, E)
// table at vec (the first cell's t_e, t_bb, tau): grids in `dg`, the 5-D
// table in `dI`, the 2-D table in `dslab`
int split_device(cudaStream_t st, const xgpu_atmos5d *atmos, const double *vec, Dev &dg,
                 Dev &dI, Dev &dslab, xg::Atmos4D *out) {
  if (!atmos || !atmos->intensity) return fail_msg("the split integrator needs the 5-D atmosphere");
  size_t nI = 1, ng = 0;
  for (int d = 0; d < 5; d++) {
    if (atmos->n[d] < 4) return fail_msg("split grids need at least 4 nodes per dimension");
    nI *= atmos->n[d];
    ng += atmos->n[d];
  }
  const size_t nmu = atmos->n[3], nE = atmos->n[4];
  int rc;
  if ((rc = dalloc(dg, ng * 8, st)) || (rc = upload(dI, atmos->intensity, nI, st)) ||
      (rc = dalloc(dslab, nmu * nE * 8, st)))
    return rc;
  xg::SplitArgs sa{};
  double *gp = dg.as<double>();
  for (int d = 0; d < 5; d++) {
    CK(cudaMemcpyAsync(gp, atmos->grid[d], atmos->n[d] * 8, cudaMemcpyHostToDevice, st));
    sa.grid[d] = gp;
    sa.n[d] = (int)atmos->n[d];
    gp += atmos->n[d];
  }
  sa.I = dI.as<double>();
  // produce_2D_data at the first cell's parameter vector
  // (integrator_for_azimuthal_invariance_split.pyx:270)
  for (int d = 0; d < 3; d++) sa.vec[d] = vec[d];
  sa.out = dslab.as<double>();
  xg::launch_split_reduce(sa, st);
  CK(cudaGetLastError());
  *out = xg::Atmos4D{};
  out->mu = sa.grid[3];
  out->logE = sa.grid[4];
  out->I = dslab.as<double>();
  out->nmu = (int)nmu;
  out->nE = (int)nE;
  return 0;
}
}  // namespace

namespace {
// the drop-in integrators' common host path: upload, one batched launch on
// the library stream, copy back
int integrate_host(cudaStream_t st, double omega, double inclination, size_t S0,
                   size_t S1, const double *cellArea, const double *radius,
                   const double *r_s_over_r, const double *theta, const double *phi,
                   const double *srcCellParams, size_t n_params, const int32_t *radiates,
                   const double *correction, size_t n_correction, size_t N_R,
                   const double *deflection, const double *cos_alpha, const double *lag,
                   const double *maxDeflection, const double *cos_gamma, size_t N_E,
                   const double *energies, size_t N_L, const double *leaves, size_t N_P,
                   const double *phases, int atm_ext, const xg::Atmos4D &A,
                   int else_atm_ext, int image_order_limit, int beam_opt, double *flux) {
  int rc;
  if (n_params < 2) return fail_msg("srcCellParams needs at least 2 parameters per cell");
  if (correction && else_atm_ext != 1)
    return fail_msg("the GPU integrator corrects for a blackbody elsewhere only");
  if (correction && n_correction < 1)
    return fail_msg("correction vectors need at least 1 parameter per cell");
  const size_t cells = S0 * S1;
  Dev dcorr;
  if (correction && (rc = upload(dcorr, correction, cells * n_correction, st))) return rc;
  std::vector<double> theta0(S0);
  for (size_t i = 0; i < S0; i++) theta0[i] = theta[i * S1];
  std::vector<int32_t> row_mesh(S0, 0);
  Dev dA, drad, du, dth0, dphi, dpar, dR, dD, dCA, dL, dMD, dcg, dE, dLv, dP, dF, dst, drm;
  if ((rc = upload(dA, cellArea, cells, st)) || (rc = upload(drad, radius, S0, st)) ||
      (rc = upload(du, r_s_over_r, S0, st)) || (rc = upload(dth0, theta0.data(), S0, st)) ||
      (rc = upload(dphi, phi, cells, st)) || (rc = upload(dpar, srcCellParams, cells * n_params, st)) ||
      (rc = upload(dR, radiates, cells, st)) || (rc = upload(dD, deflection, S0 * N_R, st)) ||
      (rc = upload(dCA, cos_alpha, S0 * N_R, st)) || (rc = upload(dL, lag, S0 * N_R, st)) ||
      (rc = upload(dMD, maxDeflection, S0, st)) || (rc = upload(dcg, cos_gamma, S0, st)) ||
      (rc = upload(dE, energies, N_E, st)) || (rc = upload(dLv, leaves, N_L, st)) ||
      (rc = upload(dP, phases, N_P, st)) || (rc = dalloc(dF, N_E * N_P * 8, st)) ||
      (rc = dalloc(dst, 16, st)) || (rc = upload(drm, row_mesh.data(), S0, st)))
    return rc;
  xgpu_mesh mesh{(int32_t)S0, (int32_t)S1, 0, 0, omega, inclination, image_order_limit,
                 atm_ext, 0, beam_opt, 0};
  xgpu_integrate_batch_data d{};
  d.row_mesh = drm.as<int32_t>();
  d.radius = drad.as<double>(); d.u = du.as<double>(); d.cos_gamma = dcg.as<double>();
  d.theta0 = dth0.as<double>(); d.maxDeflection = dMD.as<double>();
  d.deflection = dD.as<double>(); d.cos_alpha = dCA.as<double>(); d.lag = dL.as<double>();
  d.cellArea = dA.as<double>(); d.phi = dphi.as<double>(); d.params = dpar.as<double>();
  d.n_params = (int32_t)n_params; d.radiates = dR.as<int32_t>();
  d.energies = dE.as<double>(); d.leaves = dLv.as<double>(); d.phases = dP.as<double>();
  if (atm_ext == 2 || atm_ext == 4 || atm_ext == 6) {
    d.atmos = xgpu_atmos4d{A.logT, A.logg, A.mu, A.logE, A.I, (size_t)A.nT, (size_t)A.ng,
                           (size_t)A.nmu, (size_t)A.nE, nullptr};
  }
  d.flux = dF.as<double>();
  d.mesh_status = dst.as<int32_t>();
  d.correction = correction ? dcorr.as<double>() : nullptr;
  d.n_correction = (int32_t)n_correction;
  rc = integrate_batch_impl(1, &mesh, (int64_t)S0, (int)N_R, (int)N_E, (int)N_L, (int)N_P, &d,
                            0, st, 0, (atm_ext == 4 || atm_ext == 6) ? 1 : 0);
  if (rc) return rc;
  int32_t status = 0;
  CK(cudaMemcpyAsync(&status, dst.p, 4, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(flux, dF.p, N_E * N_P * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return status != 0 ? 1 : 0;
}

}  // namespace

extern "C" {

int xgpu_integrate(double R, double omega, double r_s, double inclination, size_t S0,
                   size_t S1, const double *cellArea, const double *radius,
                   const double *r_s_over_r, const double *theta, const double *phi,
                   const double *srcCellParams, size_t n_params, const int32_t *radiates,
                   const double *correction, size_t n_correction, size_t N_R,
                   const double *deflection, const double *cos_alpha, const double *lag,
                   const double *maxDeflection, const double *cos_gamma, size_t N_E,
                   const double *energies, size_t N_L, const double *leaves, size_t N_P,
                   const double *phases, int atm_ext, const xgpu_atmos4d *atmos,
                   int else_atm_ext, int image_order_limit, int beam_opt, double *flux) {
  cudaStream_t st;
  int rc;
  if ((rc = lib_stream(&st))) return rc;
  if ((atm_ext == 2 || atm_ext == 4) && !atmos)
    return fail_msg("numerical atmospheres (atm_ext 2, 4) need the table");
  if (atm_ext < 1 || atm_ext > 4)
    return fail_msg("atm_ext must be 1 (BB), 2 (Num4D), 3 (burst BB) or 4 (Pol_Num2D)");
  xg::Atmos4D A{};
  Dev dt;
  if (atm_ext == 2 && (rc = atmos_device(atmos, st, &A))) return rc;
  if (atm_ext == 4 && (rc = table2d_device(st, atmos, nullptr, dt, &A, nullptr))) return rc;
  return integrate_host(st, omega, inclination, S0, S1, cellArea, radius, r_s_over_r, theta,
                        phi, srcCellParams, n_params, radiates, correction, n_correction, N_R,
                        deflection, cos_alpha, lag, maxDeflection, cos_gamma, N_E, energies,
                        N_L, leaves, N_P, phases, atm_ext, A, else_atm_ext, image_order_limit,
                        beam_opt, flux);
}

int xgpu_integrate_split(double R, double omega, double r_s, double inclination, size_t S0,
                         size_t S1, const double *cellArea, const double *radius,
                         const double *r_s_over_r, const double *theta, const double *phi,
                         const double *srcCellParams, size_t n_params,
                         const int32_t *radiates, const double *correction,
                         size_t n_correction, size_t N_R, const double *deflection,
                         const double *cos_alpha, const double *lag,
                         const double *maxDeflection, const double *cos_gamma, size_t N_E,
                         const double *energies, size_t N_L, const double *leaves,
                         size_t N_P, const double *phases, const xgpu_atmos5d *atmos,
                         int else_atm_ext, int image_order_limit, double *flux) {
  (void)R;
  (void)r_s;
  cudaStream_t st;
  int rc;
  if ((rc = lib_stream(&st))) return rc;
  if (n_params < 3) return fail_msg("the split atmosphere needs 3 parameters per cell");
  if (S0 * S1 == 0) return fail_msg("empty cell mesh");
  Dev dg, dI, dslab;
  xg::Atmos4D A{};
  if ((rc = split_device(st, atmos, srcCellParams, dg, dI, dslab, &A))) return rc;
  return integrate_host(st, omega, inclination, S0, S1, cellArea, radius, r_s_over_r, theta,
                        phi, srcCellParams, n_params, radiates, correction, n_correction, N_R,
                        deflection, cos_alpha, lag, maxDeflection, cos_gamma, N_E, energies,
                        N_L, leaves, N_P, phases, 6, A, else_atm_ext, image_order_limit, 0,
                        flux);
}

}  // extern "C"

namespace {
// the Stokes drop-ins' common host path: upload, the Stokes kernel on the
// library stream, copy back
int stokes_host(cudaStream_t st, double omega, double inclination, size_t S0,
                          size_t S1, const double *cellArea, const double *radius,
                          const double *r_s_over_r, const double *theta, const double *phi,
                          const double *srcCellParams, size_t n_params, const int32_t *radiates,
                          const double *correction, size_t n_correction, size_t N_R,
                          const double *deflection, const double *cos_alpha, const double *lag,
                          const double *maxDeflection, const double *cos_gamma, size_t N_E,
                          const double *energies, size_t N_L, const double *leaves, size_t N_P,
                          const double *phases, int atm_ext, const xg::Atmos4D &A,
                          const double *dQ, int else_atm_ext, int image_order_limit,
                          double *flux_I, double *flux_Q, double *flux_U) {
  int rc;
  if (S0 == 0 || S1 == 0 || N_E == 0 || N_P == 0) return 0;
  if (N_L < 5) return fail_msg("num_leaves must be at least 5 (Akima spline)");
  if (N_R < 3) return fail_msg("num_rays must be at least 3");
  if (n_params < 1) return fail_msg("srcCellParams needs at least 1 parameter per cell");
  if (correction && else_atm_ext != 1)
    return fail_msg("the GPU integrator corrects for a blackbody elsewhere only");
  if (correction && n_correction < 1)
    return fail_msg("correction vectors need at least 1 parameter per cell");
  if (xg::stokes_smem_bytes((int)N_L, (int)N_P, (int)N_E, (int)N_R, A.I ? A.nmu : 0,
                            A.I ? A.nE : 0) > 227 * 1024)
    return fail_msg("num_leaves and num_rays too large for one CTA's shared memory");
  const size_t cells = S0 * S1;
  std::vector<double> theta0(S0);
  for (size_t i = 0; i < S0; i++) theta0[i] = theta[i * S1];
  std::vector<int32_t> row_mesh(S0, 0);
  Dev dA, drad, du, dth0, dphi, dpar, dR, dD, dCA, dL, dMD, dcg, dE, dLv, dP, dF, dst, drm;
  Dev dcorr, dmem, dpart, dstate;
  if ((rc = upload(dA, cellArea, cells, st)) || (rc = upload(drad, radius, S0, st)) ||
      (rc = upload(du, r_s_over_r, S0, st)) || (rc = upload(dth0, theta0.data(), S0, st)) ||
      (rc = upload(dphi, phi, cells, st)) || (rc = upload(dpar, srcCellParams, cells * n_params, st)) ||
      (rc = upload(dR, radiates, cells, st)) || (rc = upload(dD, deflection, S0 * N_R, st)) ||
      (rc = upload(dCA, cos_alpha, S0 * N_R, st)) || (rc = upload(dL, lag, S0 * N_R, st)) ||
      (rc = upload(dMD, maxDeflection, S0, st)) || (rc = upload(dcg, cos_gamma, S0, st)) ||
      (rc = upload(dE, energies, N_E, st)) || (rc = upload(dLv, leaves, N_L, st)) ||
      (rc = upload(dP, phases, N_P, st)) || (rc = dalloc(dF, 3 * N_E * N_P * 8, st)) ||
      (rc = dalloc(dst, 16, st)) || (rc = upload(drm, row_mesh.data(), S0, st)))
    return rc;
  if (correction && (rc = upload(dcorr, correction, cells * n_correction, st))) return rc;
  xg::MemberDesc mesh{(int32_t)S0, (int32_t)S1, 0, 0, omega, inclination, image_order_limit,
                      atm_ext, 0};
  if ((rc = upload(dmem, &mesh, 1, st))) return rc;
  xg::IntegrateArgs a{};
  a.n_members = 1;
  a.n_rows = (int64_t)S0;
  a.members = dmem.as<xg::MemberDesc>();
  a.row_member = drm.as<int32_t>();
  a.radius = drad.as<double>(); a.u = du.as<double>(); a.cos_gamma = dcg.as<double>();
  a.theta0 = dth0.as<double>(); a.maxDeflection = dMD.as<double>();
  a.deflection = dD.as<double>(); a.cos_alpha = dCA.as<double>(); a.lag = dL.as<double>();
  a.N_R = (int)N_R;
  a.cellArea = dA.as<double>(); a.phi = dphi.as<double>(); a.params = dpar.as<double>();
  a.n_params = (int)n_params; a.radiates = dR.as<int32_t>();
  a.correction = correction ? dcorr.as<double>() : nullptr;
  a.n_correction = (int)n_correction;
  a.N_E = (int)N_E; a.N_L = (int)N_L; a.N_P = (int)N_P;
  a.energies = dE.as<double>(); a.leaves = dLv.as<double>(); a.phases = dP.as<double>();
  a.member_status = dst.as<int32_t>();
  if (A.I) {
    a.atmos = A;
    a.table_q = dQ;
    if ((rc = dalloc(dstate, 3 * S0 + 16, st))) return rc;
    uint8_t *sb = dstate.as<uint8_t>();
    a.row_has_eval = sb; a.row_last_top = sb + S0; a.row_entry_top = sb + 2 * S0;
  }
  a.flux = dF.as<double>();
  a.flux_q = a.flux + N_E * N_P;
  a.flux_u = a.flux_q + N_E * N_P;
  const size_t np = xg::stokes_partial_doubles(a);
  if ((rc = dalloc(dpart, np * 8, st))) return rc;
  CK(cudaMemsetAsync(dpart.p, 0, np * 8, st));
  CK(cudaMemsetAsync(dst.p, 0, 16, st));
  a.partial = dpart.as<double>();
  rc = xg::launch_stokes(a, st);
  if (rc == -2) return fail_msg("integrator shared memory too large");
  CK(cudaGetLastError());
  int32_t status = 0;
  CK(cudaMemcpyAsync(&status, dst.p, 4, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(flux_I, a.flux, N_E * N_P * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(flux_Q, a.flux_q, N_E * N_P * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(flux_U, a.flux_u, N_E * N_P * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return status != 0 ? 1 : 0;
}

}  // namespace

extern "C" {

int xgpu_integrate_stokes(double R, double omega, double r_s, double inclination, size_t S0,
                          size_t S1, const double *cellArea, const double *radius,
                          const double *r_s_over_r, const double *theta, const double *phi,
                          const double *srcCellParams, size_t n_params, const int32_t *radiates,
                          const double *correction, size_t n_correction, size_t N_R,
                          const double *deflection, const double *cos_alpha, const double *lag,
                          const double *maxDeflection, const double *cos_gamma, size_t N_E,
                          const double *energies, size_t N_L, const double *leaves, size_t N_P,
                          const double *phases, int atm_ext, const xgpu_atmos4d *atmos_I,
                          const xgpu_atmos4d *atmos_Q, int else_atm_ext, int image_order_limit,
                          double *flux_I, double *flux_Q, double *flux_U) {
  (void)R;
  (void)r_s;
  cudaStream_t st;
  int rc;
  if ((rc = lib_stream(&st))) return rc;
  if (atm_ext != 1 && atm_ext != 3 && atm_ext != 4)
    return fail_msg("the Stokes integrator takes atm_ext 1 (BB), 3 (burst BB) or 4 (Pol_Num2D)");
  xg::Atmos4D A{};
  const double *dQ = nullptr;
  Dev dt;
  if (atm_ext == 4) {
    if (!atmos_I || !atmos_Q) return fail_msg("atm_ext 4 (Pol_Num2D) needs the I and Q tables");
    if ((rc = table2d_device(st, atmos_I, atmos_Q, dt, &A, &dQ))) return rc;
  }
  return stokes_host(st, omega, inclination, S0, S1, cellArea, radius, r_s_over_r, theta, phi,
                     srcCellParams, n_params, radiates, correction, n_correction, N_R,
                     deflection, cos_alpha, lag, maxDeflection, cos_gamma, N_E, energies, N_L,
                     leaves, N_P, phases, atm_ext, A, dQ, else_atm_ext, image_order_limit,
                     flux_I, flux_Q, flux_U);
}

int xgpu_integrate_split_stokes(double R, double omega, double r_s, double inclination,
                                size_t S0, size_t S1, const double *cellArea,
                                const double *radius, const double *r_s_over_r,
                                const double *theta, const double *phi,
                                const double *srcCellParams, size_t n_params,
                                const int32_t *radiates, const double *correction,
                                size_t n_correction, size_t N_R, const double *deflection,
                                const double *cos_alpha, const double *lag,
                                const double *maxDeflection, const double *cos_gamma,
                                size_t N_E, const double *energies, size_t N_L,
                                const double *leaves, size_t N_P, const double *phases,
                                const xgpu_atmos5d *atmos_I, const xgpu_atmos5d *atmos_Q,
                                int else_atm_ext, int image_order_limit, double *flux_I,
                                double *flux_Q, double *flux_U) {
  (void)R;
  (void)r_s;
  cudaStream_t st;
  int rc;
  if ((rc = lib_stream(&st))) return rc;
  if (n_params < 3) return fail_msg("the split atmosphere needs 3 parameters per cell");
  if (S0 * S1 == 0) return fail_msg("empty cell mesh");
  if (!atmos_I || !atmos_Q) return fail_msg("the split Stokes integrator needs I and Q tables");
  for (int d = 3; d < 5; d++) {
    if (atmos_I->n[d] != atmos_Q->n[d]) return fail_msg("I and Q tables on different grids");
    for (size_t k = 0; k < atmos_I->n[d]; k++)
      if (atmos_I->grid[d][k] != atmos_Q->grid[d][k])
        return fail_msg("I and Q tables on different grids");
  }
  // each table reduced by its own evaluator (:310-322)
  Dev gI, tI, sI, gQ, tQ, sQ;
  xg::Atmos4D A{}, AQ{};
  if ((rc = split_device(st, atmos_I, srcCellParams, gI, tI, sI, &A)) ||
      (rc = split_device(st, atmos_Q, srcCellParams, gQ, tQ, sQ, &AQ)))
    return rc;
  return stokes_host(st, omega, inclination, S0, S1, cellArea, radius, r_s_over_r, theta, phi,
                     srcCellParams, n_params, radiates, correction, n_correction, N_R,
                     deflection, cos_alpha, lag, maxDeflection, cos_gamma, N_E, energies, N_L,
                     leaves, N_P, phases, 6, A, AQ.I, else_atm_ext, image_order_limit, flux_I,
                     flux_Q, flux_U);
}

}  // extern "C"

namespace {
// the general integrators' common host path (I, or I, Q and U)
int general_host(cudaStream_t st, double omega, double inclination, size_t S0,
                           size_t S1, const double *cellArea, const double *radius,
                           const double *r_s_over_r, const double *theta, const double *phi,
                           const double *srcCellParams, size_t n_params,
                           const int32_t *radiates, const double *correction,
                           size_t n_correction, size_t N_R, const double *deflection,
                           const double *cos_alpha, const double *lag,
                           const double *maxDeflection, const double *cos_gamma, size_t N_E,
                           const double *energies, size_t N_L, const double *leaves,
                           size_t N_P, const double *phases, int atm_ext,
                           const xg::Atmos4D &A, const double *dQ, int else_atm_ext,
                           int image_order_limit, double *flux, double *flux_Q,
                           double *flux_U) {
  int rc;
  const int stokes = (flux_Q != nullptr && flux_U != nullptr) ? 1 : 0;
  const int ns = stokes ? 3 : 1;
  if (S0 == 0 || S1 == 0 || N_E == 0 || N_P == 0) return 0;
  if (N_L < 5) return fail_msg("num_leaves must be at least 5 (Akima spline)");
  if (N_R < 3) return fail_msg("num_rays must be at least 3");
  if (atm_ext == 2 && n_params < 2)
    return fail_msg("srcCellParams needs (log T, log g) per cell for Num4D");
  if (n_params < 1) return fail_msg("srcCellParams needs at least 1 parameter per cell");
  if (correction && else_atm_ext != 1)
    return fail_msg("the GPU integrator corrects for a blackbody elsewhere only");
  if (correction && n_correction < 1)
    return fail_msg("correction vectors need at least 1 parameter per cell");
  if (xg::general_geometry_smem_bytes((int)N_R, (int)N_L) > 227 * 1024)
    return fail_msg("num_rays and num_leaves too large for one CTA's shared memory");
  // images per parallel: the reference's image order of the rows it evaluates
  int IOmax = 1;
  for (size_t i = 0; i < S0; i++) {
    bool any = false;
    for (size_t j = 0; j < S1 && !any; j++) any = radiates[i * S1 + j] == 1;
    if (!any) continue;
    const double io = image_order_limit > 0 ? (double)image_order_limit
                                            : std::ceil(maxDeflection[i] / 3.14159265358979323846);
    if (io > 64.0) return fail_msg("a parallel has more than 64 images");
    IOmax = std::max(IOmax, (int)io);
  }
  const size_t cells = S0 * S1;
  std::vector<double> theta0(S0);
  for (size_t i = 0; i < S0; i++) theta0[i] = theta[i * S1];
  const size_t n_ent = cells * (size_t)IOmax * N_P;
  Dev dA, drad, du, dth0, dphi, dpar, dR, dD, dCA, dL, dMD, dcg, dE, dLv, dP, dF, dst, dcorr;
  Dev deG, deZ, deA, dimg, dpart, dchi, dFq;
  if ((rc = upload(dA, cellArea, cells, st)) || (rc = upload(drad, radius, S0, st)) ||
      (rc = upload(du, r_s_over_r, S0, st)) || (rc = upload(dth0, theta0.data(), S0, st)) ||
      (rc = upload(dphi, phi, cells, st)) || (rc = upload(dpar, srcCellParams, cells * n_params, st)) ||
      (rc = upload(dR, radiates, cells, st)) || (rc = upload(dD, deflection, S0 * N_R, st)) ||
      (rc = upload(dCA, cos_alpha, S0 * N_R, st)) || (rc = upload(dL, lag, S0 * N_R, st)) ||
      (rc = upload(dMD, maxDeflection, S0, st)) || (rc = upload(dcg, cos_gamma, S0, st)) ||
      (rc = upload(dE, energies, N_E, st)) || (rc = upload(dLv, leaves, N_L, st)) ||
      (rc = upload(dP, phases, N_P, st)) || (rc = dalloc(dF, N_E * N_P * 8, st)) ||
      (rc = dalloc(dst, 16, st)) || (rc = dalloc(deG, n_ent * 8, st)) ||
      (rc = dalloc(deZ, n_ent * 8, st)) || (rc = dalloc(deA, n_ent * 8, st)) ||
      (rc = dalloc(dimg, S0 * 4, st)) ||
      (rc = dalloc(dpart, S0 * (size_t)IOmax * ns * N_E * N_P * 8, st)) ||
      (rc = dalloc(dchi, S0 * (size_t)IOmax * 2 * 8, st)))
    return rc;
  if (stokes && (rc = dalloc(dFq, 2 * N_E * N_P * 8, st))) return rc;
  if (correction && (rc = upload(dcorr, correction, cells * n_correction, st))) return rc;
  CK(cudaMemsetAsync(dst.p, 0, 16, st));
  xg::GeneralArgs a{};
  a.S0 = (int)S0; a.S1 = (int)S1; a.N_R = (int)N_R; a.N_L = (int)N_L; a.N_P = (int)N_P;
  a.N_E = (int)N_E; a.IOmax = IOmax;
  a.omega = omega; a.inclination = inclination; a.image_order_limit = image_order_limit;
  a.atm_ext = atm_ext;
  a.stokes = stokes;
  a.radiates = dR.as<int32_t>();
  a.cellArea = dA.as<double>(); a.phi = dphi.as<double>(); a.params = dpar.as<double>();
  a.n_params = (int)n_params;
  a.correction = correction ? dcorr.as<double>() : nullptr;
  a.n_correction = (int)n_correction;
  a.radius = drad.as<double>(); a.u = du.as<double>(); a.cos_gamma = dcg.as<double>();
  a.theta0 = dth0.as<double>(); a.maxDeflection = dMD.as<double>();
  a.deflection = dD.as<double>(); a.cos_alpha = dCA.as<double>(); a.lag = dL.as<double>();
  a.energies = dE.as<double>(); a.leaves = dLv.as<double>(); a.phases = dP.as<double>();
  a.atmos = A;
  a.table_q = dQ;
  a.chi2 = dchi.as<double>();
  a.eG = deG.as<double>(); a.eZ = deZ.as<double>(); a.eA = deA.as<double>();
  a.n_img = dimg.as<int32_t>();
  a.partial = dpart.as<double>();
  a.flux = dF.as<double>();
  a.flux_q = stokes ? dFq.as<double>() : nullptr;
  a.flux_u = stokes ? dFq.as<double>() + N_E * N_P : nullptr;
  a.status = dst.as<int32_t>();
  rc = xg::launch_general(a, st);
  if (rc == -2) return fail_msg("integrator shared memory too large");
  CK(cudaGetLastError());
  int32_t status = 0;
  CK(cudaMemcpyAsync(&status, dst.p, 4, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(flux, dF.p, N_E * N_P * 8, cudaMemcpyDeviceToHost, st));
  if (stokes) {
    CK(cudaMemcpyAsync(flux_Q, a.flux_q, N_E * N_P * 8, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(flux_U, a.flux_u, N_E * N_P * 8, cudaMemcpyDeviceToHost, st));
  }
  CK(cudaStreamSynchronize(st));
  if (status == XGPU_BAD_INPUT) return fail_msg("a parallel has more images than held");
  return status != 0 ? 1 : 0;
}
}  // namespace

extern "C" {

int xgpu_integrate_general(double R, double omega, double r_s, double inclination, size_t S0,
                           size_t S1, const double *cellArea, const double *radius,
                           const double *r_s_over_r, const double *theta, const double *phi,
                           const double *srcCellParams, size_t n_params,
                           const int32_t *radiates, const double *correction,
                           size_t n_correction, size_t N_R, const double *deflection,
                           const double *cos_alpha, const double *lag,
                           const double *maxDeflection, const double *cos_gamma, size_t N_E,
                           const double *energies, size_t N_L, const double *leaves,
                           size_t N_P, const double *phases, int atm_ext,
                           const xgpu_atmos4d *atmos, int else_atm_ext, int image_order_limit,
                           double *flux) {
  (void)R;
  (void)r_s;
  cudaStream_t st;
  int rc;
  if ((rc = lib_stream(&st))) return rc;
  if (atm_ext < 1 || atm_ext > 4)
    return fail_msg("atm_ext must be 1 (BB), 2 (Num4D), 3 (burst BB) or 4 (Pol_Num2D)");
  if ((atm_ext == 2 || atm_ext == 4) && !atmos)
    return fail_msg("numerical atmospheres (atm_ext 2, 4) need the table");
  xg::Atmos4D A{};
  Dev dt;
  if (atm_ext == 2 && (rc = atmos_device(atmos, st, &A))) return rc;
  if (atm_ext == 4 && (rc = table2d_device(st, atmos, nullptr, dt, &A, nullptr))) return rc;
  return general_host(st, omega, inclination, S0, S1, cellArea, radius, r_s_over_r, theta, phi,
                      srcCellParams, n_params, radiates, correction, n_correction, N_R,
                      deflection, cos_alpha, lag, maxDeflection, cos_gamma, N_E, energies, N_L,
                      leaves, N_P, phases, atm_ext, A, nullptr, else_atm_ext,
                      image_order_limit, flux, nullptr, nullptr);
}

int xgpu_integrate_general_stokes(double R, double omega, double r_s, double inclination,
                                  size_t S0, size_t S1, const double *cellArea,
                                  const double *radius, const double *r_s_over_r,
                                  const double *theta, const double *phi,
                                  const double *srcCellParams, size_t n_params,
                                  const int32_t *radiates, const double *correction,
                                  size_t n_correction, size_t N_R, const double *deflection,
                                  const double *cos_alpha, const double *lag,
                                  const double *maxDeflection, const double *cos_gamma,
                                  size_t N_E, const double *energies, size_t N_L,
                                  const double *leaves, size_t N_P, const double *phases,
                                  int atm_ext, const xgpu_atmos4d *atmos_I,
                                  const xgpu_atmos4d *atmos_Q, int else_atm_ext,
                                  int image_order_limit, double *flux_I, double *flux_Q,
                                  double *flux_U) {
  (void)R;
  (void)r_s;
  cudaStream_t st;
  int rc;
  if ((rc = lib_stream(&st))) return rc;
  if (atm_ext < 1 || atm_ext > 4)
    return fail_msg("atm_ext must be 1 (BB), 2 (Num4D), 3 (burst BB) or 4 (Pol_Num2D)");
  if (atm_ext == 2 && !atmos_I) return fail_msg("atm_ext 2 (Num4D) needs the I table");
  if (atm_ext == 4 && (!atmos_I || !atmos_Q))
    return fail_msg("atm_ext 4 (Pol_Num2D) needs the I and Q tables");
  xg::Atmos4D A{};
  const double *dQ = nullptr;
  Dev dt;
  if (atm_ext == 2 && (rc = atmos_device(atmos_I, st, &A))) return rc;
  if (atm_ext == 4 && (rc = table2d_device(st, atmos_I, atmos_Q, dt, &A, &dQ))) return rc;
  return general_host(st, omega, inclination, S0, S1, cellArea, radius, r_s_over_r, theta, phi,
                      srcCellParams, n_params, radiates, correction, n_correction, N_R,
                      deflection, cos_alpha, lag, maxDeflection, cos_gamma, N_E, energies, N_L,
                      leaves, N_P, phases, atm_ext, A, dQ, else_atm_ext, image_order_limit,
                      flux_I, flux_Q, flux_U);
}

int xgpu_energy_integrator(size_t N_E, size_t N_P, const double *signal,
                           const double *log10_energies, size_t n_edges,
                           const double *log10_edges, double *out) {
  cudaStream_t st;
  int rc;
  if ((rc = lib_stream(&st))) return rc;
  if (n_edges < 2) return 0;
  int64_t zero = 0;
  Dev ds, dE, ded, dout, doff;
  size_t nout = (n_edges - 1) * N_P;
  if ((rc = upload(ds, signal, N_E * N_P, st)) || (rc = upload(dE, log10_energies, N_E, st)) ||
      (rc = upload(ded, log10_edges, n_edges, st)) || (rc = dalloc(dout, nout * 8, st)) ||
      (rc = upload(doff, &zero, 1, st)))
    return rc;
  CK(cudaMemsetAsync(dout.p, 0, nout * 8, st));
  rc = xgpu_energy_batch(1, (int)N_E, (int)N_P, (int)n_edges, ds.as<double>(),
                         doff.as<int64_t>(), dE.as<double>(), ded.as<double>(), nullptr,
                         dout.as<double>(), doff.as<int64_t>(), 0, st);
  if (rc) return rc;
  CK(cudaMemcpyAsync(out, dout.p, nout * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return 0;
}

int xgpu_response_fold(size_t K, size_t q, size_t N, const double *matrix, size_t ld,
                       const double *signal, double *out) {
  cudaStream_t st;
  int rc;
  if ((rc = lib_stream(&st))) return rc;
  Dev dM, ds, dout;
  if ((rc = upload(dM, matrix, K * ld, st)) || (rc = upload(ds, signal, q * N, st)) ||
      (rc = dalloc(dout, K * N * 8, st)))
    return rc;
  rc = xgpu_fold_batch(1, (int)K, (int)q, (int)N, dM.as<double>(), (int)ld, ds.as<double>(),
                       dout.as<double>(), st);
  if (rc) return rc;
  CK(cudaMemcpyAsync(out, dout.p, K * N * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return 0;
}

int xgpu_precomputation(size_t K, size_t B, const int32_t *counts, double *out) {
  cudaStream_t st;
  int rc;
  if ((rc = lib_stream(&st))) return rc;
  Dev dc, dout;
  if ((rc = upload(dc, counts, K * B, st)) || (rc = dalloc(dout, K * 8, st))) return rc;
  xg::launch_precomputation((int)K, (int)B, dc.as<int32_t>(), dout.as<double>(), st);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(out, dout.p, K * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return 0;
}

int xgpu_eval_marginal_likelihood(double exposure_time, size_t B, const double *phase_edges,
                                  size_t K, const double *counts, size_t H,
                                  const double *const *components, const size_t *n_phases,
                                  const double *const *component_phases,
                                  const double *phase_shifts, const double *precomp,
                                  const double *support, double epsabs, double epsrel,
                                  double epsilon, double sigmas, double llzero,
                                  const int32_t *allow_negative, double slim,
                                  const double *background, double *loglike, double *star,
                                  double *mcl_bg, double *mcl_bg_support) {
  cudaStream_t st;
  int rc;
  if ((rc = lib_stream(&st))) return rc;
  if (H == 0) return fail_msg("at least one component is needed");
  const size_t N_P = n_phases[0];
  for (size_t h = 1; h < H; h++) {
    if (n_phases[h] != N_P ||
        std::memcmp(component_phases[h], component_phases[0], N_P * sizeof(double)) != 0)
      return fail_msg("components must share one phase grid");
  }
  std::vector<double> sig(H * K * N_P);
  for (size_t h = 0; h < H; h++)
    std::memcpy(sig.data() + h * K * N_P, components[h], K * N_P * sizeof(double));
  Dev dpe, dcp, dcnt, dpre, dsup, dbg, dsig, dsh, dan, dll, dfl, dstar, dmb, dmbs, dL, dS;
  if ((rc = upload(dpe, phase_edges, B + 1, st)) ||
      (rc = upload(dcp, component_phases[0], N_P, st)) || (rc = upload(dcnt, counts, K * B, st)) ||
      (rc = upload(dpre, precomp, K, st)) || (rc = upload(dsup, support, 2 * K, st)) ||
      (rc = upload(dsig, sig.data(), sig.size(), st)) || (rc = upload(dsh, phase_shifts, H, st)) ||
      (rc = upload(dan, allow_negative, H, st)) || (rc = dalloc(dll, K * 8, st)) ||
      (rc = dalloc(dfl, K * 4, st)) || (rc = dalloc(dstar, K * B * 8, st)) ||
      (rc = dalloc(dmb, K * 8, st)) || (rc = dalloc(dmbs, K * 8, st)) ||
      (rc = dalloc(dL, 8, st)) || (rc = dalloc(dS, 4, st)))
    return rc;
  if (background && (rc = upload(dbg, background, K * B, st))) return rc;
  CK(cudaMemsetAsync(dmb.p, 0, K * 8, st));
  CK(cudaMemsetAsync(dmbs.p, 0, K * 8, st));
  xgpu_likelihood_batch_data d{};
  d.n_vec = 1; d.K = (int32_t)K; d.B = (int32_t)B; d.H = (int32_t)H; d.N_P = (int32_t)N_P;
  d.exposure = exposure_time; d.epsabs = epsabs; d.epsrel = epsrel; d.epsilon = epsilon;
  d.sigmas = sigmas; d.llzero = llzero; d.slim = slim;
  d.phase_edges = dpe.as<double>(); d.comp_phases = dcp.as<double>();
  d.counts = dcnt.as<double>(); d.precomp = dpre.as<double>(); d.support = dsup.as<double>();
  d.background = background ? dbg.as<double>() : nullptr;
  d.signals = dsig.as<double>(); d.shifts = dsh.as<double>();
  d.allow_negative = dan.as<int32_t>();
  d.chan_ll = dll.as<double>(); d.chan_flag = dfl.as<int32_t>();
  d.star = dstar.as<double>(); d.mcl_bg = dmb.as<double>(); d.mcl_bg_support = dmbs.as<double>();
  d.loglike = dL.as<double>(); d.status = dS.as<int32_t>();
  rc = xgpu_likelihood_batch(&d, st);
  if (rc) return rc;
  int32_t status = 0;
  std::vector<int32_t> flags(K);
  CK(cudaMemcpyAsync(loglike, dL.p, 8, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(&status, dS.p, 4, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(flags.data(), dfl.p, K * 4, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(star, dstar.p, K * B * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(mcl_bg, dmb.p, K * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(mcl_bg_support, dmbs.p, K * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  // channels after an early exit are left as the reference leaves them (zero)
  for (size_t ch = 0; ch < K; ch++) {
    if (flags[ch] != 0) {
      size_t first_zero = (flags[ch] == 1) ? ch + 1 : ch + 1;
      for (size_t c2 = first_zero; c2 < K; c2++) {
        std::memset(star + c2 * B, 0, B * sizeof(double));
        mcl_bg[c2] = 0.0;
        mcl_bg_support[c2] = 0.0;
      }
      break;
    }
  }
  return status;
}

// ------------------------------------------------------------ elsewhere
int xgpu_elsewhere_batch(int n_meshes, const xgpu_elsewhere_mesh *meshes, int64_t n_rows,
                         int N_R, int N_E, int max_images, const xgpu_elsewhere_batch_data *d,
                         void *stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (n_meshes <= 0) return 0;
  if (N_R < 3) return fail_msg("num_rays must be at least 3");
  if (N_E < 1) return fail_msg("at least one energy is needed");
  if (max_images <= 0) max_images = 8;
  int max_S = 0;
  int64_t rows = 0;
  for (int m = 0; m < n_meshes; m++) {
    const xgpu_elsewhere_mesh &M = meshes[m];
    if (M.atm_ext != 1 && M.atm_ext != 2) return fail_msg("atm_ext must be 1 (BB) or 2 (Num4D)");
    if (M.atm_ext == 2 && d->atmos.intensity == nullptr)
      return fail_msg("a Num4D mesh needs the atmosphere table");
    if (M.atm_ext == 2 && (d->atmos.nT < 4 || d->atmos.ng < 4 || d->atmos.nmu < 4 ||
                           d->atmos.nE < 4))
      return fail_msg("Num4D grids need at least 4 nodes per dimension");
    if (M.atm_ext == 2 && d->n_params < 2)
      return fail_msg("Num4D needs (log T, log g) per cell");
    if (M.S < 1 || M.row_off < 0 || M.row_off + M.S > n_rows)
      return fail_msg("closed mesh rows outside the packed parallels");
    max_S = std::max(max_S, (int)M.S);
    rows += M.S;
  }
  if (n_rows > INT32_MAX) return fail_msg("too many parallels in one launch");
  if (xg::elsewhere_smem_bytes(N_R, max_S, max_images) > 227 * 1024)
    return fail_msg("closed mesh too large for one CTA's shared memory");
  Dev dm, drow;
  int rc;
  static_assert(sizeof(xgpu_elsewhere_mesh) == sizeof(xg::ElseMeshDesc), "elsewhere layout");
  if ((rc = upload(dm, reinterpret_cast<const xg::ElseMeshDesc *>(meshes), n_meshes, st)))
    return rc;
  if ((rc = dalloc(drow, (size_t)n_rows * N_E * sizeof(double), st))) return rc;
  CK(cudaMemsetAsync(drow.p, 0, (size_t)n_rows * N_E * sizeof(double), st));
  CK(cudaMemsetAsync(d->mesh_status, 0, n_meshes * sizeof(int32_t), st));
  xg::ElsewhereArgs a{};
  a.n_meshes = n_meshes;
  a.n_rows = n_rows;
  a.N_R = N_R;
  a.N_E = N_E;
  a.max_S = max_S;
  a.max_images = max_images;
  a.meshes = dm.as<xg::ElseMeshDesc>();
  a.row_mesh = d->row_mesh;
  a.radius = d->radius; a.u = d->u; a.cos_gamma = d->cos_gamma; a.theta0 = d->theta0;
  a.maxDeflection = d->maxDeflection;
  a.deflection = d->deflection; a.cos_alpha = d->cos_alpha;
  a.phi = d->phi; a.params = d->params; a.n_params = d->n_params;
  a.energies = d->energies;
  a.atmos = xg::Atmos4D{d->atmos.logT, d->atmos.logg, d->atmos.mu, d->atmos.logE,
                        d->atmos.intensity, (int)d->atmos.nT, (int)d->atmos.ng,
                        (int)d->atmos.nmu, (int)d->atmos.nE, nullptr};
  a.row_flux = drow.as<double>();
  a.flux = d->flux;
  a.status = d->mesh_status;
  a.signal = d->signal;
  a.signal_stride = d->signal_stride;
  a.signal_N_P = d->signal_N_P;
  rc = xg::launch_elsewhere(a, st);
  if (rc == -2) return fail_msg("closed mesh too large for one CTA's shared memory");
  CK(cudaGetLastError());
  return rc;
}

int xgpu_integrate_time_invariant(double R, double omega, double r_s, double inclination,
                                  size_t S, double cellArea, const double *radius,
                                  const double *r_s_over_r, const double *theta,
                                  const double *phi, const double *srcCellParams,
                                  size_t n_params, size_t N_R, const double *deflection,
                                  const double *cos_alpha, const double *maxDeflection,
                                  const double *cos_gamma, size_t N_E, const double *energies,
                                  int atm_ext, const xgpu_atmos4d *atmos, int image_order_limit,
                                  double *flux) {
  (void)R;
  (void)r_s;
  cudaStream_t st;
  int rc;
  if ((rc = lib_stream(&st))) return rc;
  if (S == 0 || N_E == 0) return 0;
  if (n_params < 1) return fail_msg("srcCellParams needs at least 1 parameter per cell");
  if (atm_ext == 2 && !atmos) return fail_msg("atm_ext 2 (Num4D) needs the atmosphere");
  xg::Atmos4D A{};
  if (atm_ext == 2 && (rc = atmos_device(atmos, st, &A))) return rc;
  const size_t cells = S * S;
  std::vector<double> theta0(S);
  for (size_t i = 0; i < S; i++) theta0[i] = theta[i * S];
  std::vector<int32_t> row_mesh(S, 0);
  Dev drad, du, dth0, dphi, dpar, dD, dCA, dMD, dcg, dE, dF, dst, drm;
  if ((rc = upload(drad, radius, S, st)) || (rc = upload(du, r_s_over_r, S, st)) ||
      (rc = upload(dth0, theta0.data(), S, st)) || (rc = upload(dphi, phi, cells, st)) ||
      (rc = upload(dpar, srcCellParams, cells * n_params, st)) ||
      (rc = upload(dD, deflection, S * N_R, st)) || (rc = upload(dCA, cos_alpha, S * N_R, st)) ||
      (rc = upload(dMD, maxDeflection, S, st)) || (rc = upload(dcg, cos_gamma, S, st)) ||
      (rc = upload(dE, energies, N_E, st)) || (rc = dalloc(dF, N_E * 8, st)) ||
      (rc = dalloc(dst, 16, st)) || (rc = upload(drm, row_mesh.data(), S, st)))
    return rc;
  xgpu_elsewhere_mesh mesh{(int32_t)S, 0, 0, omega, inclination, cellArea, image_order_limit,
                           atm_ext};
  xgpu_elsewhere_batch_data d{};
  d.row_mesh = drm.as<int32_t>();
  d.radius = drad.as<double>(); d.u = du.as<double>(); d.cos_gamma = dcg.as<double>();
  d.theta0 = dth0.as<double>(); d.maxDeflection = dMD.as<double>();
  d.deflection = dD.as<double>(); d.cos_alpha = dCA.as<double>();
  d.phi = dphi.as<double>(); d.params = dpar.as<double>(); d.n_params = (int32_t)n_params;
  d.energies = dE.as<double>();
  if (atm_ext == 2)
    d.atmos = xgpu_atmos4d{A.logT, A.logg, A.mu, A.logE, A.I, (size_t)A.nT, (size_t)A.ng,
                           (size_t)A.nmu, (size_t)A.nE, nullptr};
  d.flux = dF.as<double>();
  d.mesh_status = dst.as<int32_t>();
  rc = xgpu_elsewhere_batch(1, &mesh, (int64_t)S, (int)N_R, (int)N_E, 0, &d, st);
  if (rc) return rc;
  int32_t status = 0;
  CK(cudaMemcpyAsync(&status, dst.p, 4, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(flux, dF.p, N_E * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (status == XGPU_BAD_INPUT) return fail_msg("a parallel has more than 8 images");
  return status != 0 ? 1 : 0;
}

// ------------------------------------------------------------- synthesis
int xgpu_expected_counts_batch(int n_sets, int K, int B, int H, double exposure,
                               const double *phase_edges, const xgpu_component *components,
                               const int32_t *allow_negative, const double *background,
                               double *out, void *stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (n_sets <= 0 || K <= 0 || B <= 0) return 0;
  if (H <= 0) return fail_msg("at least one component is needed");
  static_assert(sizeof(xgpu_component) == sizeof(xg::CompDesc), "component layout");
  for (int64_t c = 0; c < (int64_t)n_sets * H; c++)
    if (components[c].n < 1 || (components[c].n > 1 && components[c].n < 5))
      return fail_msg("a component needs one phase or at least five (Akima spline)");
  Dev dc;
  int rc;
  if ((rc = upload(dc, reinterpret_cast<const xg::CompDesc *>(components),
                   (size_t)n_sets * H, st)))
    return rc;
  xg::ExpectedArgs a{n_sets, K, B, H, exposure, phase_edges, dc.as<xg::CompDesc>(),
                     allow_negative, background, out};
  xg::launch_expected_counts(a, st);
  CK(cudaGetLastError());
  return 0;
}

int xgpu_poisson_batch(int64_t n, const double *mean, double *out, uint64_t seed,
                       uint64_t offset, int32_t *fail_flag, void *stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (n <= 0) return 0;
  Dev df;
  int rc;
  if (!fail_flag) {
    if ((rc = dalloc(df, 16, st))) return rc;
    fail_flag = df.as<int32_t>();
    CK(cudaMemsetAsync(fail_flag, 0, 4, st));
  }
  xg::launch_poisson(n, mean, out, seed, offset, fail_flag, st);
  CK(cudaGetLastError());
  return 0;
}

int xgpu_compute_expected_counts(double exposure_time, size_t B, const double *phases, size_t K,
                                 size_t H, const xgpu_component *components,
                                 const double *background, const int32_t *allow_negative,
                                 double *out) {
  cudaStream_t st;
  int rc;
  if ((rc = lib_stream(&st))) return rc;
  if (K == 0 || B == 0) return 0;
  if (H == 0) return fail_msg("at least one component is needed");
  std::vector<Dev> keep(2 * H);
  std::vector<xgpu_component> dcomp(H);
  for (size_t h = 0; h < H; h++) {
    const xgpu_component &c = components[h];
    if (c.n < 1 || c.ld < c.n) return fail_msg("component shape is invalid");
    if ((rc = upload(keep[2 * h], c.signal, K * (size_t)c.ld, st)) ||
        (rc = upload(keep[2 * h + 1], c.phases, (size_t)c.n, st)))
      return rc;
    dcomp[h] = xgpu_component{keep[2 * h].as<double>(), keep[2 * h + 1].as<double>(), c.ld, c.n,
                              c.shift};
  }
  Dev de, dneg, dbg, dout;
  if ((rc = upload(de, phases, B + 1, st)) || (rc = upload(dneg, allow_negative, H, st)) ||
      (background && (rc = upload(dbg, background, K * B, st))) ||
      (rc = dalloc(dout, K * B * 8, st)))
    return rc;
  rc = xgpu_expected_counts_batch(1, (int)K, (int)B, (int)H, exposure_time, de.as<double>(),
                                  dcomp.data(), dneg.as<int32_t>(),
                                  background ? dbg.as<double>() : nullptr, dout.as<double>(), st);
  if (rc) return rc;
  CK(cudaMemcpyAsync(out, dout.p, K * B * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return 0;
}

int xgpu_poisson_loglike_batch(int n_sets, int K, int B, const double *expected,
                               const double *counts, const double *precomp, double *loglike,
                               int32_t *n_penalty, void *stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (n_sets <= 0 || K <= 0) return 0;
  if (B <= 0) return fail_msg("at least one phase bin is needed");
  Dev dll, dpen;
  int rc;
  if ((rc = dalloc(dll, (size_t)n_sets * K * 8, st)) ||
      (rc = dalloc(dpen, (size_t)n_sets * K * 4, st)))
    return rc;
  xg::PoissonArgs a{n_sets, K, B, expected, counts, precomp, dll.as<double>(),
                    dpen.as<int32_t>(), loglike, n_penalty};
  xg::launch_poisson_loglike(a, st);
  CK(cudaGetLastError());
  return 0;
}

int xgpu_poisson_likelihood_given_background(double exposure_time, size_t B,
                                             const double *phases, size_t K,
                                             const double *counts, size_t H,
                                             const xgpu_component *components,
                                             const double *background,
                                             const double *neg_sum_ln_data_factorial,
                                             const int32_t *allow_negative, double *expected,
                                             double *loglike, int64_t *n_penalty) {
  cudaStream_t st;
  int rc;
  if ((rc = lib_stream(&st))) return rc;
  if (K == 0 || B == 0) {
    *loglike = 0.0;
    *n_penalty = 0;
    return 0;
  }
  if ((rc = xgpu_compute_expected_counts(exposure_time, B, phases, K, H, components, background,
                                         allow_negative, expected)))
    return rc;
  Dev dE, dC, dP, dL, dN;
  if ((rc = upload(dE, expected, K * B, st)) || (rc = upload(dC, counts, K * B, st)) ||
      (neg_sum_ln_data_factorial && (rc = upload(dP, neg_sum_ln_data_factorial, K, st))) ||
      (rc = dalloc(dL, 8, st)) || (rc = dalloc(dN, 4, st)))
    return rc;
  rc = xgpu_poisson_loglike_batch(1, (int)K, (int)B, dE.as<double>(), dC.as<double>(),
                                  neg_sum_ln_data_factorial ? dP.as<double>() : nullptr,
                                  dL.as<double>(), dN.as<int32_t>(), st);
  if (rc) return rc;
  int32_t pen = 0;
  CK(cudaMemcpyAsync(loglike, dL.p, 8, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(&pen, dN.p, 4, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  *n_penalty = pen;
  return 0;
}

int xgpu_phase_integrator(double exposure_time, size_t n_edges, const double *phases, size_t rows,
                          size_t n_phases, const double *signal, const double *signal_phases,
                          double phase_shift, int allow_negative, double *out) {
  cudaStream_t st;
  int rc;
  if ((rc = lib_stream(&st))) return rc;
  if (rows == 0 || n_edges < 2) return 0;
  if (n_phases < 5) return fail_msg("the signal needs at least five phases (Akima spline)");
  const size_t B = n_edges - 1;
  Dev de, ds, dp, dout;
  if ((rc = upload(de, phases, n_edges, st)) || (rc = upload(ds, signal, rows * n_phases, st)) ||
      (rc = upload(dp, signal_phases, n_phases, st)) || (rc = dalloc(dout, rows * B * 8, st)))
    return rc;
  xg::PhaseIntArgs a{(int64_t)rows, (int)n_phases, (int)B, exposure_time, phase_shift,
                     allow_negative ? 1 : 0, de.as<double>(), ds.as<double>(), dp.as<double>(),
                     dout.as<double>()};
  xg::launch_phase_integrator(a, st);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(out, dout.p, rows * B * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return 0;
}

int xgpu_phase_interpolator(size_t n_new, const double *new_phases, size_t n_phases,
                            const double *phases, size_t rows, const double *signal,
                            double phase_shift, int allow_negative, double *out) {
  cudaStream_t st;
  int rc;
  if ((rc = lib_stream(&st))) return rc;
  if (rows == 0 || n_new == 0) return 0;
  if (n_phases < 5) return fail_msg("the signal needs at least five phases (Akima spline)");
  Dev dn, dp, ds, dout;
  if ((rc = upload(dn, new_phases, n_new, st)) || (rc = upload(dp, phases, n_phases, st)) ||
      (rc = upload(ds, signal, rows * n_phases, st)) || (rc = dalloc(dout, rows * n_new * 8, st)))
    return rc;
  xg::InterpArgs a{(int64_t)rows, (int)n_phases, (int)n_new, dp.as<double>(), dn.as<double>(),
                   ds.as<double>(), phase_shift, allow_negative ? 1 : 0, dout.as<double>()};
  xg::launch_phase_interpolator(a, st);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(out, dout.p, rows * n_new * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return 0;
}

int xgpu_energy_interpolator(size_t N_E, size_t n_cols, const double *signal,
                             const double *log10_energies, size_t n_new,
                             const double *log10_new_energies, double *out) {
  cudaStream_t st;
  int rc;
  if ((rc = lib_stream(&st))) return rc;
  if (n_cols == 0 || n_new == 0) return 0;
  if (N_E < 3) return fail_msg("at least three energies are needed (Steffen spline)");
  Dev dE, dn, ds, dout;
  if ((rc = upload(dE, log10_energies, N_E, st)) ||
      (rc = upload(dn, log10_new_energies, n_new, st)) ||
      (rc = upload(ds, signal, N_E * n_cols, st)) || (rc = dalloc(dout, n_new * n_cols * 8, st)))
    return rc;
  xg::InterpArgs a{(int64_t)n_cols, (int)N_E, (int)n_new, dE.as<double>(), dn.as<double>(),
                   ds.as<double>(), 0.0, 0, dout.as<double>()};
  xg::launch_energy_interpolator(a, st);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(out, dout.p, n_new * n_cols * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return 0;
}

int xgpu_poisson(size_t n, const double *mean, uint64_t seed, uint64_t offset, double *out) {
  cudaStream_t st;
  int rc;
  if ((rc = lib_stream(&st))) return rc;
  if (n == 0) return 0;
  Dev dm, dout, df;
  if ((rc = upload(dm, mean, n, st)) || (rc = dalloc(dout, n * 8, st)) ||
      (rc = dalloc(df, 16, st)))
    return rc;
  CK(cudaMemsetAsync(df.p, 0, 4, st));
  if ((rc = xgpu_poisson_batch((int64_t)n, dm.as<double>(), dout.as<double>(), seed, offset,
                               df.as<int32_t>(), st)))
    return rc;
  int32_t hit_bound = 0;
  CK(cudaMemcpyAsync(out, dout.p, n * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(&hit_bound, df.p, 4, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return hit_bound ? 1 : 0;
}

int xgpu_gaussian_loglike_batch(int n_sets, int rows, int cols, const double *model,
                                int64_t model_set_stride, int64_t model_row_stride,
                                const double *data, const double *errors, double *loglike,
                                void *stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (n_sets <= 0) return 0;
  xg::launch_gaussian(n_sets, rows, cols, model, model_set_stride, model_row_stride, data,
                      errors, loglike, st);
  CK(cudaGetLastError());
  return 0;
}

int xgpu_gaussian_loglike(size_t rows, size_t cols, const double *model,
                          size_t model_row_stride, const double *data, const double *errors,
                          double *loglike) {
  cudaStream_t st;
  int rc;
  if ((rc = lib_stream(&st))) return rc;
  if (rows == 0 || cols == 0) {
    *loglike = 0.0;
    return 0;
  }
  const size_t model_n = model_row_stride ? (rows - 1) * model_row_stride + cols : cols;
  Dev dm, dd, de, dl;
  if ((rc = upload(dm, model, model_n, st)) || (rc = upload(dd, data, rows * cols, st)) ||
      (rc = upload(de, errors, rows * cols, st)) || (rc = dalloc(dl, 8, st)))
    return rc;
  if ((rc = xgpu_gaussian_loglike_batch(1, (int)rows, (int)cols, dm.as<double>(), 0,
                                        (int64_t)model_row_stride, dd.as<double>(),
                                        de.as<double>(), dl.as<double>(), st)))
    return rc;
  CK(cudaMemcpyAsync(loglike, dl.p, 8, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return 0;
}

}  // extern "C"
