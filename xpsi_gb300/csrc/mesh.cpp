// mesh.cpp -- host-side cell meshes: the cell budget
// (xpsi/cellmesh/mesh_tools.pyx:892-1099, allocate_cells), the hot-region
// spot / polar-cap meshes (xpsi/cellmesh/mesh.pyx:23-417,
// polar_mesh.pyx:23-430) and the closed mesh of the photosphere elsewhere
// (xpsi/cellmesh/global_mesh.pyx:21-137), built from the shared steps of
// mesh_math.h.  Meshes of many parameter
// vectors are built concurrently on the host's cores (one std::thread per
// slice); mesh_gpu.cu builds the same meshes on the GPU.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <thread>
#include <vector>

#include "../../include/xpsi_gb300.h"
#include "mesh_math.h"

namespace {

using namespace xgm;
using Work = WorkT<4000>;

struct MeshOut {
  double *theta, *phi, *r, *area, *maxAlpha, *cos_gamma, *effGrav;
};

// mesh.pyx:23-417 (polar = false) and polar_mesh.pyx:23-430 (polar = true)
int build_mesh(bool polar, size_t numCell, size_t S, const Star &s, double cedeRadius,
               double cedeColat, double superRadius, double superColat, double superAzi,
               const MeshOut &o, Work &w) {
  if (S < 2) return -1;
  MeshPlan pl;
  mesh_plan(polar, numCell, S, cedeRadius, cedeColat, superRadius, superColat, superAzi, pl);
  std::vector<double> colat(kAreaTab), areaTab(kAreaTab), parallels(S - 1), colatC(S);
  for (int i = 0; i < kAreaTab; i++) {
    colat[i] = mesh_table_colat(pl, i);
    areaTab[i] = integrateArea(colat[i], pl.lims[1], s, 0, w);
  }
  double cellArea, eta;
  mesh_cell_area(pl, areaTab[kAreaTab - 1], cellArea, eta);
  mesh_parallels(pl, colat.data(), areaTab.data(), eta, parallels.data());
  for (size_t j = 0; j < S * S; j++) o.area[j] = 0.0;
  for (size_t i = 0; i < S; i++) {
    double lower, upper;
    mesh_row_bounds(pl, parallels.data(), i, lower, upper);
    const RowOut r = mesh_row(s, lower, upper, eta, w);
    colatC[i] = r.colat;
    o.r[i] = r.r;
    o.effGrav[i] = r.effGrav;
    o.cos_gamma[i] = r.cos_gamma;
    o.maxAlpha[i] = r.maxAlpha;
    for (size_t j = 0; j < pl.j_max; j++) {
      const double A = mesh_cell(pl, s, i, j, lower, upper, colatC[i], cellArea, w);
      o.area[i * S + j] = A;
      if (pl.sym) o.area[i * S + (S - 1 - j)] = A;
    }
  }
  for (size_t i = 0; i < S; i++)
    for (size_t j = 0; j < S; j++) {
      o.theta[i * S + j] = pl.invert ? PI - colatC[i] : colatC[i];
      o.phi[i * S + j] = mesh_phi(pl, j);
    }
  return 0;
}

// global_mesh.pyx:21-137: the closed mesh of the whole star.  S rows of
// equal area (the northern S/2 computed, the southern mirrored) by S cells of
// equal azimuth width; every cell has the same area.
int build_closed_mesh(size_t S, size_t numCell, const Star &s, double *theta, double *phi,
                      double *r, double *cellArea_out, double *maxAlpha, double *cos_gamma,
                      double *effGrav, Work &w) {
  if (S < 4 || S % 2 != 0 || numCell == 0) return -1;
  const size_t nc = S / 2;
  double cellArea = TWO_PI * integrateArea(0.0, PI_2, s, 0, w) / (double)numCell;
  cellArea *= 2.0;
  const double eta = cellArea * (double)S / TWO_PI;
  // np.linspace(pi/2, 0, 1000) and the area from each colatitude to the equator
  std::vector<double> colat(kAreaTab), areaTab(kAreaTab), parallels(nc - 1), colatC(S);
  const double step = (0.0 - PI_2) / (double)(kAreaTab - 1);
  for (int i = 0; i < kAreaTab; i++) {
    colat[i] = (i == kAreaTab - 1) ? 0.0 : PI_2 + (double)i * step;
    areaTab[i] = integrateArea(colat[i], PI_2, s, 0, w);
  }
  double i_eta = (double)nc * eta;
  for (size_t i = 0; i + 1 < nc; i++) {
    i_eta -= eta;
    parallels[i] = steffen_at(areaTab.data(), colat.data(), kAreaTab, i_eta);
  }
  for (size_t i = 0; i < nc; i++) {
    const double lower = (i == 0) ? 0.0 : parallels[i - 1];
    const double upper = (i == nc - 1) ? PI_2 : parallels[i];
    const RowOut o = mesh_row(s, lower, upper, eta, w);
    colatC[i] = o.colat;
    r[i] = o.r;
    effGrav[i] = o.effGrav;
    cos_gamma[i] = o.cos_gamma;
    maxAlpha[i] = o.maxAlpha;
  }
  for (size_t i = nc; i < S; i++) {
    colatC[i] = PI - colatC[S - i - 1];
    r[i] = r[S - i - 1];
    cos_gamma[i] = cos_gamma[S - i - 1];
    effGrav[i] = effGrav[S - i - 1];
    maxAlpha[i] = maxAlpha[S - i - 1];
  }
  // np.linspace(-pi + d/2, pi - d/2, S) with d = 2 pi / S, as a meshgrid
  const double d = TWO_PI / (double)S;
  const double a = -PI + 0.5 * d, b = PI - 0.5 * d;
  const double pstep = (b - a) / (double)(S - 1);
  for (size_t i = 0; i < S; i++)
    for (size_t j = 0; j < S; j++) {
      theta[i * S + j] = colatC[i];
      phi[i * S + j] = (j == S - 1) ? b : a + (double)j * pstep;
    }
  *cellArea_out = cellArea;
  return 0;
}

// mesh_tools.pyx:892-1099 (returns the superseding mesh side only; X-PSI's
// cede member is allocated by the same formula and is not used here)
void allocate(size_t num_cells, size_t mn, size_t mx, const Star &s, double superRadius,
              double cedeRadius, double superColat, double cedeColat, double superAzi,
              double holeColat, double holeRadius, double holeAzi, double out[4], Work &w) {
  double super_lims[2], super_cellArea, super_bphi, superColat_cpy = superColat;
  if (superColat - superRadius < 0.0 || superColat + superRadius > PI) {
    super_lims[0] = 0.0;
    if (superColat + superRadius > PI) {
      super_lims[1] = PI - superColat + superRadius;
      superColat = PI - superColat;
      holeColat = PI - holeColat;
    } else {
      super_lims[1] = superColat + superRadius;
    }
    super_bphi = PI;
    super_cellArea = TWO_PI;
  } else {
    super_lims[0] = superColat - superRadius;
    super_lims[1] = superColat + superRadius;
    super_bphi = std::asin(std::sin(superRadius) / std::sin(superColat));
    super_cellArea = 2.0 * super_bphi;
  }
  (void)super_bphi;
  super_cellArea *= integrateArea(super_lims[0], super_lims[1], s, 0, w);
  Region gs = make_region(superColat, superRadius, holeRadius, holeAzi, holeColat);
  double super_area = integrateSpot(super_lims[0], super_lims[1], s, gs, w);
  auto clamp_even = [&](double v) {
    if (v < (double)mn) v = (double)mn;
    else if (v > (double)mx) v = (double)mx;
    if ((size_t)v % 2 != 0) v += 1.0;
    return v;
  };
  if (are_equal(cedeRadius, 0.0)) {
    if (are_equal(super_area, 0.0)) super_area = super_cellArea / 1000.0;
    double sq = std::ceil(std::sqrt((double)num_cells * super_cellArea / super_area));
    sq = clamp_even(sq);
    out[0] = sq; out[1] = sq * sq; out[2] = 0.0; out[3] = 0.0;
    return;
  }
  double cede_lims[2], cede_cellArea;
  if (cedeColat - cedeRadius < 0.0 || cedeColat + cedeRadius > PI) {
    cede_lims[0] = 0.0;
    if (cedeColat + cedeRadius > PI) {
      cede_lims[1] = PI - cedeColat + cedeRadius;
      cedeColat = PI - cedeColat;
      superColat = PI - superColat_cpy;
    } else {
      cede_lims[1] = cedeColat + cedeRadius;
      superColat = superColat_cpy;
    }
    cede_cellArea = TWO_PI;
  } else {
    cede_lims[0] = cedeColat - cedeRadius;
    cede_lims[1] = cedeColat + cedeRadius;
    superColat = superColat_cpy;
    cede_cellArea = 2.0 * std::asin(std::sin(cedeRadius) / std::sin(cedeColat));
  }
  cede_cellArea *= integrateArea(cede_lims[0], cede_lims[1], s, 0, w);
  Region gc = make_region(cedeColat, cedeRadius, superRadius, superAzi, superColat);
  double cede_area = integrateSpot(cede_lims[0], cede_lims[1], s, gc, w);
  if (are_equal(super_area, 0.0)) super_area = super_cellArea / 1000.0;
  if (are_equal(cede_area, 0.0)) cede_area = cede_cellArea / 1000.0;
  double y = cede_area / super_area - 1.0, sn, cn;
  if (are_equal(y, 0.0)) { sn = 0.5 * num_cells; cn = 0.5 * num_cells; }
  else { sn = (double)num_cells * ((std::sqrt(1.0 + y) - 1.0) / y); cn = (double)num_cells - sn; }
  double ss = clamp_even(std::ceil(std::sqrt(sn * super_cellArea / super_area)));
  double cs = clamp_even(std::ceil(std::sqrt(cn * cede_cellArea / cede_area)));
  out[0] = ss; out[1] = ss * ss; out[2] = cs; out[3] = cs * cs;
}

}  // namespace

extern "C" {

int xgpu_allocate_cells(size_t num_cells, size_t min_sqrt, size_t max_sqrt, double R_eq,
                        double Omega, double zeta, double epsilon, int star_shape_ind,
                        double super_radius, double cede_radius, double super_colatitude,
                        double cede_colatitude, double super_azimuth, double hole_colatitude,
                        double hole_radius, double hole_azimuth, double *out4) {
  Star s{R_eq, epsilon, zeta, Omega, star_shape_ind};
  std::unique_ptr<Work> w(new Work);
  allocate(num_cells, min_sqrt, max_sqrt, s, super_radius, cede_radius, super_colatitude,
           cede_colatitude, super_azimuth, hole_colatitude, hole_radius, hole_azimuth, out4, *w);
  return 0;
}

int xgpu_cell_mesh(int polar, size_t num_cells, size_t S, double R_eq, double zeta,
                   double epsilon, int star_shape_ind, double cede_radius,
                   double cede_colatitude, double super_radius, double super_colatitude,
                   double super_azimuth, double *theta, double *phi, double *r, double *area,
                   double *maxAlpha, double *cos_gamma, double *effGrav) {
  Star s{R_eq, epsilon, zeta, 0.0, star_shape_ind};
  std::unique_ptr<Work> w(new Work);
  MeshOut o{theta, phi, r, area, maxAlpha, cos_gamma, effGrav};
  return build_mesh(polar != 0, num_cells, S, s, cede_radius, cede_colatitude, super_radius,
                    super_colatitude, super_azimuth, o, *w);
}

int xgpu_closed_cell_mesh(size_t S, size_t num_cells, double R_eq, double zeta,
                          double epsilon, int star_shape_ind, double *theta, double *phi,
                          double *r, double *cellArea, double *maxAlpha, double *cos_gamma,
                          double *effGrav) {
  Star s{R_eq, epsilon, zeta, 0.0, star_shape_ind};
  std::unique_ptr<Work> w(new Work);
  return build_closed_mesh(S, num_cells, s, theta, phi, r, cellArea, maxAlpha, cos_gamma,
                           effGrav, *w);
}

int xgpu_closed_cell_mesh_many(int n, const xgpu_closed_mesh_request *req, int n_threads) {
  if (n <= 0) return 0;
  if (n_threads <= 0) n_threads = (int)std::max(1u, std::thread::hardware_concurrency());
  n_threads = std::min(n_threads, n);
  std::vector<std::thread> pool;
  std::vector<int> rc(n, 0);
  auto work = [&](int t) {
    std::unique_ptr<Work> wp(new Work);
    for (int i = t; i < n; i += n_threads) {
      const xgpu_closed_mesh_request &q = req[i];
      Star s{q.R_eq, q.epsilon, q.zeta, 0.0, q.star_shape_ind};
      rc[i] = build_closed_mesh(q.S, q.num_cells, s, q.theta, q.phi, q.r, q.cellArea,
                                q.maxAlpha, q.cos_gamma, q.effGrav, *wp);
    }
  };
  for (int t = 0; t < n_threads; t++) pool.emplace_back(work, t);
  for (auto &th : pool) th.join();
  for (int i = 0; i < n; i++)
    if (rc[i]) return rc[i];
  return 0;
}

int xgpu_allocate_cells_many(int n, xgpu_alloc_request *req, int n_threads) {
  if (n <= 0) return 0;
  if (n_threads <= 0) n_threads = (int)std::max(1u, std::thread::hardware_concurrency());
  n_threads = std::min(n_threads, n);
  std::vector<std::thread> pool;
  auto work = [&](int t) {
    std::unique_ptr<Work> w(new Work);
    for (int i = t; i < n; i += n_threads) {
      xgpu_alloc_request &q = req[i];
      Star s{q.R_eq, q.epsilon, q.zeta, q.Omega, q.star_shape_ind};
      allocate(q.num_cells, q.min_sqrt, q.max_sqrt, s, q.super_radius, q.cede_radius,
               q.super_colatitude, q.cede_colatitude, q.super_azimuth, q.hole_colatitude,
               q.hole_radius, q.hole_azimuth, q.out, *w);
    }
  };
  for (int t = 0; t < n_threads; t++) pool.emplace_back(work, t);
  for (auto &th : pool) th.join();
  return 0;
}

int xgpu_cell_mesh_many(int n, const xgpu_mesh_request *req, int n_threads) {
  if (n_threads <= 0) n_threads = (int)std::max(1u, std::thread::hardware_concurrency());
  std::vector<std::thread> pool;
  std::vector<int> rc(n, 0);
  auto work = [&](int t) {
    std::unique_ptr<Work> wp(new Work);
    Work &w = *wp;
    for (int i = t; i < n; i += n_threads) {
      const xgpu_mesh_request &q = req[i];
      Star s{q.R_eq, q.epsilon, q.zeta, 0.0, q.star_shape_ind};
      MeshOut o{q.theta, q.phi, q.r, q.area, q.maxAlpha, q.cos_gamma, q.effGrav};
      rc[i] = build_mesh(q.polar != 0, q.num_cells, q.S, s, q.cede_radius, q.cede_colatitude,
                         q.super_radius, q.super_colatitude, q.super_azimuth, o, w);
    }
  };
  for (int t = 0; t < n_threads; t++) pool.emplace_back(work, t);
  for (auto &th : pool) th.join();
  for (int i = 0; i < n; i++)
    if (rc[i]) return rc[i];
  return 0;
}

}  // extern "C"
