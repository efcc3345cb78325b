"""Host-side cell meshes (C++ in the native library), mirroring
xpsi.cellmesh.mesh_tools.allocate_cells (mesh_tools.pyx:892-1099),
xpsi.cellmesh.mesh.construct_spot_cellMesh (mesh.pyx:23-417) and
xpsi.cellmesh.polar_mesh.construct_polar_cellMesh (polar_mesh.pyx:23-430)."""
import ctypes as C

import numpy as np

from .._arr import ptr
from .._native import MeshRequest, check, lib


def allocate_cells(num_cells, min_sqrt_num_cells, max_sqrt_num_cells, mass, r_s, R_eq, Omega,
                   zeta, epsilon, star_shape_ind, superRadius, cedeRadius, superColatitude,
                   cedeColatitude, superAzimuth, holeColatitude, holeRadius, holeAzimuth):
    """Cell budget per member: (super_sqrt, super_num, cede_sqrt, cede_num), with
    the reference's types (floats; integer zeros for the ceding region when
    there is none, mesh_tools.pyx:985-1004)."""
    out = np.zeros(4)
    check(lib().xgpu_allocate_cells(int(num_cells), int(min_sqrt_num_cells),
                                    int(max_sqrt_num_cells), float(R_eq), float(Omega),
                                    float(zeta), float(epsilon), int(star_shape_ind),
                                    float(superRadius), float(cedeRadius),
                                    float(superColatitude), float(cedeColatitude),
                                    float(superAzimuth), float(holeColatitude),
                                    float(holeRadius), float(holeAzimuth), ptr(out)))
    if abs(float(cedeRadius)) < 1.0e-12:
        return (float(out[0]), float(out[1]), 0, 0)
    return (float(out[0]), float(out[1]), float(out[2]), float(out[3]))


def _mesh(polar, numThreads, numCell, sqrt_numCell, mass, r_s, R_eq, zeta, epsilon,
          star_shape_ind, cedeRadius, cedeColatitude, superRadius, superColatitude,
          superAzimuth):
    S = int(sqrt_numCell)
    th = np.empty((S, S)); ph = np.empty((S, S)); A = np.empty((S, S))
    r = np.empty(S); ma = np.empty(S); cg = np.empty(S); g = np.empty(S)
    check(lib().xgpu_cell_mesh(int(polar), int(numCell), S, float(R_eq), float(zeta),
                               float(epsilon), int(star_shape_ind), float(cedeRadius),
                               float(cedeColatitude), float(superRadius),
                               float(superColatitude), float(superAzimuth), ptr(th), ptr(ph),
                               ptr(r), ptr(A), ptr(ma), ptr(cg), ptr(g)))
    return (th, ph, r, A, ma, cg, g)


def construct_spot_cellMesh(*args):
    """(theta, phi, r, cellArea, maxEmissionAngle, cos_gamma, effGrav)."""
    return _mesh(0, *args)


def construct_polar_cellMesh(*args):
    """(theta, phi, r, cellArea, maxEmissionAngle, cos_gamma, effGrav)."""
    return _mesh(1, *args)


def build_many(requests, n_threads=0):
    """Build many meshes concurrently.  Each request is a dict with keys
    polar, num_cells, S, R_eq, zeta, epsilon, star_shape_ind, cede_radius,
    cede_colatitude, super_radius, super_colatitude, super_azimuth; the
    outputs are added to it as arrays."""
    n = len(requests)
    arr = (MeshRequest * n)()
    keep = []
    for i, q in enumerate(requests):
        S = int(q["S"])
        out = dict(theta=np.empty((S, S)), phi=np.empty((S, S)), area=np.empty((S, S)),
                   r=np.empty(S), maxAlpha=np.empty(S), cos_gamma=np.empty(S),
                   effGrav=np.empty(S))
        q.update(out)
        keep.append(out)
        arr[i] = MeshRequest(int(q["polar"]), int(q["num_cells"]), S, float(q["R_eq"]),
                             float(q["zeta"]), float(q["epsilon"]), int(q["star_shape_ind"]),
                             float(q["cede_radius"]), float(q["cede_colatitude"]),
                             float(q["super_radius"]), float(q["super_colatitude"]),
                             float(q["super_azimuth"]), out["theta"].ctypes.data,
                             out["phi"].ctypes.data, out["r"].ctypes.data,
                             out["area"].ctypes.data, out["maxAlpha"].ctypes.data,
                             out["cos_gamma"].ctypes.data, out["effGrav"].ctypes.data)
    check(lib().xgpu_cell_mesh_many(n, arr, int(n_threads)))
    return requests
