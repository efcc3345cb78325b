"""Drop-in for xpsi.cellmesh.global_mesh.construct_closed_cellMesh
(xpsi/cellmesh/global_mesh.pyx:21-137): the closed mesh of the photosphere
elsewhere, built by host C++ in the native library."""
import numpy as np

from .._arr import ptr
from .._native import ClosedMeshRequest, check, lib


def construct_closed_cellMesh(numThreads, sqrt_numCell, numCell, mass, r_s, R_eq, zeta,
                              epsilon, star_shape_ind):
    """(theta[S,S], phi[S,S], r[S], cellArea, maxEmissionAngle[S], cos_gamma[S],
    effGrav[S]) as the reference returns them; cellArea is one float (every
    cell of the closed mesh has the same area).  sqrt_numCell must be even
    and at least 4 (Elsewhere.py:199-212 asks for an even number >= 10)."""
    S = int(sqrt_numCell)
    if S < 4 or S % 2 != 0:
        raise ValueError("sqrt_numCell must be an even integer >= 4")
    th = np.empty((S, S)); ph = np.empty((S, S))
    r = np.empty(S); ma = np.empty(S); cg = np.empty(S); g = np.empty(S)
    area = np.zeros(1)
    check(lib().xgpu_closed_cell_mesh(S, int(numCell), float(R_eq), float(zeta),
                                      float(epsilon), int(star_shape_ind), ptr(th), ptr(ph),
                                      ptr(r), ptr(area), ptr(ma), ptr(cg), ptr(g)))
    return (th, ph, r, float(area[0]), ma, cg, g)


def build_many(requests, n_threads=0):
    """Closed meshes of many stars at once.  Each request is a dict with keys
    S, num_cells, R_eq, zeta, epsilon, star_shape_ind; the outputs theta,
    phi, r, cellArea, maxAlpha, cos_gamma, effGrav are added to it."""
    n = len(requests)
    arr = (ClosedMeshRequest * n)()
    for i, q in enumerate(requests):
        S = int(q["S"])
        if S < 4 or S % 2 != 0:
            raise ValueError("S must be an even integer >= 4")
        q.update(theta=np.empty((S, S)), phi=np.empty((S, S)), r=np.empty(S),
                 cellArea=np.zeros(1), maxAlpha=np.empty(S), cos_gamma=np.empty(S),
                 effGrav=np.empty(S))
        arr[i] = ClosedMeshRequest(S, int(q["num_cells"]), float(q["R_eq"]), float(q["zeta"]),
                                   float(q["epsilon"]), int(q["star_shape_ind"]),
                                   q["theta"].ctypes.data, q["phi"].ctypes.data,
                                   q["r"].ctypes.data, q["cellArea"].ctypes.data,
                                   q["maxAlpha"].ctypes.data, q["cos_gamma"].ctypes.data,
                                   q["effGrav"].ctypes.data)
    check(lib().xgpu_closed_cell_mesh_many(n, arr, int(n_threads)))
    for q in requests:
        q["cellArea"] = float(q["cellArea"][0])
    return requests
