"""Build and load the in-tree CUDA library (libxpsi_gb300.so) and bind the
C ABI declared in include/xpsi_gb300.h with ctypes.

The library is compiled for sm_103a only.  Every compute entry point of this
package goes through it; when it cannot be loaded (no CUDA device, build
missing) calls fail loudly -- there is no CPU fallback.
"""
import ctypes as C
import os
import subprocess
import threading
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libxpsi_gb300.so")
UNITS = ["rays", "integrator", "energy", "fold", "fold_tc", "likelihood", "abi", "mesh",
         "mesh_gpu", "elsewhere", "general", "synth"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
              "--expt-relaxed-constexpr", "-diag-suppress", "177"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _sources_mtime():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)
             if f.endswith((".cu", ".cuh", ".h", ".cpp"))]
    files.append(os.path.join(ROOT, "include", "xpsi_gb300.h"))
    return max(os.path.getmtime(f) for f in files)


def build(force=False, verbose=False):
    """Compile every CUDA unit for sm_103a (in parallel) and link the library."""
    os.makedirs(BUILD, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _sources_mtime():
        return LIB
    nvcc = _nvcc()

    def compile_unit(u):
        obj = os.path.join(BUILD, u + ".o")
        src = os.path.join(CSRC, u + ".cu")
        if os.path.exists(src):
            cmd = [nvcc, *ARCH, *NVCC_FLAGS, "-c", src, "-o", obj]
        else:  # host C++ unit
            cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-c",
                   os.path.join(CSRC, u + ".cpp"), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s%s" % (u, r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)
        return obj

    with ThreadPoolExecutor(len(UNITS)) as ex:
        objs = list(ex.map(compile_unit, UNITS))
    tmp = LIB + ".tmp%d" % os.getpid()
    r = subprocess.run([nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart", "-lpthread"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, LIB)
    return LIB


_lock = threading.Lock()
_lib = None

P = C.c_void_p
D = C.c_double
SZ = C.c_size_t
I32 = C.c_int32
I64 = C.c_int64


class Atmos4D(C.Structure):
    _fields_ = [("logT", P), ("logg", P), ("mu", P), ("logE", P), ("intensity", P),
                ("nT", SZ), ("ng", SZ), ("nmu", SZ), ("nE", SZ), ("intensity_f32", P)]


class Atmos5D(C.Structure):
    """xgpu_atmos5d: a split atmosphere's 5 grids and intensity table."""
    _fields_ = [("grid", P * 5), ("n", SZ * 5), ("intensity", P)]


class Mesh(C.Structure):
    _fields_ = [("S0", I32), ("S1", I32), ("row_off", I64), ("cell_off", I64),
                ("omega", D), ("inclination", D), ("image_order_limit", I32),
                ("atm_ext", I32), ("flux_off", I64), ("beam_opt", I32), ("reserved", I32)]


class IntegrateBatchData(C.Structure):
    _fields_ = [("row_mesh", P), ("radius", P), ("u", P), ("cos_gamma", P),
                ("theta0", P), ("maxDeflection", P), ("deflection", P),
                ("cos_alpha", P), ("lag", P), ("cellArea", P), ("phi", P),
                ("params", P), ("n_params", I32), ("radiates", P), ("energies", P),
                ("leaves", P), ("phases", P), ("atmos", Atmos4D), ("flux", P),
                ("mesh_status", P), ("flop_counter", P), ("correction", P),
                ("n_correction", I32)]


class MeshRequest(C.Structure):
    _fields_ = [("polar", I32), ("num_cells", SZ), ("S", SZ), ("R_eq", D), ("zeta", D),
                ("epsilon", D), ("star_shape_ind", I32), ("cede_radius", D),
                ("cede_colatitude", D), ("super_radius", D), ("super_colatitude", D),
                ("super_azimuth", D), ("theta", P), ("phi", P), ("r", P), ("area", P),
                ("maxAlpha", P), ("cos_gamma", P), ("effGrav", P)]


class AllocRequest(C.Structure):
    _fields_ = [("num_cells", SZ), ("min_sqrt", SZ), ("max_sqrt", SZ), ("R_eq", D),
                ("Omega", D), ("zeta", D), ("epsilon", D), ("star_shape_ind", I32),
                ("super_radius", D), ("cede_radius", D), ("super_colatitude", D),
                ("cede_colatitude", D), ("super_azimuth", D), ("hole_colatitude", D),
                ("hole_radius", D), ("hole_azimuth", D), ("out", D * 4)]


class MeshMember(C.Structure):
    _fields_ = [("polar", I32), ("num_cells", SZ), ("S", SZ), ("R_eq", D), ("zeta", D),
                ("epsilon", D), ("star_shape_ind", I32), ("cede_radius", D),
                ("cede_colatitude", D), ("super_radius", D), ("super_colatitude", D),
                ("super_azimuth", D), ("row_off", I64), ("cell_off", I64), ("r_s", D),
                ("lag_scale", D), ("omit_azimuth", D), ("logT", D), ("antiphased", I32)]


class MeshBatchOut(C.Structure):
    _fields_ = [("u", P), ("r_s", P), ("maxAlpha", P), ("radius", P), ("cos_gamma", P),
                ("theta0", P), ("lag_C", P), ("lag_scale", P), ("row_mesh", P),
                ("cellArea", P), ("phi", P), ("params", P), ("radiates", P)]


class ClosedMeshRequest(C.Structure):
    _fields_ = [("S", SZ), ("num_cells", SZ), ("R_eq", D), ("zeta", D), ("epsilon", D),
                ("star_shape_ind", I32), ("theta", P), ("phi", P), ("r", P),
                ("cellArea", P), ("maxAlpha", P), ("cos_gamma", P), ("effGrav", P)]


class ElsewhereMesh(C.Structure):
    _fields_ = [("S", I32), ("row_off", I32), ("cell_off", I64), ("omega", D),
                ("inclination", D), ("cellArea", D), ("image_order_limit", I32),
                ("atm_ext", I32)]


class ElsewhereBatchData(C.Structure):
    _fields_ = [("row_mesh", P), ("radius", P), ("u", P), ("cos_gamma", P),
                ("theta0", P), ("maxDeflection", P), ("deflection", P), ("cos_alpha", P),
                ("phi", P), ("params", P), ("n_params", I32), ("energies", P),
                ("atmos", Atmos4D), ("flux", P), ("mesh_status", P), ("signal", P),
                ("signal_stride", I64), ("signal_N_P", I32)]


class Component(C.Structure):
    _fields_ = [("signal", P), ("phases", P), ("ld", I64), ("n", I32), ("shift", D)]


class LikelihoodBatchData(C.Structure):
    _fields_ = [("n_vec", I32), ("K", I32), ("B", I32), ("H", I32), ("N_P", I32),
                ("exposure", D), ("epsabs", D), ("epsrel", D), ("epsilon", D),
                ("sigmas", D), ("llzero", D), ("slim", D),
                ("phase_edges", P), ("comp_phases", P), ("counts", P), ("precomp", P),
                ("support", P), ("background", P), ("signals", P), ("shifts", P),
                ("allow_negative", P), ("chan_ll", P), ("chan_flag", P), ("star", P),
                ("mcl_bg", P), ("mcl_bg_support", P), ("loglike", P), ("status", P)]


def _bind(L):
    sig = {
        "xgpu_abi_version": (C.c_int, []),
        "xgpu_last_error": (C.c_char_p, []),
        "xgpu_atmos_cache_invalidate": (C.c_int, []),
        "xgpu_compute_rays": (C.c_int, [SZ, D, P, P, SZ, P, P, P, P]),
        "xgpu_integrate": (C.c_int, [D, D, D, D, SZ, SZ, P, P, P, P, P, P, SZ, P, P, SZ, SZ,
                                     P, P, P, P, P, SZ, P, SZ, P, SZ, P, C.c_int,
                                     C.POINTER(Atmos4D), C.c_int, C.c_int, C.c_int, P]),
        "xgpu_integrate_split": (C.c_int, [D, D, D, D, SZ, SZ, P, P, P, P, P, P, SZ, P, P, SZ,
                                           SZ, P, P, P, P, P, SZ, P, SZ, P, SZ, P,
                                           C.POINTER(Atmos5D), C.c_int, C.c_int, P]),
        "xgpu_energy_integrator": (C.c_int, [SZ, SZ, P, P, SZ, P, P]),
        "xgpu_response_fold": (C.c_int, [SZ, SZ, SZ, P, SZ, P, P]),
        "xgpu_precomputation": (C.c_int, [SZ, SZ, P, P]),
        "xgpu_eval_marginal_likelihood": (C.c_int, [D, SZ, P, SZ, P, SZ, P, P, P, P, P,
                                                    P, D, D, D, D, D, P, D, P, P, P, P,
                                                    P]),
        "xgpu_rays_batch": (C.c_int, [I64, C.c_int, P, P, P, P, P, P, P, P, P, P, P]),
        "xgpu_integrate_batch": (C.c_int, [C.c_int, C.POINTER(Mesh), I64, C.c_int,
                                           C.c_int, C.c_int, C.c_int,
                                           C.POINTER(IntegrateBatchData), C.c_int, P]),
        "xgpu_integrate_batch_mixed": (C.c_int, [C.c_int, C.POINTER(Mesh), I64, C.c_int,
                                                 C.c_int, C.c_int, C.c_int,
                                                 C.POINTER(IntegrateBatchData), C.c_int, P]),
        "xgpu_energy_batch": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, P, P, P, P,
                                        P, P, P, C.c_int, P]),
        "xgpu_fold_batch": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, P, C.c_int, P,
                                      P, P]),
        "xgpu_fold_batch_tc": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, P, C.c_int, P,
                                         P, P, P]),
        "xgpu_fold_tc_timeout_selftest": (C.c_int, [P]),
        "xgpu_likelihood_batch": (C.c_int, [C.POINTER(LikelihoodBatchData), P]),
        "xgpu_likelihood_batch_static": (C.c_int, [C.POINTER(LikelihoodBatchData), P]),
        "xgpu_allocate_cells": (C.c_int, [SZ, SZ, SZ, D, D, D, D, C.c_int, D, D, D, D, D, D,
                                          D, D, P]),
        "xgpu_cell_mesh": (C.c_int, [C.c_int, SZ, SZ, D, D, D, C.c_int, D, D, D, D, D, P, P,
                                     P, P, P, P, P]),
        "xgpu_cell_mesh_many": (C.c_int, [C.c_int, C.POINTER(MeshRequest), C.c_int]),
        "xgpu_allocate_cells_many": (C.c_int, [C.c_int, C.POINTER(AllocRequest), C.c_int]),
        "xgpu_mesh_batch": (C.c_int, [C.c_int, C.POINTER(MeshMember), I64, I64,
                                      C.POINTER(MeshBatchOut), P]),
        "xgpu_peak_probe": (C.c_double, [C.c_int, C.c_int, C.c_int, C.c_int, P, P]),
        "xgpu_gaussian_loglike": (C.c_int, [SZ, SZ, P, SZ, P, P, P]),
        "xgpu_gaussian_loglike_batch": (C.c_int, [C.c_int, C.c_int, C.c_int, P, I64, I64, P, P,
                                                  P, P]),
        "xgpu_integrate_stokes": (C.c_int, [D, D, D, D, SZ, SZ, P, P, P, P, P, P, SZ, P, P, SZ,
                                            SZ, P, P, P, P, P, SZ, P, SZ, P, SZ, P, C.c_int,
                                            C.POINTER(Atmos4D), C.POINTER(Atmos4D), C.c_int,
                                            C.c_int, P, P, P]),
        "xgpu_integrate_general_stokes": (C.c_int, [D, D, D, D, SZ, SZ, P, P, P, P, P, P, SZ,
                                                    P, P, SZ, SZ, P, P, P, P, P, SZ, P, SZ, P,
                                                    SZ, P, C.c_int, C.POINTER(Atmos4D),
                                                    C.POINTER(Atmos4D), C.c_int, C.c_int, P, P,
                                                    P]),
        "xgpu_phase_interpolator": (C.c_int, [SZ, P, SZ, P, SZ, P, D, C.c_int, P]),
        "xgpu_energy_interpolator": (C.c_int, [SZ, SZ, P, P, SZ, P, P]),
        "xgpu_integrate_split_stokes": (C.c_int, [D, D, D, D, SZ, SZ, P, P, P, P, P, P, SZ, P,
                                                  P, SZ, SZ, P, P, P, P, P, SZ, P, SZ, P, SZ,
                                                  P, C.POINTER(Atmos5D), C.POINTER(Atmos5D),
                                                  C.c_int, C.c_int, P, P, P]),
        "xgpu_integrate_general": (C.c_int, [D, D, D, D, SZ, SZ, P, P, P, P, P, P, SZ, P, P,
                                             SZ, SZ, P, P, P, P, P, SZ, P, SZ, P, SZ, P,
                                             C.c_int, C.POINTER(Atmos4D), C.c_int, C.c_int,
                                             P]),
        "xgpu_compute_expected_counts": (C.c_int, [D, SZ, P, SZ, SZ, C.POINTER(Component), P, P,
                                                   P]),
        "xgpu_phase_integrator": (C.c_int, [D, SZ, P, SZ, SZ, P, P, D, C.c_int, P]),
        "xgpu_poisson": (C.c_int, [SZ, P, C.c_uint64, C.c_uint64, P]),
        "xgpu_expected_counts_batch": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, D, P,
                                                 C.POINTER(Component), P, P, P, P]),
        "xgpu_poisson_batch": (C.c_int, [I64, P, P, C.c_uint64, C.c_uint64, P, P]),
        "xgpu_poisson_loglike_batch": (C.c_int, [C.c_int, C.c_int, C.c_int, P, P, P, P, P, P]),
        "xgpu_poisson_likelihood_given_background": (C.c_int, [D, SZ, P, SZ, P, SZ,
                                                               C.POINTER(Component), P, P, P, P,
                                                               P, P]),
        "xgpu_closed_cell_mesh": (C.c_int, [SZ, SZ, D, D, D, C.c_int, P, P, P, P, P, P, P]),
        "xgpu_closed_cell_mesh_many": (C.c_int, [C.c_int, C.POINTER(ClosedMeshRequest),
                                                 C.c_int]),
        "xgpu_integrate_time_invariant": (C.c_int, [D, D, D, D, SZ, D, P, P, P, P, P, SZ, SZ,
                                                    P, P, P, P, SZ, P, C.c_int,
                                                    C.POINTER(Atmos4D), C.c_int, P]),
        "xgpu_elsewhere_batch": (C.c_int, [C.c_int, C.POINTER(ElsewhereMesh), I64, C.c_int,
                                           C.c_int, C.c_int, C.POINTER(ElsewhereBatchData),
                                           P]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    return L


EXPORTED = ["xgpu_abi_version", "xgpu_last_error", "xgpu_compute_rays", "xgpu_integrate",
            "xgpu_energy_integrator", "xgpu_response_fold", "xgpu_precomputation",
            "xgpu_eval_marginal_likelihood", "xgpu_rays_batch", "xgpu_integrate_batch",
            "xgpu_energy_batch", "xgpu_fold_batch", "xgpu_likelihood_batch",
            "xgpu_allocate_cells", "xgpu_cell_mesh", "xgpu_cell_mesh_many", "xgpu_peak_probe",
            "xgpu_likelihood_batch_static", "xgpu_integrate_batch_mixed",
            "xgpu_fold_batch_tc", "xgpu_mesh_batch", "xgpu_allocate_cells_many",
            "xgpu_closed_cell_mesh", "xgpu_closed_cell_mesh_many",
            "xgpu_integrate_time_invariant", "xgpu_elsewhere_batch",
            "xgpu_integrate_general", "xgpu_compute_expected_counts",
            "xgpu_phase_integrator", "xgpu_poisson", "xgpu_expected_counts_batch",
            "xgpu_poisson_batch", "xgpu_integrate_stokes", "xgpu_gaussian_loglike",
            "xgpu_gaussian_loglike_batch", "xgpu_integrate_split",
            "xgpu_integrate_split_stokes", "xgpu_integrate_general_stokes",
            "xgpu_phase_interpolator", "xgpu_energy_interpolator",
            "xgpu_atmos_cache_invalidate", "xgpu_poisson_loglike_batch",
            "xgpu_poisson_likelihood_given_background", "xgpu_fold_tc_timeout_selftest"]


ABI_VERSION = 4  # XGPU_ABI_VERSION of include/xpsi_gb300.h


def lib():
    """The loaded C ABI (built on first use if the sources are newer)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB) or os.path.getmtime(LIB) < _sources_mtime():
                build()
            L = _bind(C.CDLL(LIB))
            if L.xgpu_abi_version() != ABI_VERSION:
                raise RuntimeError("%s has C ABI version %d, these bindings expect %d: rebuild "
                                   "with xpsi_gb300.build(force=True)"
                                   % (LIB, L.xgpu_abi_version(), ABI_VERSION))
            _lib = L
    return _lib


class GPUError(RuntimeError):
    """A CUDA or usage failure reported by the C ABI."""


def check(rc):
    """Raise GPUError for negative return codes; pass statuses through."""
    if rc < 0:
        msg = lib().xgpu_last_error().decode(errors="replace")
        raise GPUError(msg or ("C ABI call failed with %d" % rc))
    return rc
