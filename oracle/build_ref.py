"""Build recipe for the reference's own likelihood-path extension modules.

TEST INFRASTRUCTURE.  Compiles X-PSI's Cython sources where they lie (under
the read-only reference checkout, never copied) against the oracle's GSL-API
subset (oracle/gslsub), with outputs only under oracle/_ref/.  The result is
importable through oracle/ref_harness.py and is used to pin the oracle's
C restatement and to generate tests/golden fixtures.  It runs in a container
that holds the reference checkout; the GPU host never runs it.

Flags follow the reference's setup.py (-O3 -fopenmp) with FMA contraction
switched off (-ffp-contract=off) so results do not depend on the host ISA.

Usage:  python oracle/build_ref.py --ref <reference checkout> [-j N]
        (or the checkout in $XPSI_REFERENCE)
"""
import argparse
import os
import subprocess
import sys
import sysconfig
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")

# module closure of the likelihood path (cimport graph of the hot modules)
MODULES = [
    "tools.core", "tools.phase_integrator", "tools.phase_interpolator",
    "tools.energy_integrator", "tools.energy_interpolator",
    "tools.compute_expected_counts", "tools.synthesise",
    "surface_radiation_field.preload",
    "surface_radiation_field.effective_gravity_universal",
    "surface_radiation_field.hot_BB", "surface_radiation_field.hot_Num4D",
    "surface_radiation_field.hot_BB_burst", "surface_radiation_field.hot_Num2D",
    "surface_radiation_field.hot_user", "surface_radiation_field.hot_Num5D_split",
    "surface_radiation_field.elsewhere_user",
    "surface_radiation_field.hot_wrapper",
    "surface_radiation_field.elsewhere_wrapper",
    "cellmesh.common_functions", "cellmesh.mesh_tools", "cellmesh.mesh",
    "cellmesh.polar_mesh", "cellmesh.rays", "cellmesh.integrator",
    "cellmesh.integrator_for_azimuthal_invariance",
    "cellmesh.global_mesh", "cellmesh.integrator_for_time_invariance",
    "cellmesh.integratorIQU_for_azimuthal_invariance",
    "surface_radiation_field.hot_Num2D_split",
    "cellmesh.integrator_for_azimuthal_invariance_split",
    "cellmesh.integratorIQU_for_azimuthal_invariance_split",
    "cellmesh.integratorIQU",
    "likelihoods.default_background_marginalisation",
    "likelihoods._poisson_likelihood_given_background",
    "likelihoods._gaussian_likelihood_QnUn",
    "likelihoods._gaussian_likelihood_given_background_IQU",
]


def run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(" ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("XPSI_REFERENCE"),
                    help="the reference checkout (default: $XPSI_REFERENCE)")
    ap.add_argument("-j", type=int, default=os.cpu_count() or 4)
    args = ap.parse_args()
    if not args.ref:
        ap.error("give the reference checkout with --ref or $XPSI_REFERENCE")
    ref = os.path.abspath(args.ref)
    if not os.path.isdir(os.path.join(ref, "xpsi")):
        print("reference checkout not found; nothing to build")
        return 0
    # the import harness finds the checkout these modules were built from
    os.makedirs(OUT, exist_ok=True)
    with open(os.path.join(OUT, "REFERENCE_PATH"), "w") as f:
        f.write(ref + "\n")
    import numpy
    build = os.path.join(OUT, "build")
    os.makedirs(build, exist_ok=True)
    gsl_inc = os.path.join(HERE, "gslsub", "include")
    gsl_obj = os.path.join(build, "gslsub.o")
    run(["gcc", "-O2", "-fPIC", "-ffp-contract=off", "-I", gsl_inc, "-c",
         os.path.join(HERE, "gslsub", "gslsub.c"), "-o", gsl_obj])
    suffix = sysconfig.get_config_var("EXT_SUFFIX")
    py_inc = sysconfig.get_paths()["include"]

    def one(mod):
        sub, name = mod.split(".")
        src = os.path.join(ref, "xpsi", sub, name + ".pyx")
        c_out = os.path.join(build, f"xpsi.{mod}.c")
        dst_dir = os.path.join(OUT, "xpsi", sub)
        os.makedirs(dst_dir, exist_ok=True)
        so = os.path.join(dst_dir, name + suffix)
        lang = "c"
        with open(src) as fh:
            if "libcpp" in fh.read():
                lang = "c++"
        if lang == "c++":
            c_out = c_out[:-2] + ".cpp"
        run([sys.executable, "-m", "cython", "-3", "--fast-fail",
             "-I", os.path.join(ref, "xpsi", "include"), "-I", ref,
             *(["--cplus"] if lang == "c++" else []),
             src, "-o", c_out])
        cc = "g++" if lang == "c++" else "gcc"
        run([cc, "-shared", "-fPIC", "-O3", "-fopenmp", "-ffp-contract=off",
             "-w", "-I", py_inc, "-I", numpy.get_include(), "-I", gsl_inc,
             "-DNPY_NO_DEPRECATED_API=NPY_1_7_API_VERSION",
             c_out, gsl_obj, "-o", so, "-lm"])
        return mod

    with ThreadPoolExecutor(args.j) as ex:
        for m in ex.map(one, MODULES):
            print("built", m)
    return 0


if __name__ == "__main__":
    sys.exit(main())
