"""Build recipe for oracle/_ref/libteref.so (TEST INFRASTRUCTURE ONLY).

Compiles the reference's own, unmodified core/krylovTimeEvolver.cpp,
core/matrixDataTypes.cpp, core/krylovObservables.cpp and core/krylovLogger.cpp
where they lie in the reference tree, with ref_driver.cpp, against the
stand-in headers of ref_shim/ (CBLAS and LAPACKE by exported name from numpy's
ILP64 OpenBLAS; Boost.Math quadrature and Boost.Log replaced by the oracle's
own rules in te_quadrature.h and a std::clog logger), with -DUSE_OPENBLAS, so
that spMV, expV and mulV run the reference's own loops.

The reference tree is taken from $TE_REFERENCE_DIR, else /root/reference;
nothing is built when it or numpy's OpenBLAS is missing.  Output goes to
oracle/_ref/ only.  Usage: python oracle/ref_recipe.py [--force]
"""
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref", "libteref.so")
SOURCES = ["core/krylovTimeEvolver.cpp", "core/matrixDataTypes.cpp", "core/krylovObservables.cpp",
           "core/krylovLogger.cpp"]


def reference_dir():
    d = os.environ.get("TE_REFERENCE_DIR") or "/root/reference"
    return d if os.path.isfile(os.path.join(d, SOURCES[0])) else None


def openblas():
    """numpy's bundled ILP64 OpenBLAS (exports scipy_cblas_*64_, scipy_LAPACKE_*64_)."""
    import numpy
    base = os.path.dirname(os.path.dirname(numpy.__file__))
    hits = sorted(glob.glob(os.path.join(base, "numpy.libs", "libscipy_openblas64_*.so")))
    return hits[0] if hits else None


def build_ref(force=False, verbose=False):
    """Returns the library path, or None when it cannot be built here."""
    ref, blas = reference_dir(), openblas()
    if ref is None or blas is None:
        return None
    srcs = [os.path.join(ref, s) for s in SOURCES] + [os.path.join(HERE, "ref_driver.cpp")]
    deps = srcs + glob.glob(os.path.join(HERE, "ref_shim", "**", "*"), recursive=True) + \
        [os.path.join(HERE, "te_quadrature.h")]
    if not force and os.path.exists(OUT) and os.path.getmtime(OUT) >= max(os.path.getmtime(p) for p in deps
                                                                         if os.path.isfile(p)):
        return OUT
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-pthread", "-ffp-contract=off", "-DUSE_OPENBLAS",
           "-w", "-I", os.path.join(HERE, "ref_shim"), "-I", HERE, "-I", os.path.join(ref, "core"),
           "-o", OUT] + srcs + [blas, "-Wl,-rpath," + os.path.dirname(blas)]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    return OUT


if __name__ == "__main__":
    path = build_ref(force="--force" in sys.argv, verbose=True)
    print(path or "not built: reference tree or numpy's OpenBLAS not found")
