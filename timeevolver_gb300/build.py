"""Build the native parts of timeevolver_gb300 in-tree (no cmake).

* ``_build/libtegpu.so``: the CUDA kernels and the C ABI of include/tegpu.h,
  compiled by nvcc for sm_103a only (one translation unit per file, compiled
  in parallel, then linked).
* ``_build/libtimeevolver.so``: the C++ drop-in layer (krylovTimeEvolver,
  smatrix, observables, basis, Hamiltonian), compiled by g++ against
  libtegpu.so.
"""
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
CSRC = os.path.join(HERE, "csrc")
HOST = os.path.join(HERE, "host")
LIB_TEGPU = os.path.join(BUILD, "libtegpu.so")
LIB_HOST = os.path.join(BUILD, "libtimeevolver.so")

CUDA_SOURCES = ["te_common.cu", "te_matrix.cu", "te_lanczos.cu", "te_krylov.cu", "te_sample.cu", "te_evolver.cu",
                "te_batch.cu", "te_adjoint.cu", "te_synth.cu", "te_model.cu", "te_probe.cu",
                "te_fixed.cu"]
NVCC_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-std=c++17",
              "-Xcompiler", "-fPIC"]
HOST_SOURCES = ["matrixDataTypes.cpp", "krylovObservables.cpp", "krylovTimeEvolver.cpp", "krylovLogger.cpp",
                "krylovHelper.cpp", "h5min.cpp",
                "Basis.cpp", "hamiltonian.cpp", "te_host_c.cpp"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off"]
# te_krylov.cu holds the persistent batched kernel, which rereads data that its
# own blocks rewrite between grid barriers (instance states, schedule, active
# list): global loads without an explicit cache operator bypass L1 there.  It
# is compiled without implicit multiply-add contraction, so that the Krylov
# step body, inlined into three kernels (single evolution, batched block per
# instance, persistent batch), rounds the same way in each.
NVCC_FILE_FLAGS = {"te_krylov.cu": ["-Xptxas", "-dlcm=cg", "-fmad=false"]}


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libtegpu")


def _cuda_lib_dir():
    base = os.path.dirname(os.path.dirname(os.path.realpath(_nvcc())))
    for sub in ("lib64", "lib", "targets/sbsa-linux/lib", "targets/x86_64-linux/lib"):
        d = os.path.join(base, sub)
        if os.path.exists(os.path.join(d, "libcudart.so")):
            return d
    return os.path.join(base, "lib64")


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def _run(cmd):
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), p.stdout, p.stderr))
    return p.stdout + p.stderr


def build_tegpu(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")]
    headers += [os.path.join(ROOT, "include", h) for h in ("tegpu.h", "te_diag.h")]
    srcs = [os.path.join(CSRC, f) for f in CUDA_SOURCES]
    if not force and not _stale(LIB_TEGPU, srcs + headers):
        return LIB_TEGPU
    nvcc = _nvcc()

    def one(src):
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        if force or _stale(obj, [src] + headers):
            extra = os.environ.get("TE_NVCC_FLAGS", "").split()  # e.g. -DTE_NO_PDL
            per_file = NVCC_FILE_FLAGS.get(os.path.basename(src), [])
            out = _run([nvcc] + NVCC_FLAGS + per_file + extra + (["-Xptxas", "-v"] if verbose else []) +
                       ["-c", src, "-o", obj])
            if verbose:
                print(out)
        return obj

    with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(one, srcs))
    _run([nvcc, "-shared", "-o", LIB_TEGPU] + objs + ["-Xcompiler", "-fPIC"])
    return LIB_TEGPU


def build_host(force=False):
    """The C++ drop-in layer (reference class API) over libtegpu."""
    srcs = [os.path.join(HOST, f) for f in HOST_SOURCES]
    headers = [os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".h")]
    headers.append(os.path.join(ROOT, "include", "tegpu.h"))
    if not force and not _stale(LIB_HOST, srcs + headers + [LIB_TEGPU]):
        return LIB_HOST
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(_nvcc()))), "include")

    def one(src):
        obj = os.path.join(BUILD, "host_" + os.path.basename(src)[:-4] + ".o")
        if force or _stale(obj, [src] + headers):
            _run(["g++"] + CXX_FLAGS + ["-I", HOST, "-I", os.path.join(ROOT, "include"), "-I", cuda_inc,
                                        "-c", src, "-o", obj])
        return obj

    with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(one, srcs))
    _run(["g++", "-shared", "-o", LIB_HOST] + objs + ["-L", BUILD, "-ltegpu", "-Wl,-rpath,$ORIGIN"])
    return LIB_HOST


def build_all(force=False, verbose=False):
    build_tegpu(force=force, verbose=verbose)
    if os.path.isdir(HOST):
        build_host(force=force)
    return LIB_TEGPU


if __name__ == "__main__":
    import sys
    build_all(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print("built", LIB_TEGPU)
