"""The reference's own example programs compile and link unchanged against the
drop-in C++ layer (timeevolver_gb300/host) and its libraries.

Reads the reference tree named by the environment variable TE_REFERENCE_DIR;
skipped where it is unset.  Running them needs a GPU; the runtime behaviour of the same API is
covered by test_cpp_dropin.py.
"""
import os
import subprocess

import pytest

REF_DIR = os.environ.get("TE_REFERENCE_DIR", "")
REF_EXAMPLES = os.path.join(REF_DIR, "example") if REF_DIR else ""
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HOST = os.path.join(ROOT, "timeevolver_gb300", "host")
INC = os.path.join(ROOT, "include")
BUILD = os.path.join(ROOT, "timeevolver_gb300", "_build")

pytestmark = pytest.mark.skipif(not REF_EXAMPLES or not os.path.isdir(REF_EXAMPLES),
                                reason="TE_REFERENCE_DIR not set (reference tree absent)")


def _cuda_include():
    nvcc = subprocess.run(["which", "nvcc"], capture_output=True, text=True).stdout.strip() or "/usr/local/cuda/bin/nvcc"
    return os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")


@pytest.fixture(scope="module")
def libs():
    import timeevolver_gb300 as te
    te.build()
    return BUILD


def _compile(src, out, extra_inc=()):
    cmd = ["g++", "-std=c++17", "-O1", "-c", src, "-I", HOST, "-I", INC, "-I", _cuda_include(), "-o", out]
    for d in extra_inc:
        cmd += ["-I", d]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


def test_simple_example_builds(libs, tmp_path):
    obj = str(tmp_path / "simpleExample.o")
    _compile(os.path.join(REF_EXAMPLES, "simpleExample.cpp"), obj)
    exe = str(tmp_path / "simpleExample")
    r = subprocess.run(["g++", "-o", exe, obj, "-L", libs, "-ltimeevolver", "-ltegpu", "-Wl,-rpath," + libs],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    assert os.path.exists(exe)


def test_black_hole_model_compiles(libs, tmp_path):
    # the black-hole model of the reference's CLI example, written against Basis.h / hamiltonian.h
    _compile(os.path.join(REF_EXAMPLES, "exampleHamiltonian.cpp"), str(tmp_path / "exampleHamiltonian.o"),
             extra_inc=(REF_EXAMPLES,))
