"""The C++ drop-in API: a program written against the reference's classes
compiles against timeevolver_gb300/host (CPU) and reproduces the reference's
goldens on the GPU."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")
BUILD = os.path.join(ROOT, "timeevolver_gb300", "_build")
EXE = os.path.join(BUILD, "dropin_driver")


def _compile():
    import timeevolver_gb300 as te
    te.build()
    src = os.path.join(ROOT, "tests", "cpp", "dropin_driver.cpp")
    if os.path.exists(EXE) and os.path.getmtime(EXE) > max(os.path.getmtime(src), os.path.getmtime(te.LIB_PATH)):
        return EXE
    subprocess.check_call(["g++", "-std=c++17", "-O2", src, "-I", os.path.join(ROOT, "timeevolver_gb300", "host"),
                           "-I", os.path.join(ROOT, "include"), "-I", "/usr/local/cuda/include", "-L", BUILD,
                           "-ltimeevolver", "-ltegpu", "-Wl,-rpath," + BUILD, "-o", EXE])
    return EXE


def _run(*args):
    out = subprocess.run([_compile()] + list(args), capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    rows, res = [], None
    for line in out.stdout.splitlines():
        if line.startswith("RESULT"):
            res = dict(kv.split("=") for kv in line.split()[1:])
        else:
            rows.append([float(x) for x in line.split()[1:]])
    return np.array(rows), res


def test_dropin_compiles():
    assert os.path.exists(_compile())


@pytest.mark.gpu
def test_dropin_black_hole_golden():
    samples, res = _run("blackhole", "20", "2", "4", "10", "0.01")
    gold = np.load(os.path.join(GOLD, "blackhole_N20.npy"))
    assert samples.shape == gold.shape
    assert np.max(np.abs(samples - gold)) < 1e-8
    assert int(res["samples"]) == 1001 and float(res["err"]) <= 1e-8


@pytest.mark.gpu
def test_dropin_lucky_breakdown_golden():
    samples, res = _run("blackhole", "1", "1", "1", "1000", "1")
    gold = np.load(os.path.join(GOLD, "blackhole_N1_LB.npy"))
    assert np.max(np.abs(samples - gold)) < 1e-8
    assert int(res["status"]) == 1 and int(res["krylov"]) == 4


@pytest.mark.gpu
def test_dropin_simple_example_golden():
    samples, res = _run("simple")
    gold = np.load(os.path.join(GOLD, "simple_example.npy"))
    assert np.max(np.abs(samples - gold)) <= 6e-4


def test_save_result_csv(tmp_path):
    """saveResult (the reference's CSV branch): file name from the flagged
    parameters, samples joined by ', ' in the default stream format."""
    src = tmp_path / "save.cpp"
    src.write_text(r'''
#include "krylovHelper.h"
int main(int, char** argv) {
  std::vector<std::unique_ptr<krylovBasicObservable>> obs;
  obs.push_back(std::make_unique<krylovOutputObservable>("n0", std::vector<double>{1.0, 0.123456789, 2.5e-7, -3.0}));
  obs.push_back(std::make_unique<krylovOutputObservable>("n1", std::vector<double>{100.125, 1e20}));
  parameter_list para;
  para.push_back(paraPush("N", true, 20));
  para.push_back(paraPush("tol", false, 1e-8));
  para.push_back(paraPush("dt", true, 0.1));
  saveResult(obs, para, std::string(argv[1]) + "/Result");
  return 0;
}
''')
    import timeevolver_gb300 as te
    te.build()
    exe = str(tmp_path / "save")
    subprocess.check_call(["g++", "-std=c++17", "-O1", str(src), "-I", os.path.join(ROOT, "timeevolver_gb300", "host"),
                           "-I", os.path.join(ROOT, "include"), "-I", "/usr/local/cuda/include", "-L", BUILD,
                           "-ltimeevolver", "-ltegpu", "-Wl,-rpath," + BUILD, "-o", exe])
    subprocess.check_call([exe, str(tmp_path)])
    assert (tmp_path / "Result_N20_dt0.1n0.csv").read_text() == "1, 0.123457, 2.5e-07, -3"
    assert (tmp_path / "Result_N20_dt0.1n1.csv").read_text() == "100.125, 1e+20"


@pytest.mark.gpu
def test_dropin_simple_example_csv_matches_golden_text(tmp_path):
    """The reference's simple example written through saveResult reproduces the
    text of its golden CSV output (values at the default 6 digits)."""
    _run("simple", str(tmp_path / "SimpleExampleOutputOccupationNumber"))
    gold = np.load(os.path.join(GOLD, "simple_example.npy"))
    for k in range(2):
        text = (tmp_path / ("SimpleExampleOutputOccupationNumber%d.csv" % k)).read_text()
        expected = ", ".join("%g" % x for x in gold[k])
        assert text == expected
