"""The HDF5 branch of saveResult and saveSparseMatrix (helper/krylovHelper.cpp:
27-92, 112-155), written by the library's own writer (host/h5min.cpp).

The reader (tests/hdf5_min.py) is pinned on the reference's golden HDF5 files:
tests/golden/h5_manifest.json records what it finds there (made by
tests/golden/make_h5_manifest.py; re-checked here when TE_REFERENCE_DIR names
the reference tree).  A program written against the reference's API, compiled
with USE_HDF, then saves the golden trajectories with the golden parameter
list, and the file must hold the same datasets (names, order, shape, float64
little endian, values bit for bit), the same attributes (names, order, types,
values) and the same kinds of header messages as the golden files.
"""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
BUILD = os.path.join(ROOT, "timeevolver_gb300", "_build")
sys.path.insert(0, HERE)
import hdf5_min  # noqa: E402

REF_DIR = os.environ.get("TE_REFERENCE_DIR", "")
N20 = "ResultBlackHole_N20_Nm2_K4_C1_DeltaN12_C01_Cm1_maxT10_tol1e-08_samplingStep0.01_m40_fastIntegration0.h5"
N1 = "ResultBlackHole_N1_Nm1_K1_C1_DeltaN12_C01_Cm1_maxT1000_tol1e-08_samplingStep1_m40_fastIntegration0.h5"

SAVE_SRC = r'''
#include <cstdio>
#include <fstream>
#include "krylovHelper.h"
// argv: out_name samples.bin n_obs n_samples  then the golden parameter values
int main(int argc, char** argv) {
  const int n_obs = atoi(argv[3]), n_s = atoi(argv[4]);
  std::vector<double> buf((size_t)n_obs * n_s);
  std::ifstream in(argv[2], std::ios::binary);
  in.read(reinterpret_cast<char*>(buf.data()), buf.size() * 8);
  std::vector<std::unique_ptr<krylovBasicObservable>> obs;
  for (int k = 0; k < n_obs; ++k)
    obs.push_back(std::make_unique<krylovOutputObservable>(
        "mode" + std::to_string(k), std::vector<double>(buf.begin() + (size_t)k * n_s, buf.begin() + (size_t)(k + 1) * n_s)));
  parameter_list para;
  para.push_back(paraPush("DeltaN", false, atof(argv[5])));
  para.push_back(paraPush("C0", false, atof(argv[6])));
  para.push_back(paraPush("Cm", false, atof(argv[7])));
  para.push_back(paraPush("MaxT", false, atof(argv[8])));
  para.push_back(paraPush("Tolerance", false, atof(argv[9])));
  para.push_back(paraPush("SamplingStep", false, atof(argv[10])));
  para.push_back(paraPush("N0", false, atoi(argv[11])));
  para.push_back(paraPush("Nm", false, atoi(argv[12])));
  para.push_back(paraPush("K", false, atoi(argv[13])));
  para.push_back(paraPush("Capacity", false, atoi(argv[14])));
  para.push_back(paraPush("m", false, atoi(argv[15])));
  para.push_back(paraPush("fastIntegration", false, false));
  saveResult(obs, para, argv[1]);
  return 0;
}
'''

FLAGGED_SRC = r'''
#include "krylovHelper.h"
int main(int, char** argv) {
  std::vector<std::unique_ptr<krylovBasicObservable>> obs;
  for (int k = 0; k < 20; ++k)
    obs.push_back(std::make_unique<krylovOutputObservable>("obs" + std::to_string(k), std::vector<double>{k + 0.5, -1.0 * k}));
  parameter_list para;
  para.push_back(paraPush("N", true, 20));
  para.push_back(paraPush("tol", false, 1e-8));
  para.push_back(paraPush("dt", true, 0.1));
  para.push_back(paraPush("fast", true, true));
  saveResult(obs, para, std::string(argv[1]) + "/Result");
  std::vector<std::complex<double>> v = {{1.0, -2.0}, {0.25, 0.0}, {-3.0, 4.5}};
  std::vector<size_t> r = {0, 1, 2}, c = {2, 0, 1};
  smatrix M(v.data(), c.data(), r.data(), 3, 3, 3);
  saveSparseMatrix(&M, std::string(argv[1]) + "/sparse.h5");
  return 0;
}
'''


def _compile(tmp_path, src_text, name):
    import timeevolver_gb300 as te
    te.build()
    src = tmp_path / (name + ".cpp")
    src.write_text(src_text)
    exe = str(tmp_path / name)
    subprocess.check_call(["g++", "-std=c++17", "-O1", "-DUSE_HDF", str(src), "-I",
                           os.path.join(ROOT, "timeevolver_gb300", "host"), "-I", os.path.join(ROOT, "include"),
                           "-I", "/usr/local/cuda/include", "-L", BUILD, "-ltimeevolver", "-ltegpu",
                           "-Wl,-rpath," + BUILD, "-o", exe])
    return exe


def _manifest():
    with open(os.path.join(GOLD, "h5_manifest.json")) as fh:
        return json.load(fh)


@pytest.mark.skipif(not REF_DIR, reason="TE_REFERENCE_DIR not set (reference tree absent)")
def test_reader_on_reference_goldens():
    """The reader finds in the golden files what the manifest records, and
    the same trajectories the .npy fixtures hold (extracted at fixed offsets)."""
    sys.path.insert(0, GOLD)
    import make_h5_manifest
    man = _manifest()
    for f in (N20, N1):
        assert make_h5_manifest.describe(os.path.join(REF_DIR, "output", f)) == man[f]
    d = hdf5_min.read(os.path.join(REF_DIR, "output", N1))
    gold = np.load(os.path.join(GOLD, "blackhole_N1_LB.npy"))
    for k in range(4):
        assert np.array_equal(d["mode%d" % k][0], gold[k])


def test_reader_rejects_damaged_files(tmp_path):
    exe = _compile(tmp_path, FLAGGED_SRC, "flagged")
    subprocess.check_call([exe, str(tmp_path)])
    good = (tmp_path / "Result_N20_dt0.1_fast1.h5").read_bytes()
    hdf5_min.read(str(tmp_path / "Result_N20_dt0.1_fast1.h5"))
    for damage in (lambda b: b[:-8],                       # truncated: end-of-file address disagrees
                   lambda b: b[:1] + b"X" + b[2:],          # signature
                   lambda b: b.replace(b"SNOD", b"SNOX"),   # symbol-table node
                   lambda b: b.replace(b"TREE", b"TREX")):  # B-tree node
        p = tmp_path / "bad.h5"
        p.write_bytes(damage(good))
        with pytest.raises(hdf5_min.FormatError):
            hdf5_min.read(str(p))


@pytest.mark.parametrize("golden,fixture,params", [
    (N20, "blackhole_N20.npy", ["12", "1", "1", "10", "1e-8", "0.01", "20", "2", "4", "1", "40"]),
    (N1, "blackhole_N1_LB.npy", ["12", "1", "1", "1000", "1e-8", "1", "1", "1", "1", "1", "40"]),
])
def test_save_result_hdf5_matches_golden_layout(tmp_path, golden, fixture, params):
    gold = np.load(os.path.join(GOLD, fixture))
    (tmp_path / "s.bin").write_bytes(np.ascontiguousarray(gold, dtype="<f8").tobytes())
    exe = _compile(tmp_path, SAVE_SRC, "save")
    out = str(tmp_path / "out")
    subprocess.check_call([exe, out, str(tmp_path / "s.bin"), str(gold.shape[0]), str(gold.shape[1])] + params)
    ours = hdf5_min.read(out + ".h5", with_layout=True)
    ref = _manifest()[golden]
    assert list(ours) == [e["name"] for e in ref]
    for k, e in enumerate(ref):
        arr, attrs, kinds, addr = ours[e["name"]]
        assert list(arr.shape) == e["shape"] and arr.dtype.str == e["dtype"]
        assert np.array_equal(arr, gold[int(e["name"][4:])])  # bit for bit
        # the golden headers spill into continuation blocks (0x10, with NIL
        # padding 0x00); the messages themselves are the same kinds
        assert sorted(set(kinds)) == sorted(set(e["messages"]) - {0x00, 0x10})
        got = [[n, v.dtype.str, v.tolist()] for n, v in attrs.items()]
        assert [a[:2] for a in got] == [a[:2] for a in e["attributes"]]
        for (n, _, v), (_, _, w) in zip(got, e["attributes"]):
            if n == "fastIntegration":
                # a bool written as int32; the golden's upper bytes are not
                # the value (only its low byte is set)
                assert v == [0] and (w[0] & 0xFF) == 0
            else:
                assert v == w, n


def test_save_result_hdf5_file_name_many_datasets_and_sparse_matrix(tmp_path):
    exe = _compile(tmp_path, FLAGGED_SRC, "flagged")
    subprocess.check_call([exe, str(tmp_path)])
    d = hdf5_min.read(str(tmp_path / "Result_N20_dt0.1_fast1.h5"))
    assert list(d) == sorted("obs%d" % k for k in range(20))  # links in name order
    for k in range(20):
        arr, attrs = d["obs%d" % k]
        assert arr.tolist() == [k + 0.5, -1.0 * k]
        assert [(n, v.dtype.str, v.tolist()) for n, v in attrs.items()] == [
            ("N", "<i4", [20]), ("tol", "<f8", [1e-8]), ("dt", "<f8", [0.1]), ("fast", "<i4", [1])]
    s = hdf5_min.read(str(tmp_path / "sparse.h5"))
    assert list(s) == ["columIndex", "dimension", "rowIndex", "valuesImagPart", "valuesRealPart"]
    assert s["valuesRealPart"][0].tolist() == [1.0, 0.25, -3.0]
    assert s["valuesImagPart"][0].tolist() == [-2.0, 0.0, 4.5]
    assert s["columIndex"][0].dtype.str == "<u8" and s["columIndex"][0].tolist() == [2, 0, 1]
    assert s["rowIndex"][0].tolist() == [0, 1, 2] and s["dimension"][0].tolist() == [3]
