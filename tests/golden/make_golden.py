"""Extract the reference's golden observable trajectories into small .npy fixtures.

The reference ships its expected outputs as HDF5 files (``output/*.h5``) and
6-significant-digit CSV copies (``output/*.csv``).  Each HDF5 dataset
``mode<i>`` is stored as a contiguous little-endian float64 array of 1001
values; the byte offsets below were located once and are verified here against
the CSV copies (relative agreement at the CSV's 6-digit precision), so no HDF5
library is needed.

Fixtures written next to this script:

* ``blackhole_N20.npy``   (10, 1001)  -- ``test/testBlackHole.cpp:23`` golden,
  tensorBasis(20,2,2,8,1), dim 588, tol 1e-8, samplingStep 0.01, m 40.
* ``blackhole_N1_LB.npy`` (4, 1001)   -- ``test/testBlackHoleLB.cpp:24`` golden,
  dim 4, t=1000, samplingStep 1, lucky breakdown.
* ``simple_example.npy``  (2, 1001)   -- ``test/testSimpleExample.cpp`` golden
  (CSV only, 6 significant digits), two coupled oscillators, dim 201, tol 1e-6.

Run from anywhere: ``python tests/golden/make_golden.py [reference_root]`` (default:
``$TE_REFERENCE_DIR``).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

N20 = ("ResultBlackHole_N20_Nm2_K4_C1_DeltaN12_C01_Cm1_maxT10_tol1e-08_"
       "samplingStep0.01_m40_fastIntegration0")
N1 = ("ResultBlackHole_N1_Nm1_K1_C1_DeltaN12_C01_Cm1_maxT1000_tol1e-08_"
      "samplingStep1_m40_fastIntegration0")
N20_OFFSETS = [2048, 12104, 20112, 30168, 38176, 48232, 56240, 66296, 76352, 84360]
N1_OFFSETS = [2048, 12104, 20112, 30168]
NVALS = 1001


def _read_csv(path):
    with open(path) as f:
        return np.array([float(x) for x in f.read().split(",")])


def _extract(out_dir, stem, offsets):
    raw = open(os.path.join(out_dir, stem + ".h5"), "rb").read()
    rows = []
    for i, off in enumerate(offsets):
        a = np.frombuffer(raw[off:off + 8 * NVALS], dtype="<f8").copy()
        csv = _read_csv(os.path.join(out_dir, stem + "mode%d.csv" % i))
        assert csv.shape == (NVALS,)
        rel = np.max(np.abs(a - csv) / np.maximum(1.0, np.abs(a)))
        assert rel < 1e-5, (stem, i, rel)
        rows.append(a)
    return np.stack(rows)


def main(ref_root):
    out_dir = os.path.join(ref_root, "output")
    np.save(os.path.join(HERE, "blackhole_N20.npy"), _extract(out_dir, N20, N20_OFFSETS))
    np.save(os.path.join(HERE, "blackhole_N1_LB.npy"), _extract(out_dir, N1, N1_OFFSETS))
    simple = np.stack([_read_csv(os.path.join(out_dir, "SimpleExampleOutputOccupationNumber%d.csv" % i))
                       for i in range(2)])
    np.save(os.path.join(HERE, "simple_example.npy"), simple)


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("TE_REFERENCE_DIR")
    if not root:
        sys.exit("usage: make_golden.py REFERENCE_DIR (or set TE_REFERENCE_DIR)")
    main(root)
