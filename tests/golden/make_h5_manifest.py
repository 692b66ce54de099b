"""Record the structure of the reference's golden HDF5 result files as JSON
(datasets in link order with shape, dtype, data address and message types;
attributes with dtype and value), read with tests/hdf5_min.py.  The tests
compare this library's HDF5 writer against it and, where the reference tree
is present, re-read the golden files to check the reader.

Run: ``python tests/golden/make_h5_manifest.py [reference_root]`` (default:
``$TE_REFERENCE_DIR``).
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
import hdf5_min  # noqa: E402

FILES = ["ResultBlackHole_N20_Nm2_K4_C1_DeltaN12_C01_Cm1_maxT10_tol1e-08_samplingStep0.01_m40_fastIntegration0.h5",
         "ResultBlackHole_N1_Nm1_K1_C1_DeltaN12_C01_Cm1_maxT1000_tol1e-08_samplingStep1_m40_fastIntegration0.h5"]


def describe(path):
    out = []
    for name, (arr, attrs, kinds, addr) in hdf5_min.read(path, with_layout=True).items():
        out.append({"name": name, "shape": list(arr.shape), "dtype": arr.dtype.str, "data_address": addr,
                    "messages": sorted(set(kinds)),
                    "attributes": [[k, v.dtype.str, v.tolist()] for k, v in attrs.items()]})
    return out


def main(ref_root):
    man = {f: describe(os.path.join(ref_root, "output", f)) for f in FILES}
    with open(os.path.join(HERE, "h5_manifest.json"), "w") as fh:
        json.dump(man, fh, indent=1)


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("TE_REFERENCE_DIR")
    if not root:
        sys.exit("usage: make_h5_manifest.py REFERENCE_DIR (or set TE_REFERENCE_DIR)")
    main(root)
