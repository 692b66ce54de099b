"""Hardware probes of the library used by the benchmark's FP64 roofline
(include/te_diag.h; needs a GB300)."""
import math

import pytest

pytestmark = pytest.mark.gpu


def test_fp64_throughput_probe(te_gpu):
    tf = te_gpu.probe_fp64_tflops()
    assert math.isfinite(tf) and tf > 0.1


def test_fp64_issue_probe(te_gpu):
    one = te_gpu.probe_fp64_issue(1)
    four = te_gpu.probe_fp64_issue(4)
    for indep, chain in (one, four):
        assert math.isfinite(indep) and indep > 0.0
        assert math.isfinite(chain) and chain > 0.0
    # four warps share the SM's FP64 issue: per warp FMA the SM needs no more
    # cycles than with one warp, and a chain's FMAs come no faster
    assert four[0] <= one[0] * 1.05
    assert four[1] >= one[1] * 0.95


def test_fp64_issue_probe_rejects_bad_shapes(te_gpu):
    with pytest.raises(te_gpu.TeError):
        te_gpu.probe_fp64_issue(0)
    with pytest.raises(te_gpu.TeError):
        te_gpu.probe_fp64_issue(33)
