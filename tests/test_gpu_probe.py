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


def test_gather_probe_modes_agree(te_gpu):
    """Ordinary loads and TMA tile::gather4 copies fetch the same rows: equal
    checksums, on random indices and on a matrix's SELL slot columns."""
    from timeevolver_gb300 import models
    # the same launch shape for both, so that the warps walk the same indices
    lsu = te_gpu.probe_gather(0, 2, blocks_per_sm=3, n_rows=1 << 20, n_gathers=1 << 23)
    tma = te_gpu.probe_gather(1, 8, blocks_per_sm=3, n_rows=1 << 20, n_gathers=1 << 23)
    assert lsu[0] > 0 and tma[0] > 0
    assert lsu[1] == tma[1]
    B, coo = models.bose_hubbard(10, 10, 1.0, 2.0)
    H = te_gpu.Matrix.from_coo(len(B), coo)
    try:
        a = te_gpu.probe_gather(0, 4, blocks_per_sm=2, matrix=H)
        b = te_gpu.probe_gather(1, 4, blocks_per_sm=2, matrix=H)
        assert a[1] == b[1]
    finally:
        H.close()


def test_gather_probe_rejects_bad_shapes(te_gpu):
    with pytest.raises(te_gpu.TeError):
        te_gpu.probe_gather(0, 3)
    with pytest.raises(te_gpu.TeError):
        te_gpu.probe_gather(1, 2)
