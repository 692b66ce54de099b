"""The buffer cache of the library (include/tegpu.h: te_set_buffer_cache_limit,
te_release_buffers; needs a GB300): evolutions reuse released buffers of the
same size, and results do not depend on whether a buffer was reused."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _evolve(te, H, v, O):
    return te.evolve(H, v, 1.0, 0.25, [("sparse", O)], tol=1e-8, m=30)


def test_buffer_cache_reuse_gives_identical_results(te_gpu):
    from oracle import models
    states, H = models.bose_hubbard(9, 9, 1.0, 2.0)
    n = len(states)
    rng = np.random.default_rng(5)
    v = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    v /= np.linalg.norm(v)
    O = models.create_matrix([models.number_operator(0, 1.0)], states)
    te_gpu.set_buffer_cache_limit(8 << 30)
    te_gpu.release_buffers()
    first = _evolve(te_gpu, H, v, O)
    held = te_gpu.buffer_cache_bytes()
    assert held > 0  # the released basis and matrices are kept
    again = _evolve(te_gpu, H, v, O)  # reuses them
    te_gpu.set_buffer_cache_limit(0)
    assert te_gpu.buffer_cache_bytes() == 0
    fresh = _evolve(te_gpu, H, v, O)  # no cache at all
    assert te_gpu.buffer_cache_bytes() == 0
    te_gpu.set_buffer_cache_limit(8 << 30)
    for r in (again, fresh):
        assert np.array_equal(r["state"], first["state"])
        assert np.array_equal(r["samples"], first["samples"])
        assert r["err"] == first["err"] and r["n_steps"] == first["n_steps"]
    te_gpu.release_buffers()
    assert te_gpu.buffer_cache_bytes() == 0


def test_buffer_cache_limit_rejects_negative(te_gpu):
    with pytest.raises(te_gpu.TeError):
        te_gpu.set_buffer_cache_limit(-1)
