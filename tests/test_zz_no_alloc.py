"""te_matrix_spmv_noalloc: the sparse product for callers that cannot
allocate device memory (stream capture, real-time loops, preallocated memory
budgets).  It must give the same result as te_matrix_spmv, on two calls in a
row (the fixed scratch keeps the previous call's contents), and refuse
matrices larger than its fixed scratch.  Collected last on purpose."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.complex128).view(np.float64)).cuda()


def test_noalloc_spmv_matches_allocating_spmv():
    torch = pytest.importorskip("torch")
    import timeevolver_gb300 as te
    from timeevolver_gb300 import models
    te.build()
    te.lib().te_set_device(0)
    B, H = models.bose_hubbard(8, 8, 1.0, 2.0)
    n = len(B)
    M = te.Matrix.from_coo(n, H)
    rng = np.random.default_rng(11)
    for call, alpha in enumerate([-0.5j, 0.25 + 1.5j]):
        x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        xd = _dev(torch, x)
        y_ref = torch.zeros_like(xd)
        y_na = torch.full_like(xd, float("nan"))
        a = complex(alpha)
        rc = te.lib().te_matrix_spmv(M.handle, a.real, a.imag, ctypes.c_void_p(xd.data_ptr()),
                                     ctypes.c_void_p(y_ref.data_ptr()), None)
        assert rc == 0
        rc = te.lib().te_matrix_spmv_noalloc(M.handle, a.real, a.imag, ctypes.c_void_p(xd.data_ptr()),
                                             ctypes.c_void_p(y_na.data_ptr()), None)
        assert rc == 0, te.lib().te_last_error()
        torch.cuda.synchronize()
        r = y_ref.cpu().numpy().view(np.complex128)
        g = y_na.cpu().numpy().view(np.complex128)
        assert np.all(np.isfinite(g)), call
        assert np.linalg.norm(g - r) <= 1e-13 * np.linalg.norm(r), call


def test_noalloc_spmv_rejects_oversized_matrix():
    torch = pytest.importorskip("torch")
    import timeevolver_gb300 as te
    te.build()
    te.lib().te_set_device(0)
    n = (1 << 18) + 1
    idx = np.arange(n)
    M = te.Matrix(n, idx, idx, np.ones(n, dtype=np.complex128))
    xd = torch.zeros(2 * n, dtype=torch.float64, device="cuda")
    yd = torch.zeros_like(xd)
    rc = te.lib().te_matrix_spmv_noalloc(M.handle, 1.0, 0.0, ctypes.c_void_p(xd.data_ptr()),
                                         ctypes.c_void_p(yd.data_ptr()), None)
    assert rc == -9
    assert b"exceed the fixed scratch" in te.lib().te_last_error()
