"""timeevolver_gb300 -- Krylov real-time evolution exp(-iHt)v on one GB300.

Python binding (ctypes) of the C ABI in include/tegpu.h, implemented by the
hand-written sm_103a kernels in ``csrc/`` (built into ``_build/libtegpu.so``).
The native library is required: every entry point raises if it is missing;
there is no CPU fallback.

Mirrors TimeEvolver's krylovTimeEvolver API (core/krylovTimeEvolver.h:56-68):
``Evolver(H, v, t, sampling_step, observables, exp_factor, tol, m,
fast_integration).time_evolve()`` returns the krylovReturn fields.
"""
import ctypes
import os

import numpy as np

from . import build as _build

LIB_PATH = _build.LIB_TEGPU

TE_OK = 0
ERRORS = {
    -1: "invalid argument", -2: "CUDA error", -3: "invalid Hilbert-space dimension",
    -4: "initial vector is not normalized", -5: "no small enough time step found to meet the tolerance",
    -6: "Krylov eigensolver did not converge", -7: "incompatible dimensions", -8: "out of device memory",
    -9: "unsupported size or parameter", -10: "device wait timed out",
}
STATUS = {0: "ok", 1: "lucky breakdown", 2: "analytic error below roundoff estimate", 3: "stopped by observable",
          10: "roundoff may spoil the error", 11: "tolerance unreachable (roundoff)",
          20: "quadrature inaccurate", 30: "norm drift", 100: "multiple warnings"}


class TeParams(ctypes.Structure):
    _fields_ = [("t", ctypes.c_double), ("sampling_step", ctypes.c_double), ("exp_factor", ctypes.c_double),
                ("tol", ctypes.c_double), ("m", ctypes.c_int32), ("fast_integration", ctypes.c_int32),
                ("progress_bar", ctypes.c_int32), ("reorth", ctypes.c_int32)]


class TeResult(ctypes.Structure):
    _fields_ = [("err", ctypes.c_double), ("evolved_time", ctypes.c_double), ("num_samples", ctypes.c_int64),
                ("n_steps", ctypes.c_int64), ("dim", ctypes.c_int64), ("krylov_dim", ctypes.c_int64),
                ("status", ctypes.c_int32), ("nb_err_roundoff", ctypes.c_int32), ("nb_err_int", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


class TeStepRecord(ctypes.Structure):
    _fields_ = [("t_now", ctypes.c_double), ("t_step", ctypes.c_double), ("err_step", ctypes.c_double),
                ("h", ctypes.c_double), ("m_eff", ctypes.c_int32), ("breakdown", ctypes.c_int32),
                ("code", ctypes.c_int32), ("n_integrals", ctypes.c_int32)]


OBSERVABLE_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_int64,
                                 ctypes.POINTER(ctypes.c_double))

# every entry point of include/tegpu.h: name -> (restype, argtypes)
_P = ctypes.c_void_p
_I64, _I32, _D, _I = ctypes.c_int64, ctypes.c_int32, ctypes.c_double, ctypes.c_int
SIGNATURES = {
    "te_last_error": (ctypes.c_char_p, []),
    "te_abi_version": (_I, []),
    "te_set_device": (_I, [_I]),
    "te_set_buffer_cache_limit": (_I, [_I64]),
    "te_release_buffers": (_I, []),
    "te_buffer_cache_bytes": (_I64, []),
    "te_matrix_create_coo": (_I, [_I64, _I64, _I64, _P, _P, _P, _P]),
    "te_matrix_create_csr": (_I, [_I64, _I64, _I64, _P, _P, _P, _I, _P]),
    "te_matrix_destroy": (_I, [_P]),
    "te_matrix_info": (_I, [_P, _P, _P, _P, _P, _P]),
    "te_matrix_spmv": (_I, [_P, _D, _D, _P, _P, _P]),
    "te_matrix_spmv_host": (_I, [_P, _D, _D, _P, _P]),
    "te_matrix_spmv_noalloc": (_I, [_P, _D, _D, _P, _P, _P]),
    "te_matrix_create_csr_device": (_I, [_I64, _I64, _I64, _P, _P, _P, _I, _P]),
    "te_matrix_download_csr": (_I, [_P, _P, _P, _P]),
    "te_matrix_set_spmv_lanes": (_I, [_P, _I]),
    "te_matrix_layout": (_I, [_P, _P, _P, _P]),
    "te_matrix_long_segments": (_I, [_P, _P, _P, _P]),
    "te_model_create_device": (_I, [_I, _I, _I, _P, _I, _P, _P]),
    "te_model_state_index": (_I, [_I, _I, _I, _P, _P]),
    "te_model_create_device_basis": (_I, [_P, _P, _I, _P, _P]),
    "te_model_basis_index": (_I, [_P, _P, _P]),
    "te_matrix_spmv_lanes": (_I, [_P, _I]),
    "te_matrix_fixed_layout": (_I, [_P, _P, _P, _P]),
    "te_matrix_set_fixed_blocks": (_I, [_P, _I]),
    "te_matrix_create_zipf": (_I, [_I64, _D, ctypes.c_int32, ctypes.c_int32, ctypes.c_uint64, ctypes.c_int32, _P, _P]),
    "te_evolver_create": (_I, [_P, _P, _P, _P]),
    "te_evolver_destroy": (_I, [_P]),
    "te_evolver_add_sparse_observable": (_I, [_P, _P]),
    "te_evolver_add_vector_observable": (_I, [_P, _P]),
    "te_evolver_add_callback_observable": (_I, [_P, OBSERVABLE_FN, _P]),
    "te_evolver_run": (_I, [_P, _P]),
    "te_evolver_samples": (_I, [_P, _I, _P, _I64]),
    "te_evolver_state": (_I, [_P, _P]),
    "te_evolver_state_device": (_I, [_P, _P]),
    "te_evolver_trace": (_I, [_P, _P, _I64, _P]),
    "te_evolver_launch_count": (_I64, [_P]),
    "te_evolver_krylov_matrix": (_I, [_P, _P, _P, _P, _P, _P]),
    "te_evolver_reset": (_I, [_P, _P, _I]),
    "te_evolver_stream": (_P, [_P]),
    "te_evolver_profile": (_I, [_P, _I]),
    "te_evolver_kernel_time": (_I, [_P, _I, _P, _P]),
    "te_probe_fp64_tflops": (_I, [_P]),
    "te_probe_fp64_issue": (_I, [_I, _I, _P, _P]),
    "te_probe_gather": (_I, [_P, _I64, _I64, _I, _I, _I, _P, _P]),
    "te_batch_create": (_I, [_I, _P, _P, _P, _P]),
    "te_batch_destroy": (_I, [_P]),
    "te_batch_add_observable": (_I, [_P, _I, _P]),
    "te_batch_run": (_I, [_P, _P]),
    "te_batch_samples": (_I, [_P, _I, _I, _P, _I64]),
    "te_batch_state": (_I, [_P, _I, _P]),
    "te_batch_launch_count": (_I64, [_P]),
    "te_batch_stream": (_P, [_P]),
    "te_batch_global_steps": (_I64, [_P]),
    "te_batch_set_option": (_I, [_P, _I, _I]),
    "te_evolver_set_option": (_I, [_P, _I, _I]),
    "te_evolver_add_dense_observable": (_I, [_P, _P, _I64]),
    "te_evolver_add_stop_condition": (_I, [_P, _I, _D, _I]),
    "te_adjoint_create": (_I, [_I, _P, _P, _P, _D, _D, _I, _D, _I, _P]),
    "te_adjoint_destroy": (_I, [_P]),
    "te_adjoint_run": (_I, [_P, _P, _P, _P]),
    "te_adjoint_forward": (_I, [_P, _P, _P]),
    "te_adjoint_stats": (_I, [_P, _P, _P, _P, _P]),
    "te_adjoint_phase_times": (_I, [_P, _P]),
}

_lib = None


class TeError(RuntimeError):
    def __init__(self, code, where):
        msg = lib().te_last_error().decode(errors="replace")
        super().__init__("%s failed: %s (%d) %s" % (where, ERRORS.get(code, "error"), code, msg))
        self.code = code


def build(force=False, verbose=False):
    return _build.build_all(force=force, verbose=verbose)


def lib():
    """The loaded libtegpu.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libtegpu.so is missing (%s): run timeevolver_gb300.build() first; "
                               "there is no CPU fallback" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def state_index_device(n_particles, occupation, quant=1):
    """Index of an occupation vector in basis(n_particles, len(occupation)) (te_model_state_index)."""
    occ = np.ascontiguousarray(occupation, dtype=np.int32)
    r = ctypes.c_int64()
    _check(lib().te_model_state_index(int(n_particles), len(occ), int(quant), _ptr(occ), ctypes.byref(r)),
           "te_model_state_index")
    return r.value


def set_buffer_cache_limit(device_bytes):
    """Cap the device bytes the library keeps for reuse after releasing
    buffers (0 disables the cache and frees what it holds)."""
    _check(lib().te_set_buffer_cache_limit(int(device_bytes)), "te_set_buffer_cache_limit")


def release_buffers():
    """Free every buffer the library keeps for reuse."""
    _check(lib().te_release_buffers(), "te_release_buffers")


def buffer_cache_bytes():
    """Device bytes currently kept for reuse."""
    return int(lib().te_buffer_cache_bytes())


def probe_fp64_tflops():
    """Measured FP64 FMA throughput of the current device (TFLOP/s)."""
    x = ctypes.c_double()
    _check(lib().te_probe_fp64_tflops(ctypes.byref(x)), "te_probe_fp64_tflops")
    return x.value


def probe_fp64_issue(warps, blocks=1):
    """FP64 FMA issue with ``warps`` warps per block on ``blocks`` blocks:
    (cycles per warp FMA per block with 8 independent chains per thread,
    cycles per FMA of one dependent chain)."""
    a, b = ctypes.c_double(), ctypes.c_double()
    _check(lib().te_probe_fp64_issue(int(warps), int(blocks), ctypes.byref(a), ctypes.byref(b)),
           "te_probe_fp64_issue")
    return a.value, b.value


def probe_gather(mode, depth, blocks_per_sm=6, matrix=None, n_rows=1352078, n_gathers=16871581):
    """Gathers of 16-byte rows per second (include/te_diag.h): mode 0 ordinary
    loads (depth rows in flight per lane), mode 1 TMA tile::gather4 (depth
    stages per warp); the indices are the SELL slot columns of ``matrix`` or
    uniform random.  Returns (rows_per_s, checksum)."""
    rate, csum = ctypes.c_double(), ctypes.c_ulonglong()
    _check(lib().te_probe_gather(matrix.handle if matrix is not None else None, int(n_rows), int(n_gathers),
                                 int(mode), int(depth), int(blocks_per_sm), ctypes.byref(rate), ctypes.byref(csum)),
           "te_probe_gather")
    return rate.value, csum.value


def _check(rc, where):
    if rc != TE_OK:
        raise TeError(rc, where)


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _as_u64(a):
    """Index array as uint64 (int64 input is reinterpreted without a copy;
    negative entries become out-of-range indices, which the library rejects)."""
    a = np.ascontiguousarray(a)
    if a.dtype == np.int64:
        return a.view(np.uint64)
    return np.ascontiguousarray(a, dtype=np.uint64)


OPT_FUSED_LANCZOS = 1
OPT_FIXED_SPMV = 2
OPT_BARRIER_SPIN_LIMIT = 3
OPT_BARRIER_EXTRA_ARRIVALS = 4
OPT_TS_MAX_LEVEL = 5
OPT_QR_SWEEP_LIMIT = 6
BATCH_OPT_PERSISTENT = 1
BATCH_OPT_BARRIER_SPIN_LIMIT = 2
BATCH_OPT_BARRIER_EXTRA_ARRIVALS = 3


class TeBasisDesc(ctypes.Structure):
    _fields_ = [("n_particles", ctypes.c_int32), ("n_modes", ctypes.c_int32), ("n_qudits", ctypes.c_int32),
                ("capacity", ctypes.c_int32), ("quant", ctypes.c_int32), ("n_particles2", ctypes.c_int32),
                ("n_modes2", ctypes.c_int32), ("capacity2", ctypes.c_int32)]


def basis_desc(N, K, nb_qudits=0, capacity=0, quant=1, tensor=None):
    """te_basis_desc of basis(N, K, nbQudits, capacity, quant), or with
    tensor=(N1, K1, N2, K2, C2) of tensorBasis(N1, K1, N2, K2, C2)."""
    if tensor is not None:
        N1, K1, N2, K2, C2 = tensor
        return TeBasisDesc(N1, K1, 0, 0, 1, N2, K2, C2)
    return TeBasisDesc(N, K, nb_qudits, capacity, quant, 0, 0, 0)


def basis_index_device(desc, occupation):
    """Index of an occupation vector in the basis of a te_basis_desc (te_model_basis_index)."""
    occ = np.ascontiguousarray(occupation, dtype=np.int32)
    r = ctypes.c_int64()
    _check(lib().te_model_basis_index(ctypes.byref(desc), _ptr(occ), ctypes.byref(r)), "te_model_basis_index")
    return r.value


def _term_array(terms):
    arr = (TeTerm * len(terms))()
    for t, (coef, ops, modes, caps) in zip(arr, terms):
        c = complex(coef)
        t.coef_re, t.coef_im, t.n_ops = c.real, c.imag, len(ops)
        for k, (o, m_, cp) in enumerate(zip(ops, modes, caps)):
            t.operation[k], t.mode[k], t.capacity[k] = o, m_, cp
    return arr


class TeTerm(ctypes.Structure):
    _fields_ = [("coef_re", ctypes.c_double), ("coef_im", ctypes.c_double), ("n_ops", ctypes.c_int32),
                ("operation", ctypes.c_int32 * 8), ("mode", ctypes.c_int32 * 8), ("capacity", ctypes.c_int32 * 8)]


class Matrix:
    """Device sparse matrix (TE::smatrix): from COO arrays (row, col, values)."""

    def __init__(self, n, row, col, val, n_cols=None):
        row, col = _as_u64(row), _as_u64(col)
        val = np.ascontiguousarray(val, dtype=np.complex128)
        self.handle = ctypes.c_void_p()
        self.n = int(n)
        _check(lib().te_matrix_create_coo(self.n, int(n_cols or n), len(val), _ptr(row), _ptr(col), _ptr(val),
                                          ctypes.byref(self.handle)), "te_matrix_create_coo")

    @classmethod
    def from_coo(cls, n, coo):
        return cls(n, coo[0], coo[1], coo[2])

    @classmethod
    def _adopt(cls, handle):
        M = cls.__new__(cls)
        M.handle = handle
        M.n = M.info()["n_rows"]
        return M

    @classmethod
    def from_csr(cls, n_rows, row_ptr, col, values, n_cols=None):
        """From a host CSR (te_matrix_create_csr): row_ptr (n_rows + 1), col,
        complex values; the layout is built on the host."""
        rp = np.ascontiguousarray(row_ptr, dtype=np.int64)
        ci = np.ascontiguousarray(col, dtype=np.int32)
        val = np.ascontiguousarray(values, dtype=np.complex128)
        h = ctypes.c_void_p()
        _check(lib().te_matrix_create_csr(int(n_rows), int(n_cols or n_rows), len(ci), _ptr(rp), _ptr(ci), _ptr(val),
                                          1, ctypes.byref(h)), "te_matrix_create_csr")
        return cls._adopt(h)

    @classmethod
    def from_device_csr(cls, n_rows, row_ptr, col, values, n_cols=None):
        """From a CSR already on the GPU (torch tensors: int32 row_ptr and
        col, complex128 or float64 values); the arrays are copied."""
        import torch
        assert row_ptr.dtype == torch.int32 and col.dtype == torch.int32 and row_ptr.is_cuda
        cplx = values.dtype == torch.complex128
        vals = torch.view_as_real(values.contiguous()) if cplx else values.contiguous()
        h = ctypes.c_void_p()
        _check(lib().te_matrix_create_csr_device(int(n_rows), int(n_cols or n_rows), int(col.numel()),
                                                 ctypes.c_void_p(row_ptr.data_ptr()), ctypes.c_void_p(col.data_ptr()),
                                                 ctypes.c_void_p(vals.data_ptr()), int(cplx), ctypes.byref(h)),
               "te_matrix_create_csr_device")
        return cls._adopt(h)

    @classmethod
    def zipf(cls, n, exponent=1.5, min_len=2, max_len=256, seed=1, power_iters=30):
        """The synthetic load-imbalanced Hermitian matrix generated on the
        device (te_matrix_create_zipf).  Returns (Matrix, norm_estimate)."""
        h = ctypes.c_void_p()
        est = ctypes.c_double(0.0)
        _check(lib().te_matrix_create_zipf(int(n), float(exponent), int(min_len), int(max_len), int(seed),
                                           int(power_iters), ctypes.byref(est), ctypes.byref(h)),
               "te_matrix_create_zipf")
        return cls._adopt(h), est.value

    @classmethod
    def from_terms_device(cls, n_particles, n_modes, terms, quant=1):
        """Operator matrix built on the GPU (te_model_create_device) from terms
        (coef, operations, modes, capacities) -- the tuples of
        timeevolver_gb300.models -- on basis(n_particles, n_modes).
        Returns (Matrix, dim)."""
        arr = (TeTerm * len(terms))()
        for t, (coef, ops, modes, caps) in zip(arr, terms):
            c = complex(coef)
            t.coef_re, t.coef_im, t.n_ops = c.real, c.imag, len(ops)
            for k, (o, m_, cp) in enumerate(zip(ops, modes, caps)):
                t.operation[k], t.mode[k], t.capacity[k] = o, m_, cp
        h = ctypes.c_void_p()
        dim = ctypes.c_int64()
        _check(lib().te_model_create_device(int(n_particles), int(n_modes), int(quant), arr, len(terms),
                                            ctypes.byref(h), ctypes.byref(dim)), "te_model_create_device")
        return cls._adopt(h), dim.value

    @classmethod
    def from_terms_device_basis(cls, desc, terms):
        """Operator matrix built on the GPU on the basis of a te_basis_desc
        (basis_desc(): qudit capacities, tensor bases).  Returns (Matrix, dim)."""
        arr = _term_array(terms)
        h = ctypes.c_void_p()
        dim = ctypes.c_int64()
        _check(lib().te_model_create_device_basis(ctypes.byref(desc), arr, len(terms), ctypes.byref(h),
                                                  ctypes.byref(dim)), "te_model_create_device_basis")
        return cls._adopt(h), dim.value

    def to_csr(self):
        """(row_ptr int32, col int32, values complex128) of the original-order CSR, on the host."""
        inf = self.info()
        rp = np.zeros(inf["n_rows"] + 1, dtype=np.int32)
        ci = np.zeros(max(1, inf["nnz"]), dtype=np.int32)
        val = np.zeros(max(1, inf["nnz"]), dtype=np.complex128)
        _check(lib().te_matrix_download_csr(self.handle, _ptr(rp), _ptr(ci), _ptr(val)), "te_matrix_download_csr")
        return rp, ci[:inf["nnz"]], val[:inf["nnz"]]

    def layout(self):
        """SELL-32 slots, long rows and their entries (te_matrix_layout)."""
        a, b, c = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        _check(lib().te_matrix_layout(self.handle, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)),
               "te_matrix_layout")
        return dict(sell_slots=a.value, long_rows=b.value, long_entries=c.value)

    def long_segments(self):
        """Merge-path segments of the long rows (te_matrix_long_segments)."""
        a, b, c = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        _check(lib().te_matrix_long_segments(self.handle, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)),
               "te_matrix_long_segments")
        return dict(segments=a.value, split_rows=b.value, segment_items=c.value)

    def fixed_layout(self):
        """Fixed-point form for the integer SpMV (te_matrix_fixed_layout):
        state 0 not built, 1 limbs per slot, 2 value dictionary, 3 limbs in column
        blocks (n_values = number of blocks)."""
        st, nv, sh = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _check(lib().te_matrix_fixed_layout(self.handle, ctypes.byref(st), ctypes.byref(nv), ctypes.byref(sh)),
               "te_matrix_fixed_layout")
        return dict(state=st.value, n_values=nv.value, scale_shift=sh.value)

    def set_fixed_blocks(self, n_blocks):
        """Column blocks of the fixed-point form: 0 automatic, 1 none, 2..8."""
        _check(lib().te_matrix_set_fixed_blocks(self.handle, int(n_blocks)), "te_matrix_set_fixed_blocks")

    def spmv_lanes(self, tune=True):
        """Lanes per row of the SpMV passes (tuned on first use unless pinned)."""
        k = lib().te_matrix_spmv_lanes(self.handle, int(bool(tune)))
        if k < 0:
            _check(k, "te_matrix_spmv_lanes")
        return k

    def set_spmv_lanes(self, lanes):
        """Pin the lanes per row (1, 2, 4), reopen the choice by shape (0) or
        let the autotuner time the variants on first use (-1)."""
        _check(lib().te_matrix_set_spmv_lanes(self.handle, int(lanes)), "te_matrix_set_spmv_lanes")

    def to_coo(self):
        """(row, col, values) COO triple of the matrix, on the host."""
        rp, ci, val = self.to_csr()
        row = np.repeat(np.arange(len(rp) - 1, dtype=np.int64), np.diff(rp))
        return row, ci.astype(np.int64), val

    def info(self):
        nr, nc, nnz, fl, n1 = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int(), ctypes.c_double()
        _check(lib().te_matrix_info(self.handle, ctypes.byref(nr), ctypes.byref(nc), ctypes.byref(nnz),
                                    ctypes.byref(fl), ctypes.byref(n1)), "te_matrix_info")
        return dict(n_rows=nr.value, n_cols=nc.value, nnz=nnz.value, real=bool(fl.value & 1),
                    diagonal=bool(fl.value & 2), norm1=n1.value)

    def spmv(self, x, alpha=1.0):
        x = np.ascontiguousarray(x, dtype=np.complex128)
        y = np.zeros_like(x)
        a = complex(alpha)
        _check(lib().te_matrix_spmv_host(self.handle, a.real, a.imag, _ptr(x), _ptr(y)), "te_matrix_spmv_host")
        return y

    def close(self):
        if self.handle:
            lib().te_matrix_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Evolver:
    """One time evolution (krylovTimeEvolver): construct, add observables, run.

    ``observables`` entries: ("sparse", Matrix), ("vector", ndarray),
    ("dense", n x n ndarray) or ("callback", fn) where ``fn(state) -> float``
    may raise StopEvolution (requestStopException)."""

    def __init__(self, H, v, t, sampling_step, observables=(), exp_factor=1.0, tol=1e-6, m=40,
                 fast_integration=False, reorth=False):
        self.H = H
        self.n = H.n
        v = np.ascontiguousarray(v, dtype=np.complex128)
        p = TeParams(t, sampling_step, exp_factor, tol, int(m), int(bool(fast_integration)), 0, int(bool(reorth)))
        self.handle = ctypes.c_void_p()
        _check(lib().te_evolver_create(H.handle, _ptr(v), ctypes.byref(p), ctypes.byref(self.handle)),
               "te_evolver_create")
        self.n_samples = int(np.floor(t / sampling_step)) + 1
        self._keep = []
        self.n_obs = 0
        for kind, data in observables:
            self.add(kind, data)

    def add(self, kind, data):
        if kind == "sparse":
            _check(lib().te_evolver_add_sparse_observable(self.handle, data.handle), "add_sparse_observable")
            self._keep.append(data)
        elif kind == "vector":
            o = np.ascontiguousarray(data, dtype=np.complex128)
            _check(lib().te_evolver_add_vector_observable(self.handle, _ptr(o)), "add_vector_observable")
        elif kind == "dense":
            o = np.asfortranarray(data, dtype=np.complex128)  # column-major n x n
            _check(lib().te_evolver_add_dense_observable(self.handle, _ptr(o.reshape(-1, order="F")), o.shape[0]),
                   "add_dense_observable")
        elif kind == "callback":
            fn = data

            def tramp(user, state, dim, out, fn=fn):
                arr = np.ctypeslib.as_array(state, shape=(2 * dim,)).view(np.complex128)
                try:
                    out[0] = float(fn(arr))
                    return 0
                except StopEvolution:
                    return 1

            cb = OBSERVABLE_FN(tramp)
            self._keep.append(cb)
            _check(lib().te_evolver_add_callback_observable(self.handle, cb, None), "add_callback_observable")
        else:
            raise ValueError(kind)
        self.n_obs += 1

    def time_evolve(self, trace=False):
        r = TeResult()
        _check(lib().te_evolver_run(self.handle, ctypes.byref(r)), "te_evolver_run")
        out = dict(err=r.err, evolved_time=r.evolved_time, num_samples=r.num_samples, n_steps=r.n_steps,
                   dim=r.dim, krylov_dim=r.krylov_dim, status=r.status, nb_err_roundoff=r.nb_err_roundoff,
                   nb_err_int=r.nb_err_int)
        samples = np.zeros((self.n_obs, self.n_samples))
        for i in range(self.n_obs):
            _check(lib().te_evolver_samples(self.handle, i, _ptr(samples[i]), self.n_samples), "samples")
        out["samples"] = samples
        st = np.zeros(self.n, dtype=np.complex128)
        _check(lib().te_evolver_state(self.handle, _ptr(st)), "state")
        out["state"] = st
        out["launches"] = lib().te_evolver_launch_count(self.handle)
        if trace:
            cnt = ctypes.c_int64()
            lib().te_evolver_trace(self.handle, None, 0, ctypes.byref(cnt))
            recs = (TeStepRecord * max(1, cnt.value))()
            lib().te_evolver_trace(self.handle, recs, cnt.value, ctypes.byref(cnt))
            out["trace"] = [dict(t_now=x.t_now, t_step=x.t_step, err_step=x.err_step, h=x.h, m_eff=x.m_eff,
                                 breakdown=x.breakdown, code=x.code, n_integrals=x.n_integrals)
                            for x in recs[:cnt.value]]
        return out

    def reset(self, v, device_ptr=None):
        """Re-arm the evolver with a new start vector (host array, or a device
        pointer to n complex doubles)."""
        if device_ptr is not None:
            _check(lib().te_evolver_reset(self.handle, ctypes.c_void_p(device_ptr), 1), "te_evolver_reset")
        else:
            v = np.ascontiguousarray(v, dtype=np.complex128)
            _check(lib().te_evolver_reset(self.handle, _ptr(v), 0), "te_evolver_reset")

    def run(self):
        """timeEvolve without copying results back (they stay on the device)."""
        r = TeResult()
        _check(lib().te_evolver_run(self.handle, ctypes.byref(r)), "te_evolver_run")
        return r

    def stream(self):
        return lib().te_evolver_stream(self.handle)

    def profile(self, enable=True):
        _check(lib().te_evolver_profile(self.handle, int(enable)), "te_evolver_profile")

    def add_stop_condition(self, obs_index, threshold, direction):
        """Stop at the first sample where observable obs_index >= threshold
        (direction > 0) or <= threshold (direction < 0), on the device."""
        _check(lib().te_evolver_add_stop_condition(self.handle, int(obs_index), float(threshold), int(direction)),
               "te_evolver_add_stop_condition")

    def krylov_matrix(self):
        """The last Krylov step's tridiagonal T (te_evolver_krylov_matrix):
        dict with diag, offdiag, eig_used and, when the eigen path ran,
        eigenvalues (unordered)."""
        d = np.zeros(64)
        e = np.zeros(64)
        lam = np.zeros(64)
        m, used = ctypes.c_int32(), ctypes.c_int32()
        _check(lib().te_evolver_krylov_matrix(self.handle, _ptr(d), _ptr(e), _ptr(lam), ctypes.byref(m),
                                              ctypes.byref(used)), "te_evolver_krylov_matrix")
        k = m.value
        out = dict(diag=d[:k].copy(), offdiag=e[:max(0, k - 1)].copy(), eig_used=bool(used.value))
        if used.value:
            out["eigenvalues"] = lam[:k].copy()
        return out

    def set_option(self, option, value):
        """te_evolver_set_option (OPT_FUSED_LANCZOS, OPT_FIXED_SPMV, OPT_BARRIER_SPIN_LIMIT,
        OPT_BARRIER_EXTRA_ARRIVALS, OPT_TS_MAX_LEVEL, OPT_QR_SWEEP_LIMIT)."""
        _check(lib().te_evolver_set_option(self.handle, int(option), int(value)), "te_evolver_set_option")

    def kernel_time(self, kind):
        ms, cnt = ctypes.c_double(), ctypes.c_int64()
        _check(lib().te_evolver_kernel_time(self.handle, kind, ctypes.byref(ms), ctypes.byref(cnt)),
               "te_evolver_kernel_time")
        return ms.value, cnt.value

    def close(self):
        if self.handle:
            lib().te_evolver_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Many independent evolutions advanced together (te_batch_*).

    ``instances``: list of dicts with keys H (Matrix), v, t, sampling_step and
    optional tol, m, exp_factor, fast_integration, observables (list of
    diagonal Matrix objects).  ``persistent``: run the whole batch in one
    persistent launch (TE_BATCH_OPT_PERSISTENT) instead of a graph replay per
    global step."""

    def __init__(self, instances, persistent=False):
        B = len(instances)
        self._keep = []
        Hs = (ctypes.c_void_p * B)()
        vs = (ctypes.c_void_p * B)()
        ps = (TeParams * B)()
        self.n_samples, self.dims, self.n_obs = [], [], []
        for i, ins in enumerate(instances):
            v = np.ascontiguousarray(ins["v"], dtype=np.complex128)
            self._keep += [v, ins["H"]]
            Hs[i] = ins["H"].handle
            vs[i] = v.ctypes.data
            t, dt = float(ins["t"]), float(ins["sampling_step"])
            ps[i] = TeParams(t, dt, float(ins.get("exp_factor", 1.0)), float(ins.get("tol", 1e-6)),
                             int(ins.get("m", 40)), int(bool(ins.get("fast_integration", False))), 0, 0)
            self.n_samples.append(int(np.floor(t / dt)) + 1)
            self.dims.append(len(v))
        self.handle = ctypes.c_void_p()
        _check(lib().te_batch_create(B, Hs, vs, ps, ctypes.byref(self.handle)), "te_batch_create")
        for i, ins in enumerate(instances):
            obs = ins.get("observables", [])
            for O in obs:
                self._keep.append(O)
                _check(lib().te_batch_add_observable(self.handle, i, O.handle), "te_batch_add_observable")
            self.n_obs.append(len(obs))
        self.B = B
        if persistent:
            self.set_option(BATCH_OPT_PERSISTENT, 1)

    def set_option(self, option, value):
        _check(lib().te_batch_set_option(self.handle, int(option), int(value)), "te_batch_set_option")

    def global_steps(self):
        return lib().te_batch_global_steps(self.handle)

    def run(self):
        res = (TeResult * self.B)()
        _check(lib().te_batch_run(self.handle, res), "te_batch_run")
        return [dict(err=r.err, evolved_time=r.evolved_time, num_samples=r.num_samples, n_steps=r.n_steps,
                     dim=r.dim, krylov_dim=r.krylov_dim, status=r.status) for r in res]

    def samples(self, i):
        out = np.zeros((self.n_obs[i], self.n_samples[i]))
        for k in range(self.n_obs[i]):
            _check(lib().te_batch_samples(self.handle, i, k, _ptr(out[k]), self.n_samples[i]), "te_batch_samples")
        return out

    def state(self, i):
        st = np.zeros(self.dims[i], dtype=np.complex128)
        _check(lib().te_batch_state(self.handle, i, _ptr(st)), "te_batch_state")
        return st

    def launch_count(self):
        return lib().te_batch_launch_count(self.handle)

    def stream(self):
        return lib().te_batch_stream(self.handle)

    def close(self):
        if self.handle:
            lib().te_batch_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Adjoint:
    """Gradients of <psi(T)|O|psi(T)> with respect to the couplings theta of
    H = sum_k theta_k H_k (te_adjoint_*).  ``terms``: list of Matrix; ``O``: Matrix."""

    def __init__(self, terms, O, v, T, tol=1e-10, m=40, checkpoint_interval=0.5, nodes_per_interval=24):
        self._keep = [O]  # the terms are copied at creation
        arr = (ctypes.c_void_p * len(terms))(*[t.handle.value for t in terms])
        v = np.ascontiguousarray(v, dtype=np.complex128)
        self.K = len(terms)
        self.handle = ctypes.c_void_p()
        _check(lib().te_adjoint_create(self.K, arr, O.handle, _ptr(v), float(T), float(tol), int(m),
                                       float(checkpoint_interval), int(nodes_per_interval), ctypes.byref(self.handle)),
               "te_adjoint_create")

    def run(self, theta):
        th = np.ascontiguousarray(theta, dtype=np.float64)
        loss = ctypes.c_double()
        grad = np.zeros(self.K)
        _check(lib().te_adjoint_run(self.handle, _ptr(th), ctypes.byref(loss), _ptr(grad)), "te_adjoint_run")
        return loss.value, grad

    def forward(self, theta):
        th = np.ascontiguousarray(theta, dtype=np.float64)
        loss = ctypes.c_double()
        _check(lib().te_adjoint_forward(self.handle, _ptr(th), ctypes.byref(loss)), "te_adjoint_forward")
        return loss.value

    def stats(self):
        f, b = TeResult(), TeResult()
        launches, nodes = ctypes.c_int64(), ctypes.c_int64()
        _check(lib().te_adjoint_stats(self.handle, ctypes.byref(f), ctypes.byref(b), ctypes.byref(launches),
                                      ctypes.byref(nodes)), "te_adjoint_stats")
        return dict(forward_steps=f.n_steps, forward_status=f.status, forward_err=f.err, backward_steps=b.n_steps,
                    backward_status=b.status, backward_err=b.err, launches=launches.value, nodes=nodes.value)

    def phase_times(self):
        """Host wall time (ms) of the last call's phases."""
        ms = np.zeros(4)
        _check(lib().te_adjoint_phase_times(self.handle, _ptr(ms)), "te_adjoint_phase_times")
        return dict(theta_refresh=ms[0], forward=ms[1], costate=ms[2], bilinear=ms[3])

    def close(self):
        if self.handle:
            lib().te_adjoint_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def expectation_function():
    """torch.autograd.Function over te_adjoint_run: ``f.apply(theta, adjoint)``
    returns <psi(T)|O|psi(T)> as a 0-d float64 tensor whose backward is the
    adjoint gradient."""
    import torch

    class KrylovExpectation(torch.autograd.Function):
        @staticmethod
        def forward(ctx, theta, adjoint):
            loss, grad = adjoint.run(theta.detach().cpu().numpy().astype(np.float64))
            ctx.save_for_backward(torch.from_numpy(grad).to(theta.device, theta.dtype))
            return torch.tensor(loss, dtype=theta.dtype, device=theta.device)

        @staticmethod
        def backward(ctx, g):
            (grad,) = ctx.saved_tensors
            return g * grad, None

    return KrylovExpectation


class StopEvolution(Exception):
    """Raised by a callback observable to stop the evolution (requestStopException)."""


def evolve(H_coo, v, t, sampling_step, observables=(), exp_factor=1.0, tol=1e-6, m=40, fast_integration=False,
           trace=False, reorth=False, options=None):
    """One-call evolution with COO inputs, mirroring the oracle's signature.

    ``H_coo`` may also be a Matrix already on the device.  ``observables``:
    ("sparse", (row, col, val)), ("vector", o) or ("callback", fn).
    ``options``: {OPT_*: value} for te_evolver_set_option."""
    n = len(v)
    created = []  # matrices made here are released before returning, not whenever Python collects them
    H = H_coo if isinstance(H_coo, Matrix) else Matrix.from_coo(n, H_coo)
    if H is not H_coo:
        created.append(H)
    obs = []
    ev = None
    try:
        for kind, data in observables:
            if kind == "sparse" and not isinstance(data, Matrix):
                created.append(Matrix.from_coo(n, data))
                obs.append(("sparse", created[-1]))
            else:
                obs.append((kind, data))
        ev = Evolver(H, v, t, sampling_step, obs, exp_factor, tol, m, fast_integration, reorth)
        for opt, val in (options or {}).items():
            ev.set_option(opt, val)
        return ev.time_evolve(trace=trace)
    finally:
        if ev is not None:
            ev.close()
        for M in created:
            M.close()
