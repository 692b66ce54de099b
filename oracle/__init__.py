"""CPU oracle for the Krylov evolution exp(-iHt)v (TEST INFRASTRUCTURE ONLY).

ctypes front-end of ``te_oracle.cpp`` (a C++ restatement of TimeEvolver's
krylovTimeEvolver) plus the numpy model builders in ``models.py``.  Only the
tests, ``__graft_entry__.smoke()`` and the benchmark's CPU-baseline leg use
this package; the product library never imports it.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

_lib = None


class OracleObs(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("nnz", ctypes.c_int64), ("row", ctypes.c_void_p),
                ("col", ctypes.c_void_p), ("val", ctypes.c_void_p), ("stop_at", ctypes.c_int64)]


class OracleResult(ctypes.Structure):
    _fields_ = [("err", ctypes.c_double), ("evolved_time", ctypes.c_double), ("num_samples", ctypes.c_int64),
                ("n_steps", ctypes.c_int64), ("dim", ctypes.c_int64), ("krylov_dim", ctypes.c_int64),
                ("status", ctypes.c_int32), ("nb_err_roundoff", ctypes.c_int32), ("nb_err_int", ctypes.c_int32),
                ("pad", ctypes.c_int32)]


class OracleStep(ctypes.Structure):
    _fields_ = [("t_now", ctypes.c_double), ("t_step", ctypes.c_double), ("err_step", ctypes.c_double),
                ("h", ctypes.c_double), ("m_eff", ctypes.c_int32), ("breakdown", ctypes.c_int32),
                ("code", ctypes.c_int32), ("n_integrals", ctypes.c_int32)]


OBS_SPARSE, OBS_VECTOR, OBS_STOP = 0, 1, 2


def build(force=False):
    """Compile liboracle.so with g++ (OpenMP, no FP contraction)."""
    src = os.path.join(HERE, "te_oracle.cpp")
    deps = [src, os.path.join(HERE, "te_oracle.h"), os.path.join(HERE, "te_quadrature.h")]
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= max(map(os.path.getmtime, deps)):
        return LIB_PATH
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-o", LIB_PATH, src]
    subprocess.check_call(cmd)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        I64, D, I = ctypes.c_int64, ctypes.c_double, ctypes.c_int
        L.oracle_evolve.argtypes = [I64, I64, P, P, P, P, D, D, D, D, I, I, I, I, P, P, P, P, P, I64, P, I]
        L.oracle_evolve.restype = I
        L.oracle_spmv.argtypes = [I64, I64, P, P, P, D, D, P, P]
        L.oracle_norm1.argtypes = [I64, I64, P, P]
        L.oracle_norm1.restype = D
        L.oracle_lanczos.argtypes = [I64, I64, P, P, P, P, D, D, I, P, P, P, P]
        L.oracle_krylov_eig.argtypes = [I, P, P, P]
        L.oracle_integrate_error.argtypes = [I, P, P, D, D, D, I, D, D, P]
        L.oracle_integrate_error.restype = D
        L.oracle_find_step.argtypes = [I, P, P, D, D, D, D, I, D, I, I, D, P, P, P, P]
        L.oracle_ts_test.argtypes = [I, D, D, D, D, P, P, P]
        L.oracle_ts_test.restype = D
        L.oracle_set_ts_max_level.argtypes = [I]
        L.oracle_set_ts_max_level.restype = None
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def _coo(H):
    row, col, val = H
    return (np.ascontiguousarray(row, dtype=np.int64), np.ascontiguousarray(col, dtype=np.int64),
            np.ascontiguousarray(val, dtype=np.complex128))


def evolve(H, v, t, sampling_step, observables=(), exp_factor=1.0, tol=1e-6, m=40, fast_integration=False,
           n_threads=0, trace=False, max_trace=100000, reorth=False):
    """Run the oracle evolution.  H is a COO triple (row, col, val) of size n.

    ``observables`` is a list of ("sparse", (row, col, val)), ("vector", o) or
    ("stop", sample_index).  Returns a dict with samples (n_obs x n_samples),
    state, err, evolved_time, num_samples, n_steps, krylov_dim, status and the
    optional per-step trace.
    """
    row, col, val = _coo(H)
    n = int(len(v))
    v = np.ascontiguousarray(v, dtype=np.complex128)
    keep = []
    obs_arr = (OracleObs * max(1, len(observables)))()
    n_real = 0
    for i, (kind, data) in enumerate(observables):
        o = obs_arr[i]
        if kind == "sparse":
            r, c, x = _coo(data)
            keep += [r, c, x]
            o.kind, o.nnz, o.row, o.col, o.val = OBS_SPARSE, len(x), r.ctypes.data, c.ctypes.data, x.ctypes.data
            n_real += 1
        elif kind == "vector":
            x = np.ascontiguousarray(data, dtype=np.complex128)
            keep.append(x)
            o.kind, o.val = OBS_VECTOR, x.ctypes.data
            n_real += 1
        elif kind == "stop":
            o.kind, o.stop_at = OBS_STOP, int(data)
        else:
            raise ValueError(kind)
    n_samples = int(np.floor(t / sampling_step)) + 1
    samples = np.zeros((max(1, n_real), n_samples))
    state = np.zeros(n, dtype=np.complex128)
    res = OracleResult()
    tr = (OracleStep * max_trace)() if trace else None
    ntr = ctypes.c_int64(0)
    rc = lib().oracle_evolve(n, len(val), _p(row), _p(col), _p(val), _p(v), t, sampling_step, exp_factor, tol, m,
                             int(fast_integration), int(reorth), len(observables), ctypes.addressof(obs_arr),
                             _p(samples),
                             _p(state), ctypes.byref(res), ctypes.addressof(tr) if tr is not None else None,
                             max_trace, ctypes.byref(ntr), n_threads)
    if rc != 0:
        raise RuntimeError("oracle_evolve failed with code %d" % rc)
    out = dict(samples=samples[:n_real], state=state, err=res.err, evolved_time=res.evolved_time,
               num_samples=res.num_samples, n_steps=res.n_steps, krylov_dim=res.krylov_dim, status=res.status,
               nb_err_roundoff=res.nb_err_roundoff, nb_err_int=res.nb_err_int)
    if trace:
        k = min(ntr.value, max_trace)
        out["trace"] = [dict(t_now=s.t_now, t_step=s.t_step, err_step=s.err_step, h=s.h, m_eff=s.m_eff,
                             breakdown=s.breakdown, code=s.code, n_integrals=s.n_integrals) for s in tr[:k]]
    return out


def spmv(H, x, alpha=1.0):
    row, col, val = _coo(H)
    x = np.ascontiguousarray(x, dtype=np.complex128)
    out = np.zeros_like(x)
    a = complex(alpha)
    lib().oracle_spmv(len(x), len(val), _p(row), _p(col), _p(val), a.real, a.imag, _p(x), _p(out))
    return out


def norm1(H, n):
    row, col, val = _coo(H)
    return lib().oracle_norm1(n, len(val), _p(col), _p(val))


def lanczos(H, v, m, tol_rate, exp_factor=1.0):
    row, col, val = _coo(H)
    n = len(v)
    v = np.ascontiguousarray(v, dtype=np.complex128)
    Hm = np.zeros((m, m), dtype=np.complex128, order="F")
    V = np.zeros((n, m), dtype=np.complex128, order="F")
    h = ctypes.c_double(0)
    mh = ctypes.c_int64(0)
    bd = lib().oracle_lanczos(n, len(val), _p(row), _p(col), _p(val), _p(v), exp_factor, tol_rate, m, _p(Hm),
                              _p(V), ctypes.byref(h), ctypes.byref(mh))
    return dict(H=Hm, V=V, h=h.value, m_hbd=mh.value, breakdown=bool(bd))


def krylov_eig(Hm):
    m = Hm.shape[0]
    Hf = np.asfortranarray(Hm, dtype=np.complex128)
    lam = np.zeros(m, dtype=np.complex128)
    Z = np.zeros((m, m), dtype=np.complex128, order="F")
    lib().oracle_krylov_eig(m, _p(Hf), _p(lam), _p(Z))
    return lam, Z


def integrate_error(lam, Z, h, a, b, method, tol_rate, tol):
    m = len(lam)
    lam = np.ascontiguousarray(lam, dtype=np.complex128)
    Zf = np.asfortranarray(Z, dtype=np.complex128)
    ok = ctypes.c_int(0)
    r = lib().oracle_integrate_error(m, _p(lam), _p(Zf), h, a, b, method, tol_rate, tol, ctypes.byref(ok))
    return r, bool(ok.value)


def find_step(lam, Z, h, tol_rate, t_suggest, t_max, numerical_error_estimate, increase, tol, n_substeps=50,
              fast_integration=False):
    m = len(lam)
    lam = np.ascontiguousarray(lam, dtype=np.complex128)
    Zf = np.asfortranarray(Z, dtype=np.complex128)
    ts = ctypes.c_double(0)
    es = ctypes.c_double(0)
    ni = ctypes.c_int(0)
    w = np.zeros(m, dtype=np.complex128)
    code = lib().oracle_find_step(m, _p(lam), _p(Zf), h, tol_rate, t_suggest, t_max, n_substeps,
                                  numerical_error_estimate, int(increase), int(fast_integration), tol,
                                  ctypes.byref(ts), _p(w), ctypes.byref(es), ctypes.byref(ni))
    return dict(code=code, t_step=ts.value, err_step=es.value, w=w, n_integrals=ni.value)


def ts_test(kind, p, a, b, tol):
    e = ctypes.c_double(0)
    l1 = ctypes.c_double(0)
    lv = ctypes.c_int(0)
    r = lib().oracle_ts_test(kind, p, a, b, tol, ctypes.byref(e), ctypes.byref(l1), ctypes.byref(lv))
    return r, e.value, l1.value, lv.value


def set_ts_max_level(level):
    """Last tanh-sinh level (2..8) of the oracle's later integrals (8 restores
    the default)."""
    lib().oracle_set_ts_max_level(int(level))


# ------------------------------------------------------------------------------
# The reference itself, compiled by ref_recipe.py into _ref/libteref.so where the
# reference tree is present (never on the GPU host): the restatement above is
# checked against it.

REF_LIB_PATH = os.path.join(HERE, "_ref", "libteref.so")
_ref = None


def build_ref(force=False):
    """Compile the reference's own core into _ref/libteref.so (None where the
    reference tree or numpy's OpenBLAS is missing)."""
    from oracle import ref_recipe as recipe
    return recipe.build_ref(force=force)


def ref_available():
    return os.path.exists(REF_LIB_PATH)


def ref_lib():
    global _ref
    if _ref is None:
        L = ctypes.CDLL(REF_LIB_PATH)
        P, I64, D, I = ctypes.c_void_p, ctypes.c_int64, ctypes.c_double, ctypes.c_int
        L.teref_evolve.argtypes = [I64, I64, P, P, P, P, D, D, D, D, I, I, I, P, P, P, P, P, P, I64, P, P, P]
        L.teref_evolve.restype = I
        _ref = L
    return _ref


def ref_evolve(H, v, t, sampling_step, observables=(), exp_factor=1.0, tol=1e-6, m=40, fast_integration=False):
    """The reference's own krylovTimeEvolver on the same inputs as evolve()
    (observables: ("sparse", coo) or ("vector", o)); returns the same keys
    (samples, state, err, evolved_time, num_samples, n_steps, krylov_dim,
    status)."""
    row, col, val = _coo(H)
    n = int(len(v))
    v = np.ascontiguousarray(v, dtype=np.complex128)
    k = len(observables)
    kinds = np.zeros(max(1, k), dtype=np.int32)
    nnzs = np.zeros(max(1, k), dtype=np.int64)
    rows, cols, vals = (ctypes.c_void_p * max(1, k))(), (ctypes.c_void_p * max(1, k))(), (ctypes.c_void_p * max(1, k))()
    keep = []
    for i, (kind, data) in enumerate(observables):
        if kind == "sparse":
            r, c, x = _coo(data)
            keep += [r, c, x]
            kinds[i], nnzs[i] = 0, len(x)
            rows[i], cols[i], vals[i] = r.ctypes.data, c.ctypes.data, x.ctypes.data
        elif kind == "vector":
            x = np.ascontiguousarray(data, dtype=np.complex128)
            keep.append(x)
            kinds[i], vals[i] = 1, x.ctypes.data
        else:
            raise ValueError(kind)
    cap = int(np.floor(t / sampling_step)) + 1
    samples = np.zeros((max(1, k), cap))
    state = np.zeros(n, dtype=np.complex128)
    scalars = np.zeros(2)
    counts = np.zeros(4, dtype=np.int64)
    rc = ref_lib().teref_evolve(n, len(val), _p(row), _p(col), _p(val), _p(v), t, sampling_step, exp_factor, tol, m,
                                int(fast_integration), k, _p(kinds), _p(nnzs), ctypes.addressof(rows),
                                ctypes.addressof(cols), ctypes.addressof(vals), _p(samples), cap, _p(state),
                                _p(scalars), _p(counts))
    if rc != 0:
        raise RuntimeError("teref_evolve failed with code %d" % rc)
    return dict(samples=samples[:k], state=state, err=scalars[0], evolved_time=scalars[1],
                num_samples=int(counts[0]), n_steps=int(counts[1]), krylov_dim=int(counts[2]), status=int(counts[3]))
