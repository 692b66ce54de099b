"""Model helpers: bases and operator matrices through libtimeevolver.so.

Python view of the C++ basis / Hamiltonian helpers (include/te_model.h), which
keep the reference's basis order (helper/Basis.cpp:37-121) and matrix
construction (helper/hamiltonian.cpp:318-402).  Operator terms are
``(coef, ops, modes, caps)`` exactly like the reference's opTerm: ops[0]
acts first, +1 creation, -1 annihilation, cap 0 = unbounded mode.
"""
import ctypes
import os

import numpy as np

import importlib

_build = importlib.import_module(__package__ + ".build")

_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_build.LIB_HOST):
            raise RuntimeError("libtimeevolver.so is missing (%s): build the package first" % _build.LIB_HOST)
        L = ctypes.CDLL(_build.LIB_HOST)
        P, I, I64, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_double
        sig = {
            "te_basis_create": (I, [I, I, I, I, I, P]),
            "te_tensor_basis_create": (I, [I, I, I, I, I, P]),
            "te_basis_destroy": (I, [P]),
            "te_basis_shape": (I, [P, P, P]),
            "te_basis_elements": (I, [P, P]),
            "te_basis_index": (I64, [P, P]),
            "te_operator_create": (I, [P]),
            "te_operator_destroy": (I, [P]),
            "te_operator_add_term": (I, [P, D, D, I, P, P, P]),
            "te_operator_build": (I, [P, P, P]),
            "te_operator_coo": (I, [P, P, P, P]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class Basis:
    """basis(N, K, nbQudits, capacity, quant) or tensorBasis(N1, K1, N2, K2, C2)."""

    def __init__(self, N, K, nb_qudits=0, capacity=0, quant=1, tensor=None):
        self.h = ctypes.c_void_p()
        if tensor is None:
            rc = lib().te_basis_create(N, K, nb_qudits, capacity, quant, ctypes.byref(self.h))
        else:
            rc = lib().te_tensor_basis_create(*tensor, ctypes.byref(self.h))
        if rc != 0:
            raise ValueError("invalid basis parameters")
        n, k = ctypes.c_int64(), ctypes.c_int()
        lib().te_basis_shape(self.h, ctypes.byref(n), ctypes.byref(k))
        self.size, self.modes = n.value, k.value

    @classmethod
    def tensor(cls, N1, K1, N2, K2, C2):
        return cls(0, 1, tensor=(N1, K1, N2, K2, C2))

    def elements(self):
        out = np.zeros((self.size, self.modes), dtype=np.int32)
        lib().te_basis_elements(self.h, _p(out))
        return out

    def index(self, occupations):
        occ = np.ascontiguousarray(occupations, dtype=np.int32)
        return int(lib().te_basis_index(self.h, _p(occ)))

    def __len__(self):
        return self.size

    def __del__(self):
        try:
            if self.h:
                lib().te_basis_destroy(self.h)
        except Exception:
            pass


def operator_matrix(terms, basis):
    """COO (row, col, val) of sum(terms) in ``basis``."""
    op = ctypes.c_void_p()
    lib().te_operator_create(ctypes.byref(op))
    try:
        for coef, ops, modes, caps in terms:
            c = complex(coef)
            a = np.ascontiguousarray(ops, dtype=np.int32)
            m = np.ascontiguousarray(modes, dtype=np.int32)
            k = np.ascontiguousarray(caps, dtype=np.int32)
            if lib().te_operator_add_term(op, c.real, c.imag, len(a), _p(a), _p(m), _p(k)) != 0:
                raise ValueError("invalid operator term")
        nnz = ctypes.c_int64()
        if lib().te_operator_build(op, basis.h, ctypes.byref(nnz)) != 0:
            raise ValueError("operator does not fit the basis")
        rows = np.zeros(nnz.value, dtype=np.uint64)
        cols = np.zeros(nnz.value, dtype=np.uint64)
        vals = np.zeros(nnz.value, dtype=np.complex128)
        lib().te_operator_coo(op, _p(rows), _p(cols), _p(vals))
        return rows.astype(np.int64), cols.astype(np.int64), vals
    finally:
        lib().te_operator_destroy(op)


# opTerm constructors (helper/hamiltonian.cpp:43-231)
def lin_interaction(a, b, ca, cb, conjugate, cof):
    return (cof, [-1, 1], [a, b] if conjugate else [b, a], [ca, cb] if conjugate else [cb, ca])


def number_operator(mode, cof):
    return (cof, [-1, 1], [mode, mode], [0, 0])


def four_point_a(a, b, c, d, ca, cb, cc, cd, cof):
    return (cof, [-1, 1, -1, 1], [d, c, b, a], [cd, cc, cb, ca])


def number_operator_observables(basis):
    return [operator_matrix([number_operator(i, 1.0)], basis) for i in range(basis.modes)]


def bose_hubbard(L, N, J, U, mu=0.0):
    """Open-chain Bose-Hubbard with hopping -J_b (a_b^dag a_{b+1} + h.c.) and
    on-site U/2 n(n-1), as the reference's helpers express it: per bond the
    two linInteraction terms, then per site createFourPointA(i,i,i,i, U/2)
    and createNumberOperator(i, -U/2) (and -mu n_i).  Returns (basis, COO)."""
    Js = list(J) if np.ndim(J) else [J] * (L - 1)
    terms = []
    for b in range(L - 1):
        terms.append(lin_interaction(b, b + 1, 0, 0, False, -Js[b]))
        terms.append(lin_interaction(b, b + 1, 0, 0, True, -Js[b]))
    for i in range(L):
        terms.append(four_point_a(i, i, i, i, 0, 0, 0, 0, U / 2.0))
        terms.append(number_operator(i, -U / 2.0))
        if mu != 0.0:
            terms.append(number_operator(i, -mu))
    B = Basis(N, L, 0, 0)
    return B, operator_matrix(terms, B)


def bose_hubbard_terms(L, J, U, mu=0.0):
    """The terms of bose_hubbard (same order)."""
    Js = list(J) if np.ndim(J) else [J] * (L - 1)
    terms = []
    for b in range(L - 1):
        terms.append(lin_interaction(b, b + 1, 0, 0, False, -Js[b]))
        terms.append(lin_interaction(b, b + 1, 0, 0, True, -Js[b]))
    for i in range(L):
        terms.append(four_point_a(i, i, i, i, 0, 0, 0, 0, U / 2.0))
        terms.append(number_operator(i, -U / 2.0))
        if mu != 0.0:
            terms.append(number_operator(i, -mu))
    return terms


def bose_hubbard_device(L, N, J, U, mu=0.0):
    """bose_hubbard built on the GPU: returns (Matrix, dim); the basis and the
    entries equal the host builder's."""
    from . import Matrix
    return Matrix.from_terms_device(N, L, bose_hubbard_terms(L, J, U, mu))


def bose_hubbard_term_matrices(L, N):
    """Terms of H(theta) = sum_b J_b H_hop,b + U H_int for the adjoint:
    H_hop,b = -(a_b^dag a_{b+1} + h.c.) for the L-1 bonds, H_int = 1/2 sum_i
    n_i (n_i - 1), in the basis(N, L) order.  Returns (basis, [COO, ...])."""
    B = Basis(N, L, 0, 0)
    mats = []
    for b in range(L - 1):
        mats.append(operator_matrix([lin_interaction(b, b + 1, 0, 0, False, -1.0),
                                     lin_interaction(b, b + 1, 0, 0, True, -1.0)], B))
    inter = []
    for i in range(L):
        inter.append(four_point_a(i, i, i, i, 0, 0, 0, 0, 0.5))
        inter.append(number_operator(i, -0.5))
    mats.append(operator_matrix(inter, B))
    return B, mats
