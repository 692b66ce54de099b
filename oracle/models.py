"""Model builders of the oracle (TEST INFRASTRUCTURE ONLY).

numpy restatement of TimeEvolver's basis enumeration (helper/Basis.cpp:37-121,
helper/Basis.cpp:131-182) and operator-to-matrix construction
(helper/hamiltonian.cpp:318-402, creation/annihilation operators
:410-456).  The tests use it to generate inputs for the oracle and to check
the product's C++ helpers bit for bit (same basis order, same COO arrays).

An operator term is ``(coef, ops, modes, caps)`` exactly like the
reference's ``opTerm`` (helper/hamiltonian.h:18-35): ``ops[0]`` is applied
first, +1 = creation, -1 = annihilation, cap 0 = no occupation limit.
"""
import numpy as np

EPS = np.finfo(np.float64).eps


# ----------------------------------------------------------------- basis

def basis(N, K, nb_qudits=0, capacity=0, quant=1):
    """Occupation vectors in the order of helper/Basis.cpp:37-121.

    The enumeration appends, mode by mode from K-1 down to 1, every allowed
    non-zero occupation of that mode to each state found so far (the write
    index is never reset, so earlier states keep their place); mode 0 takes
    the missing particles last.
    """
    old = np.zeros((1, K), dtype=np.int64)
    for k in range(K, 1, -1):
        occ = old.sum(axis=1)
        if k > K - nb_qudits:
            upper = np.minimum(N - occ, capacity)
        else:
            upper = N - occ
        counts = np.where(upper >= quant, (upper - quant) // quant + 1, 0)
        rep = np.repeat(np.arange(len(old)), counts)
        new = old[rep].copy()
        # occupation values quant, 2 quant, ... per parent, in order
        starts = np.cumsum(counts) - counts
        pos = np.arange(len(rep)) - np.repeat(starts, counts)
        new[:, k - 1] = quant * (pos + 1)
        old = np.concatenate([old, new], axis=0)
    missing = N - old.sum(axis=1)
    keep = np.ones(len(old), dtype=bool) if K != nb_qudits else (missing <= capacity)
    out = old[keep].copy()
    out[:, 0] = missing[keep]
    return out


def tensor_basis(N1, K1, N2, K2, C2):
    """helper/Basis.cpp:131-182: first basis index major, second minor."""
    b1 = basis(N1, K1, 0, 0)
    b2 = basis(N2, K2, K2, C2)
    if len(b2) == 0:
        return b1
    left = np.repeat(b1, len(b2), axis=0)
    right = np.tile(b2, (len(b1), 1))
    return np.concatenate([left, right], axis=1)


# ---------------------------------------------------------- operator terms

def lin_interaction(a, b, ca, cb, conjugate, cof):
    """helper/hamiltonian.cpp:43-65: a_a^dag a_b (conjugate: a_b^dag a_a)."""
    if not conjugate:
        return (complex(cof), [-1, 1], [b, a], [cb, ca])
    return (complex(cof), [-1, 1], [a, b], [ca, cb])


def number_operator(mode, cof):
    """helper/hamiltonian.cpp:73-85."""
    return (complex(cof), [-1, 1], [mode, mode], [0, 0])


def four_point_a(a, b, c, d, ca, cb, cc, cd, cof):
    """helper/hamiltonian.cpp:100-119: a_a^dag a_b a_c^dag a_d."""
    return (complex(cof), [-1, 1, -1, 1], [d, c, b, a], [cd, cc, cb, ca])


def four_point_b(a, b, c, d, ca, cb, cc, cd, cof):
    """helper/hamiltonian.cpp:134-153."""
    return (complex(cof), [-1, -1, 1, 1], [d, c, b, a], [cd, cc, cb, ca])


def four_point_c(a, b, c, d, ca, cb, cc, cd, cof):
    """helper/hamiltonian.cpp:168-187."""
    return (complex(cof), [1, 1, -1, -1], [d, c, b, a], [cd, cc, cb, ca])


def kinetic_terms(modes, gap):
    """helper/hamiltonian.cpp:11-31."""
    return [(complex(gap), [-1, 1], [m, m], [0, 0]) for m in modes]


# ------------------------------------------------------------ matrix build

def _keys(states, base):
    w = base ** np.arange(states.shape[1], dtype=np.int64)
    return states @ w


def create_matrix(terms, states):
    """COO (row, col, val) of sum(terms) in the basis ``states``.

    Matches helper/hamiltonian.cpp:318-402: per row, contributions are summed
    per column in term order (std::map), entries with |v| < DBL_EPSILON are
    dropped, rows ascend and columns ascend within a row.  Contributions whose
    target is not in the basis are skipped; zero contributions cannot change a
    non-zero sum and are dropped before summation.
    """
    n, K = states.shape
    base = int(states.max()) + 8
    assert base ** K < 2 ** 62, "occupation key would overflow"
    skeys = _keys(states, base)
    order = np.argsort(skeys, kind="stable")
    sorted_keys = skeys[order]
    contrib = []
    for coef, ops, modes, caps in terms:
        st = states.copy()
        amp = np.ones(n, dtype=np.float64)
        alive = np.ones(n, dtype=bool)
        for op, md, cap in zip(ops, modes, caps):
            occ = st[:, md]
            if op == 1:
                ok = alive if cap == 0 else alive & (occ + 1 <= cap)
                amp = np.where(ok, amp * np.sqrt(occ + 1.0), amp)
                st[:, md] = np.where(ok, occ + 1, occ)
                alive = ok
            else:
                ok = alive & (occ > 0)
                amp = np.where(ok, amp * np.sqrt(occ.astype(np.float64)), amp)
                st[:, md] = np.where(ok, occ - 1, occ)
                alive = ok
        tk = _keys(st, base)
        pos = np.searchsorted(sorted_keys, tk)
        pos = np.minimum(pos, n - 1)
        found = alive & (sorted_keys[pos] == tk)
        rows = np.nonzero(found)[0]
        cols = order[pos[found]]
        # coef * (1 * prod sqrt) -- complex times real, as std::complex does
        re = amp[found] * coef.real
        im = amp[found] * coef.imag
        contrib.append((rows, cols, re, im))
    allkeys = np.concatenate([r * n + c for r, c, _, _ in contrib]) if contrib else np.zeros(0, np.int64)
    uniq, inv = np.unique(allkeys, return_inverse=True)
    acc_re = np.zeros(len(uniq))
    acc_im = np.zeros(len(uniq))
    off = 0
    for r, c, re, im in contrib:
        sl = inv[off:off + len(r)]
        acc_re[sl] += re  # slots are distinct within one term
        acc_im[sl] += im
        off += len(r)
    keep = np.hypot(acc_re, acc_im) >= EPS
    uniq = uniq[keep]
    row = uniq // n
    col = uniq % n
    val = acc_re[keep] + 1j * acc_im[keep]
    return row.astype(np.int64), col.astype(np.int64), val.astype(np.complex128)


def number_operator_observables(states):
    """helper/hamiltonian.cpp:289-301: one diagonal n_i matrix per mode."""
    return [create_matrix([number_operator(i, 1.0)], states) for i in range(states.shape[1])]


def index_of(states, occ):
    hits = np.nonzero((states == np.asarray(occ)).all(axis=1))[0]
    return int(hits[0])


# ---------------------------------------------------------- model recipes

def bose_hubbard_terms(L, J, U, mu=0.0):
    """Open-chain Bose-Hubbard with the reference's helpers.

    Hopping -J_b (a_b^dag a_{b+1} + h.c.) per bond b (J scalar or per-bond
    list), on-site U/2 n(n-1) = U/2 (n^2 - n) via createFourPointA(i,i,i,i)
    and createNumberOperator(i, -U/2), optional -mu n_i.
    Order: all bonds' hops, then per site (four-point, number, chemical).
    """
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


def bose_hubbard(L, N, J, U, mu=0.0):
    states = basis(N, L, 0, 0)
    return states, create_matrix(bose_hubbard_terms(L, J, U, mu), states)


def _sym_break(a, b):
    """example/exampleHamiltonian.cpp:104-110."""
    c = np.fmod(np.sqrt(2.0) * float(a) ** 3 + np.sqrt(7.0) * float(b) ** 5, 1.0)
    if c < 0.5:
        c -= 1.0
    return c


def black_hole_terms(N0, Nm, DeltaN, K, C=1, C0=1.0, Cm=1.0, cgap1=1.0, cgap2=1.0):
    """example/exampleHamiltonian.cpp:27-56 (createSimplifiedHamiltonian) with
    Q1 = Q2 = K, as called by example/main.cpp:84-86."""
    Q1 = Q2 = K
    sq = np.sqrt(float(N0))
    ham = []
    for i in range(2, Q1 + 2):
        ham.append(number_operator(i, cgap1 * sq))
    for i in range(2 + Q1, Q1 + Q2 + 2):
        ham.append(number_operator(i, cgap2 * sq))
    ham.append(lin_interaction(0, 1, 0, 0, True, C0))
    ham.append(lin_interaction(0, 1, 0, 0, False, C0))
    for i in range(2, 2 + Q1):
        ham.append(four_point_a(0, 0, i, i, 0, 0, C, C, -sq * cgap1 / N0))
    for i in range(2 + Q1, 2 + Q1 + Q2):
        ham.append(four_point_a(0, 0, i, i, 0, 0, C, C, -sq * cgap2 / (N0 - DeltaN)))
    # simplifiedSphericalInteraction (:58-102)
    for m in range(2, Q1 + Q2 + 2):
        for M in range(2, Q1 + Q2 + 2):
            coeff = 0.0
            if m <= 1 + Q1 and M > Q1 + 1:
                coeff = _sym_break(m, M) * Cm
            elif ((m <= Q1 + 1 and M <= 1 + Q1) or (m > 1 + Q1 and M > 1 + Q1)) and m < M:
                coeff = _sym_break(m, M) * Cm
            if coeff != 0:
                ham.append((complex(coeff), [-1, 1], [m, M], [C, C]))
                ham.append((complex(coeff), [-1, 1], [M, m], [C, C]))
    return ham


def black_hole(N0=20, Nm=2, K=4, C=1, DeltaN=12.0, C0=1.0, Cm=1.0):
    """example/main.cpp:84-108: tensorBasis(N0, 2, Nm, 2K, C), initial state
    (N0, 0, 1 x min(K, Nm), 0...) (exampleHamiltonian.cpp:116-138)."""
    states = tensor_basis(N0, 2, Nm, 2 * K, C)
    H = create_matrix(black_hole_terms(N0, Nm, DeltaN, K, C, C0, Cm), states)
    init = [N0, 0] + [1] * min(K, Nm) + [0] * (2 * K - min(K, Nm))
    return states, H, index_of(states, init)


def simple_example(N0=200, E1=1.0, E2=2.0, lam=1.0):
    """example/simpleExample.cpp:21-67: two coupled oscillators."""
    states = basis(N0, 2, 0, 0)
    terms = [number_operator(0, E1), number_operator(1, E2),
             lin_interaction(0, 1, 0, 0, False, lam), lin_interaction(0, 1, 0, 0, True, lam)]
    return states, create_matrix(terms, states), index_of(states, [N0, 0])
