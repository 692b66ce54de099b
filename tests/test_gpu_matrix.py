"""Matrix upload (needs a GB300): the device conversion of large row-sorted
COO input, the host fallback for unsorted input, and the reference's 1-norm
(column sums of |a| in entry order, matrixDataTypes.cpp:67-79) in both."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 200_000
PER_ROW = 3  # 600k entries: above the device-conversion threshold of 2^18


def _coo(seed, sort_rows=True, real=False):
    rng = np.random.default_rng(seed)
    row = np.repeat(np.arange(N, dtype=np.int64), PER_ROW)
    col = rng.integers(0, N, size=len(row)).astype(np.int64)
    val = rng.standard_normal(len(row)) + (0 if real else 1j) * rng.standard_normal(len(row))
    if not sort_rows:
        p = rng.permutation(len(row))
        row, col, val = row[p], col[p], val[p]
    return row, col, val.astype(np.complex128)


def _reference_norm1(col, val):
    s = np.zeros(N)
    np.add.at(s, col, np.abs(val))  # sequential in entry order
    return s.max()


def _expected_csr(row, col, val):
    order = np.argsort(row, kind="stable")
    rp = np.zeros(N + 1, dtype=np.int64)
    np.add.at(rp, row + 1, 1)
    return np.cumsum(rp), col[order], val[order]


@pytest.mark.parametrize("sort_rows,copy_path", [(True, False), (True, True), (False, False)])
def test_coo_upload(te_gpu, sort_rows, copy_path, monkeypatch):
    """Row-sorted COO: read by a kernel straight from host memory where the
    device accesses pageable memory (Grace), else (TE_COO_COPY=1 here) copied
    first; unsorted COO: converted on the host."""
    if copy_path:
        monkeypatch.setenv("TE_COO_COPY", "1")
    row, col, val = _coo(1, sort_rows)
    M = te_gpu.Matrix(N, row, col, val)
    rp, ci, v = M.to_csr()
    rp0, ci0, v0 = _expected_csr(row, col, val)
    assert np.array_equal(rp, rp0) and np.array_equal(ci, ci0) and np.array_equal(v, v0)
    info = M.info()
    assert info["norm1"] == _reference_norm1(col, val)
    assert not info["real"] and not info["diagonal"]
    x = np.random.default_rng(2).standard_normal(N) + 0j
    y = np.zeros(N, dtype=np.complex128)
    np.add.at(y, row, val * x[col])
    assert np.max(np.abs(M.spmv(x) - y)) < 1e-12 * np.max(np.abs(y))


def test_coo_upload_real_and_diagonal(te_gpu):
    row, col, val = _coo(3, True, real=True)
    M = te_gpu.Matrix(N, row, col, val)
    assert M.info()["real"]
    d = np.arange(N, dtype=np.int64)
    D = te_gpu.Matrix(N, np.repeat(d, 2), np.repeat(d, 2), np.ones(2 * N, dtype=np.complex128))
    inf = D.info()
    assert inf["diagonal"] and inf["real"] and inf["norm1"] == 2.0


@pytest.mark.parametrize("copy_path", [False, True])
def test_coo_upload_rejects_out_of_range(te_gpu, copy_path, monkeypatch):
    if copy_path:
        monkeypatch.setenv("TE_COO_COPY", "1")
    row, col, val = _coo(4, True)
    col = col.copy()
    col[123_456] = N
    with pytest.raises(RuntimeError, match="entry 123456 out of range"):
        te_gpu.Matrix(N, row, col, val)
    row = row.copy()
    row[200_001] = N + 5
    with pytest.raises(RuntimeError, match="entry 123456 out of range"):
        te_gpu.Matrix(N, row, col, val)


@pytest.mark.parametrize("copy_path", [False, True])
def test_coo_upload_empty_rows(te_gpu, copy_path, monkeypatch):
    """Row pointers across empty rows, before the first and after the last
    stored row (the direct read derives them from the row boundaries)."""
    if copy_path:
        monkeypatch.setenv("TE_COO_COPY", "1")
    rng = np.random.default_rng(8)
    rows = np.sort(rng.choice(np.arange(5, N - 7), size=N // 3, replace=False))
    row = np.repeat(rows, 5).astype(np.int64)
    col = rng.integers(0, N, size=len(row)).astype(np.int64)
    val = (rng.standard_normal(len(row)) + 1j * rng.standard_normal(len(row))).astype(np.complex128)
    assert len(val) >= 1 << 18
    M = te_gpu.Matrix(N, row, col, val)
    rp, ci, v = M.to_csr()
    rp0, ci0, v0 = _expected_csr(row, col, val)
    assert np.array_equal(rp, rp0) and np.array_equal(ci, ci0) and np.array_equal(v, v0)


def _hub_matrix(n, hubs, hub_len, seed, complex_values=True):
    """A Hermitian matrix with a few 'hub' rows far longer than the rest."""
    rng = np.random.default_rng(seed)
    ent = {}
    for r in range(n):
        for c in rng.integers(0, n, size=4):
            ent[(r, int(c))] = ent.get((r, int(c)), 0) + rng.standard_normal() + (1j * rng.standard_normal()
                                                                                     if complex_values else 0)
    for h in hubs:
        for c in rng.choice(n, size=hub_len, replace=False):
            ent[(h, int(c))] = ent.get((h, int(c)), 0) + rng.standard_normal() + (1j * rng.standard_normal()
                                                                                    if complex_values else 0)
    herm = {}
    for (r, c), v in ent.items():
        herm[(r, c)] = herm.get((r, c), 0) + v / 2
        herm[(c, r)] = herm.get((c, r), 0) + np.conj(v) / 2
    keys = sorted(herm)
    row = np.array([k[0] for k in keys], dtype=np.int64)
    col = np.array([k[1] for k in keys], dtype=np.int64)
    val = np.array([herm[k] for k in keys], dtype=np.complex128)
    return row, col, val


@pytest.mark.parametrize("n,complex_values", [(6000, True), (6000, False), (40000, True)])
def test_long_rows_layout_and_evolution(te_gpu, oracle_lib, n, complex_values):
    """Rows far longer than the rest (3 hubs of 3000 entries among rows of ~8)
    are kept out of the SELL chunks and multiplied warp-per-row: no chunk
    padding, exact SpMV, an evolution within the parity bounds.  n = 40000
    exceeds the device-conversion threshold (the layout is built by kernels)."""
    row, col, val = _hub_matrix(n, [17, n // 2, n - 1], 3000, 11, complex_values)
    M = te_gpu.Matrix(n, row, col, val)
    lay = M.layout()
    assert lay["long_rows"] == 3
    assert lay["sell_slots"] <= 1.05 * (len(val) - lay["long_entries"]) + 32 * 64  # a few padded chunks at most
    rng = np.random.default_rng(2)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    y = np.zeros(n, dtype=np.complex128)
    np.add.at(y, row, val * x[col])
    assert np.max(np.abs(M.spmv(x) - y)) < 1e-12 * np.max(np.abs(y))
    v = x / np.linalg.norm(x)
    d = (np.arange(n), np.arange(n), rng.uniform(-1, 1, n).astype(np.complex128))
    gpu = te_gpu.evolve(M, v, 1.0, 0.25, [("sparse", d)], tol=1e-8, m=30)
    ref = oracle_lib.evolve((row, col, val), v, 1.0, 0.25, [("sparse", d)], tol=1e-8, m=30)
    assert gpu["status"] == ref["status"] and gpu["n_steps"] == ref["n_steps"]
    assert np.linalg.norm(gpu["state"] - ref["state"]) < 2e-8
    assert np.max(np.abs(gpu["samples"] - ref["samples"])) < 4e-8


def test_norm1_device_path_bit_identical(te_gpu):
    """The reference's 1-norm (entry-order column sums) for a row-sorted COO
    of 967 537 entries: computed on the device for a real matrix with
    symmetric |H| (rows sorted, every entry mirrored), on host threads once
    one entry breaks the symmetry -- bit-identical to the sequential sums
    either way."""
    from oracle import models
    states, H = models.bose_hubbard(10, 10, 1.0, 2.0)
    n = len(states)
    row, col = np.asarray(H[0], np.int64), np.asarray(H[1], np.int64)
    val = np.asarray(H[2], np.complex128)

    def seq_norm1(c, v):
        s = np.zeros(n)
        np.add.at(s, c, np.abs(v))  # sequential in entry order
        return s.max()

    M = te_gpu.Matrix(n, row, col, val)
    assert M.info()["norm1"] == seq_norm1(col, val)
    asym = val.copy()
    k = int(np.nonzero(row != col)[0][12345])
    asym[k] *= 1.0 + 2.0 ** -40  # (r, c) no longer mirrors (c, r)
    Ma = te_gpu.Matrix(n, row, col, asym)
    assert Ma.info()["norm1"] == seq_norm1(col, asym)


def _bh10():
    from oracle import models
    states, H = models.bose_hubbard(10, 10, 1.0, 2.0)
    return len(states), np.asarray(H[0], np.int64), np.asarray(H[1], np.int64), np.asarray(H[2], np.complex128)


def _wide_rows(n=1200, density=0.25, seed=9):
    """A Hermitian matrix with ~300 entries per row: the long-row threshold
    (32 x the mean) is too wide for the device sort's counters, so the device
    build orders the rows on the host."""
    rng = np.random.default_rng(seed)
    mask = np.triu(rng.random((n, n)) < density)
    mask = mask | mask.T
    A = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) * mask
    A = (A + A.conj().T) / 2
    row, col = np.nonzero(A)
    return n, row.astype(np.int64), col.astype(np.int64), A[row, col].astype(np.complex128)


@pytest.mark.parametrize("case", ["bh10", "hubs", "wide"])
def test_device_layout_identical_to_host_layout(te_gpu, case):
    """The SELL order built on the device (stable counting sort by length,
    long rows ordered by length on the host) equals the host's stable sort:
    the same matrix uploaded as a row-sorted COO (device build) and as a host
    CSR (host build) has the same layout and evolves to bit-identical
    results, whose reductions run in the permuted order."""
    if case == "bh10":
        n, row, col, val = _bh10()
    elif case == "wide":
        n, row, col, val = _wide_rows()
    else:
        n = 40000
        row, col, val = _hub_matrix(n, [17, n // 2, n - 1], 3000, 11, True)
    assert len(val) >= 1 << 18  # the device conversion
    rp = np.zeros(n + 1, dtype=np.int64)
    np.add.at(rp, row + 1, 1)
    rp = np.cumsum(rp)
    Md = te_gpu.Matrix(n, row, col, val)
    Mh = te_gpu.Matrix.from_csr(n, rp, col, val)
    assert Md.layout() == Mh.layout()
    if case == "hubs":
        assert Md.layout()["long_rows"] == 3
    assert Md.info()["norm1"] == Mh.info()["norm1"]
    rng = np.random.default_rng(5)
    v = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    v /= np.linalg.norm(v)
    d = (np.arange(n), np.arange(n), rng.uniform(-1, 1, n).astype(np.complex128))
    a = te_gpu.evolve(Md, v, 1.0, 0.25, [("sparse", d)], tol=1e-8, m=30)
    b = te_gpu.evolve(Mh, v, 1.0, 0.25, [("sparse", d)], tol=1e-8, m=30)
    assert a["n_steps"] == b["n_steps"] and a["status"] == b["status"]
    assert np.array_equal(a["state"], b["state"])
    assert np.array_equal(a["samples"], b["samples"])


def test_destroy_frees_the_fixed_point_form(te_gpu):
    """Destroying a matrix also frees its fixed-point form, column blocks
    included (forced here): device memory returns to where it was.  The
    hopping terms get Peierls phases (a complex Hermitian matrix, so int32
    limbs per slot rather than the real value dictionary)."""
    import torch
    n, row, col, val = _bh10()
    val = val * np.exp(0.3j * (row - col))
    rng = np.random.default_rng(6)
    v = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    v /= np.linalg.norm(v)
    d = (np.arange(n), np.arange(n), np.ones(n, dtype=np.complex128))
    free0 = None
    for it in range(4):  # the first round also loads the kernels
        M = te_gpu.Matrix(n, row, col, val)
        M.set_fixed_blocks(3)
        te_gpu.evolve(M, v, 0.5, 0.5, [("sparse", d)], tol=1e-8, m=30)
        assert M.fixed_layout()["state"] == 3
        M.close()
        torch.cuda.synchronize()
        if it == 0:
            free0 = torch.cuda.mem_get_info()[0]
    assert abs(torch.cuda.mem_get_info()[0] - free0) < 8 << 20


@pytest.mark.parametrize("copy_path", [False, True])
def test_coo_upload_rectangular(te_gpu, copy_path, monkeypatch):
    """A rectangular row-sorted COO (columns up to 2 N) through the device
    conversion: exact CSR, no SELL layout (square matrices only)."""
    if copy_path:
        monkeypatch.setenv("TE_COO_COPY", "1")
    rng = np.random.default_rng(10)
    row = np.repeat(np.arange(N, dtype=np.int64), PER_ROW)
    col = rng.integers(0, 2 * N, size=len(row)).astype(np.int64)
    val = (rng.standard_normal(len(row)) + 1j * rng.standard_normal(len(row))).astype(np.complex128)
    M = te_gpu.Matrix(N, row, col, val, n_cols=2 * N)
    rp, ci, v = M.to_csr()
    rp0, ci0, v0 = _expected_csr(row, col, val)
    assert np.array_equal(rp, rp0) and np.array_equal(ci, ci0) and np.array_equal(v, v0)
    inf = M.info()
    assert inf["n_rows"] == N and inf["n_cols"] == 2 * N
    colsum = np.zeros(2 * N)
    np.add.at(colsum, col, np.abs(val))  # the reference's entry-order column sums
    assert inf["norm1"] == colsum.max()
    with pytest.raises(RuntimeError, match="square"):
        M.layout()


def _giant_matrix(n, hubs, hub_len, seed, complex_values):
    """Random Hermitian rows of ~8 entries plus a few rows (and, mirrored,
    columns) of hub_len entries, built with numpy (n up to a few 10^5)."""
    rng = np.random.default_rng(seed)
    r = np.repeat(np.arange(n), 4)
    c = rng.integers(0, n, size=4 * n)
    rows = [r] + [np.full(hub_len, h) for h in hubs]
    cols = [c] + [rng.choice(n, size=hub_len, replace=False) for _ in hubs]
    row, col = np.concatenate(rows), np.concatenate(cols)
    val = rng.standard_normal(len(row)) + (1j * rng.standard_normal(len(row)) if complex_values else 0.0)
    # H = (A + A^H) / 2, duplicates summed, row-sorted
    R = np.concatenate([row, col])
    C = np.concatenate([col, row])
    V = np.concatenate([val, np.conj(val)]) / 2
    key = R * n + C
    uk, inv = np.unique(key, return_inverse=True)
    acc = np.zeros(len(uk), dtype=np.complex128)
    np.add.at(acc, inv, V)
    return (uk // n).astype(np.int64), (uk % n).astype(np.int64), acc


@pytest.mark.parametrize("complex_values", [False, True])
def test_giant_rows_split_into_merge_path_segments(te_gpu, oracle_lib, complex_values):
    """Rows of 120000 entries among rows of ~8 (dim 200000): each is split
    into merge-path segments (one warp each, partial sums added in segment
    order by the last warp), next to warp-per-row long rows.  The SpMV
    (allocating and allocation-free entry points, repeated: the arrival counts
    reset themselves) matches the COO product; evolutions on the fixed-point
    and the FP64 passes match the oracle and repeat bit for bit."""
    torch = pytest.importorskip("torch")
    import ctypes
    n = 200_000
    row, col, val = _giant_matrix(n, [5, n // 3, n - 2], 120_000, 21, complex_values)
    M = te_gpu.Matrix(n, row, col, val)
    seg = M.long_segments()
    assert seg["segment_items"] >= 2048
    assert seg["split_rows"] >= 3 and seg["segments"] > 3 * 50
    rng = np.random.default_rng(4)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    y = np.zeros(n, dtype=np.complex128)
    np.add.at(y, row, val * x[col])
    scale = np.max(np.abs(y))
    for _ in range(2):
        assert np.max(np.abs(M.spmv(x) - y)) < 1e-12 * scale
    xd = torch.from_numpy(x.view(np.float64).copy()).cuda()
    for _ in range(2):
        yd = torch.full_like(xd, float("nan"))
        rc = te_gpu.lib().te_matrix_spmv_noalloc(M.handle, 1.0, 0.0, ctypes.c_void_p(xd.data_ptr()),
                                                 ctypes.c_void_p(yd.data_ptr()), None)
        assert rc == 0, te_gpu.lib().te_last_error()
        torch.cuda.synchronize()
        assert np.max(np.abs(yd.cpu().numpy().view(np.complex128) - y)) < 1e-12 * scale
    v = x / np.linalg.norm(x)
    d = (np.arange(n), np.arange(n), rng.uniform(-1, 1, n).astype(np.complex128))
    ref = oracle_lib.evolve((row, col, val), v, 0.5, 0.25, [("sparse", d)], tol=1e-8, m=30)
    for fixed in (1, 0):
        runs = [te_gpu.evolve(M, v, 0.5, 0.25, [("sparse", d)], tol=1e-8, m=30,
                              options={te_gpu.OPT_FIXED_SPMV: fixed}) for _ in range(2)]
        assert np.array_equal(runs[0]["state"], runs[1]["state"])
        gpu = runs[0]
        assert gpu["status"] == ref["status"] and gpu["n_steps"] == ref["n_steps"]
        assert np.linalg.norm(gpu["state"] - ref["state"]) < 2e-8
        assert np.max(np.abs(gpu["samples"] - ref["samples"])) < 4e-8
