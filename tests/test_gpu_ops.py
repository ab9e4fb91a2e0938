"""OPS slots of the CUDA backend against the reference backends' semantics
(app/app_ccs.c, app/app_lapack.c, src/ops_multi_vec.c), restated in numpy."""
import ctypes

import numpy as np
import pytest

from gcge_gb300 import problems as P

pytestmark = pytest.mark.gpu


@pytest.fixture()
def ops(gpu_lib):
    o = gpu_lib.CudaOps()
    yield o
    o.close()


def setup(ops, n1=20, n2=13, ncx=7, ncy=6, seed=0):
    A = P.laplace2d(n1, n2)
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((A.n, ncx))
    Y = rng.standard_normal((A.n, ncy))
    hA = ops.mat(A)
    return A, A.to_scipy(), X, Y, hA, ops.multivec(hA, ncx, X), ops.multivec(hA, ncy, Y)


def test_mat_dot_multivec_and_null_copy(ops):
    A, As, X, Y, hA, x, y = setup(ops)
    ops.mat_dot(hA, x, y, (2, 1), (6, 5))
    Yr = Y.copy()
    Yr[:, 1:5] = As @ X[:, 2:6]
    np.testing.assert_allclose(ops.download(y, 0, 6), Yr, rtol=0, atol=1e-13)
    ops.mat_dot(None, x, y, (0, 0), (2, 2))                    # mat NULL -> copy
    Yr[:, 0:2] = X[:, 0:2]
    assert np.array_equal(ops.download(y, 0, 6), Yr)


def test_nonsymmetric_ccs_is_y_equals_a_x(ops, gpu_lib):
    """CCS input is A by columns: y = A x, not A^T x (app/app_ccs.c:120-131)."""
    rng = np.random.default_rng(1)
    import scipy.sparse as sp
    M = sp.random(50, 50, density=0.1, random_state=2, format="csc") + sp.eye(50, format="csc")
    M.sort_indices()
    # CCS arrays handed over as (j_col, i_row, data)
    csr_like = P.CSRMatrix(50, M.indptr.astype(np.int32), M.indices.astype(np.int32), M.data)
    h = ops.mat(csr_like)
    X = rng.standard_normal((50, 3))
    x = ops.multivec(h, 3, X)
    y = ops.multivec(h, 3)
    ops.mat_dot(h, x, y, (0, 0), (3, 3))
    np.testing.assert_allclose(ops.download(y, 0, 3), M @ X, rtol=0, atol=1e-12)


def test_ccs_upload_edge_cases(ops, gpu_lib):
    """The device-side CCS -> CSR -> SELL pipeline: unsorted row indices within
    columns, duplicate entries (summed, as y = A x sums them), empty rows and
    columns, rows longer than a slice is wide elsewhere, n not a multiple of 32;
    and an out-of-range row index is rejected with an error, not a fault."""
    import ctypes
    rng = np.random.default_rng(4)
    n = 77
    cols = []
    for j in range(n):
        if j % 11 == 5:
            cols.append(([], []))                      # empty column
            continue
        k = rng.integers(1, 6)
        rows = list(rng.choice(n, size=k, replace=False))
        if j % 7 == 0:
            rows.append(rows[0])                       # duplicate (r, j)
        rows = [r for r in rows if r % 13 != 3]        # rows 3, 16, ... stay empty
        if j == 40:
            rows += list(range(0, n, 2))               # one long column -> long rows? (columns)
        rng.shuffle(rows)                              # unsorted within the column
        cols.append((rows, list(rng.standard_normal(len(rows)))))
    rows = [r for r in range(n) if r % 13 != 3]
    cols[9] = (rows, list(rng.standard_normal(len(rows))))  # a dense column -> long rows
    indptr = np.zeros(n + 1, dtype=np.int32)
    ind, val = [], []
    for j, (rr, vv) in enumerate(cols):
        ind += [int(r) for r in rr]
        val += [float(v) for v in vv]
        indptr[j + 1] = len(ind)
    ind = np.array(ind, dtype=np.int32)
    val = np.array(val)
    dense = np.zeros((n, n))
    for j in range(n):
        for e in range(indptr[j], indptr[j + 1]):
            dense[ind[e], j] += val[e]
    h = ops.mat(P.CSRMatrix(n, indptr, ind, val))
    X = rng.standard_normal((n, 5))
    x = ops.multivec(h, 5, X)
    y = ops.multivec(h, 5)
    ops.mat_dot(h, x, y, (0, 0), (5, 5))
    np.testing.assert_allclose(ops.download(y, 0, 5), dense @ X, rtol=0, atol=1e-12)
    bad = ind.copy()
    bad[3] = n + 5
    hb = ctypes.c_void_p()
    st = gpu_lib.load().CUDA_MatCreateFromCCS(ctypes.byref(hb), ctypes.c_int(n), ctypes.c_int(n),
                                              indptr.ctypes.data_as(ctypes.c_void_p),
                                              bad.ctypes.data_as(ctypes.c_void_p),
                                              val.ctypes.data_as(ctypes.c_void_p))
    assert st == gpu_lib.GCGE_ERR_ARG
    # the library still works afterwards
    ops.mat_dot(h, x, y, (0, 0), (5, 5))
    np.testing.assert_allclose(ops.download(y, 0, 5), dense @ X, rtol=0, atol=1e-12)


@pytest.mark.parametrize("alpha,beta,usex", [(2.0, -1.0, True), (0.5, 0.0, True), (0.0, 3.0, False),
                                             (1.0, 1.0, True)])
def test_axpby(ops, alpha, beta, usex):
    A, As, X, Y, hA, x, y = setup(ops)
    ops.axpby(alpha, x if usex else None, beta, y, (1, 2), (4, 5))
    Yr = Y.copy()
    Yr[:, 2:5] = beta * Y[:, 2:5] + (alpha * X[:, 1:4] if usex else 0.0)
    np.testing.assert_allclose(ops.download(y, 0, 6), Yr, rtol=0, atol=1e-14)


def test_linear_comb_variants(ops):
    A, As, X, Y, hA, x, y = setup(ops)
    rng = np.random.default_rng(5)
    C = rng.standard_normal((9, 4))   # ldc = 9 > k = 5
    ops.linear_comb(x, y, (1, 1), (6, 5), coef=C, ldc=9)                   # beta NULL: Y = X C
    Yr = Y.copy()
    Yr[:, 1:5] = X[:, 1:6] @ C[:5, :]
    np.testing.assert_allclose(ops.download(y, 0, 6), Yr, rtol=0, atol=1e-13)
    beta = np.array([2.0, -1.0, 0.0, 0.5])
    ops.linear_comb(x, y, (0, 2), (5, 6), coef=C, ldc=9, beta=beta, incb=1)
    Yr[:, 2:6] = X[:, 0:5] @ C[:5, :] + Yr[:, 2:6] * beta
    np.testing.assert_allclose(ops.download(y, 0, 6), Yr, rtol=0, atol=1e-13)
    ops.linear_comb(None, y, (0, 0), (3, 3), beta=np.array([0.25]), incb=0)  # scale only
    Yr[:, 0:3] *= 0.25
    np.testing.assert_allclose(ops.download(y, 0, 6), Yr, rtol=0, atol=1e-13)
    ops.linear_comb(None, y, (0, 0), (3, 3))                                # no x, no beta: no-op
    np.testing.assert_allclose(ops.download(y, 0, 6), Yr, rtol=0, atol=1e-13)


def test_inner_products_N_S_D(ops):
    A, As, X, Y, hA, x, y = setup(ops)
    ip = ops.inner_prod("N", x, y, (1, 0), (7, 4), ldip=8)
    np.testing.assert_allclose(ip[:6], X[:, 1:7].T @ Y[:, 0:4], rtol=1e-13, atol=1e-12)
    s = ops.inner_prod("S", x, x, (2, 2), (6, 6))
    G = X[:, 2:6].T @ X[:, 2:6]
    np.testing.assert_allclose(s, G, rtol=1e-13, atol=1e-12)
    assert np.array_equal(s, s.T)
    d = ops.inner_prod("D", x, y, (0, 1), (5, 6))
    np.testing.assert_allclose(d, np.einsum("ij,ij->j", X[:, 0:5], Y[:, 1:6]), rtol=1e-13, atol=1e-12)


@pytest.mark.parametrize("mode", ["N", "T"])
@pytest.mark.parametrize("with_a", [True, False])
def test_qtap(ops, mode, with_a):
    A, As, X, Y, hA, x, y = setup(ops)
    ws = ops.multivec(hA, 5)
    q = ops.qtap("S", mode, x, hA if with_a else None, y, (1, 2), (6, 5), ws)
    AP = (As @ Y[:, 2:5]) if with_a else Y[:, 2:5]
    ref = X[:, 1:6].T @ AP
    np.testing.assert_allclose(q, ref.T if mode == "T" else ref, rtol=1e-12, atol=1e-11)


def test_random_fill_in_unit_interval(ops):
    A, As, X, Y, hA, x, y = setup(ops)
    ops.set_random(y, 1, 4)
    v = ops.download(y, 0, 6)
    assert np.all((v[:, 1:4] >= 0) & (v[:, 1:4] < 1)) and abs(v[:, 1:4].mean() - 0.5) < 0.05
    np.testing.assert_array_equal(v[:, [0, 4, 5]], Y[:, [0, 4, 5]])


def test_bad_handles_and_ranges_report_errors(ops, gpu_lib):
    A, As, X, Y, hA, x, y = setup(ops)
    with pytest.raises(gpu_lib.GCGEError):
        ops.axpby(1.0, x, 1.0, y, (0, 0), (9, 9))       # out of range
    with pytest.raises(gpu_lib.GCGEError):
        ops.mat_dot(hA, x, y, (0, 0), (2, 3))            # mismatched ranges


def test_mat_axpby_union_pattern(gpu_lib):
    """CUDA_MatAxpby (the OPS MatAxpby slot, src/ops.h:52): Y = alpha X + beta Y
    for matrices with different patterns, checked through MatDotMultiVec
    against scipy; X == Y scales in place."""
    import scipy.sparse as sp
    G = gpu_lib
    n = 3000
    X = P.laplace2d(60, 50)
    Y = P.diag_matrix(0.5 + P.splitmix_uniform(5, n, 0))
    Xs, Ys = X.to_scipy(), Y.to_scipy()
    rng = np.random.default_rng(7)
    v = rng.standard_normal((n, 5))
    ops = G.CudaOps()
    try:
        hX, hY = ops.mat(X), ops.mat(Y)
        ops.mat_axpby(0.75, hX, -2.0, hY)
        nnz = ctypes.c_longlong()
        G.load().CUDA_MatNnz(hY, ctypes.byref(nnz))
        assert nnz.value == (0.75 * Xs - 2.0 * Ys).nnz
        hv = ops.multivec(hY, 5, v)
        hw = ops.multivec(hY, 5)
        ops.mat_dot(hY, hv, hw, (0, 0), (5, 5))
        np.testing.assert_allclose(ops.download(hw, 0, 5), (0.75 * Xs - 2.0 * Ys) @ v,
                                   rtol=1e-14, atol=1e-13)
        ops.mat_axpby(1.5, hY, 0.5, hY)   # Y = 2 Y
        ops.mat_dot(hY, hv, hw, (0, 0), (5, 5))
        np.testing.assert_allclose(ops.download(hw, 0, 5), 2.0 * ((0.75 * Xs - 2.0 * Ys) @ v),
                                   rtol=1e-14, atol=1e-13)
        assert ops.ptr.contents.MatAxpby is None   # the slot stays NULL, as in app_ccs
    finally:
        ops.close()
