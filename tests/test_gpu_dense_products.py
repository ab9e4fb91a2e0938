"""FP64-accurate tensor-core digit products (ozaki.cu) against extended-precision
host arithmetic, next to the plain FP64 kernels they replace in the mixed
solve: the Gram product Q^T P (DenseMatQtAP with matA = NULL,
app/app_lapack.c:64-183) and the linear combination alpha X C + Y diag(beta)
(MultiVecLinearComb, app/app_lapack.c:463-534).

Error measure: max |result - exact| / max (|Q|^T |P|) (resp. the absolute
value sum of the linear combination), the scale FP64 rounding errors are
measured against.  The exact value is computed in numpy long double."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

EXT = np.longdouble


def _gram_exact(Q, P):
    return Q.astype(EXT).T @ P.astype(EXT)


def _rel_err(got, exact, scale):
    return float(np.max(np.abs(got.astype(EXT) - exact)) / np.max(scale))


@pytest.mark.parametrize("n,m,w", [(20011, 37, 20), (4096, 180, 20), (1000, 7, 3), (64, 64, 24),
                                   (129, 5, 40), (3000, 100, 16)])
def test_gram_digits_match_fp64(gpu_lib, n, m, w):
    G = gpu_lib
    rng = np.random.default_rng(n + 7 * m + w)
    Q = rng.standard_normal((n, m))
    P = rng.standard_normal((n, w))
    exact = _gram_exact(Q, P)
    scale = np.abs(Q).T @ np.abs(P)
    emu = G.dense_gram(Q, P, emulated=True)
    fp64 = G.dense_gram(Q, P, emulated=False)
    e_emu, e_fp = _rel_err(emu, exact, scale), _rel_err(fp64, exact, scale)
    assert e_emu < 5e-16, (e_emu, e_fp)
    assert e_fp < 5e-15


def test_gram_digits_wide_range_and_structure(gpu_lib):
    G = gpu_lib
    rng = np.random.default_rng(3)
    n, m, w = 9000, 24, 12
    Q = rng.standard_normal((n, m)) * 10.0 ** rng.uniform(-6, 6, (n, m))
    P = rng.standard_normal((n, w)) * 10.0 ** rng.uniform(-6, 6, (n, w))
    Q[:, 3] = 0.0                       # zero column
    Q[100:200, 5] = 1e-300              # subnormal-range products
    P[:, 7] = np.sin(np.arange(n))      # smooth column
    exact = _gram_exact(Q, P)
    scale = np.abs(Q).T @ np.abs(P)
    emu = G.dense_gram(Q, P, emulated=True)
    assert np.all(emu[3] == 0.0)
    assert _rel_err(emu, exact, scale) < 1e-14


def test_gram_digits_orthogonal_block(gpu_lib):
    """The B-orthogonalisation use: Q^T P for nearly orthogonal blocks, where
    the result is tiny against |Q|^T |P|."""
    G = gpu_lib
    rng = np.random.default_rng(5)
    n = 30000
    Q, _ = np.linalg.qr(rng.standard_normal((n, 60)))
    P = rng.standard_normal((n, 20))
    P -= Q @ (Q.T @ P)
    P -= Q @ (Q.T @ P)
    exact = _gram_exact(Q, P)
    emu = G.dense_gram(Q, P, emulated=True)
    scale = np.abs(Q).T @ np.abs(P)
    assert _rel_err(emu, exact, scale) < 5e-16
    assert np.max(np.abs(emu)) < 1e-13


def test_gram_digits_nan_propagates(gpu_lib):
    G = gpu_lib
    rng = np.random.default_rng(9)
    Q = rng.standard_normal((500, 6))
    P = rng.standard_normal((500, 4))
    Q[77, 2] = np.nan
    P[400, 1] = np.inf
    C = G.dense_gram(Q, P, emulated=True)
    assert np.all(np.isnan(C[2]))
    assert np.all(~np.isfinite(C[:, 1]))
    keep = [0, 1, 3, 4, 5]
    assert np.all(np.isfinite(C[np.ix_(keep, [0, 2, 3])]))


@pytest.mark.parametrize("n,k,m,mode", [(20011, 180, 20, "minus_one"), (5000, 37, 160, "none"),
                                        (1000, 3, 5, "vector"), (70001, 52, 24, "none"),
                                        (64, 64, 8, "vector"), (333, 200, 17, "minus_one"),
                                        (3001, 1000, 24, "minus_one"), (5000, 481, 50, "vector"),
                                        (4000, 433, 40, "none"), (2000, 145, 33, "vector")])
def test_lincomb_digits_match_fp64(gpu_lib, n, k, m, mode):
    G = gpu_lib
    rng = np.random.default_rng(n + k + m)
    X = rng.standard_normal((n, k))
    C = rng.standard_normal((k, m))
    Y0 = rng.standard_normal((n, m))
    if mode == "none":
        beta, alpha = None, 1.0
    elif mode == "minus_one":            # the orth update W = W - V C
        beta, alpha = np.ones(m), -1.0
    else:
        beta, alpha = rng.uniform(-2, 2, m), 0.75
    ex = EXT(alpha) * (X.astype(EXT) @ C.astype(EXT))
    scale = abs(alpha) * (np.abs(X) @ np.abs(C))
    if beta is not None:
        ex = ex + Y0.astype(EXT) * beta.astype(EXT)
        scale = scale + np.abs(Y0) * np.abs(beta)
    emu = G.dense_lincomb(X, C, Y0, beta=beta, alpha=alpha, emulated=True)
    fp64 = G.dense_lincomb(X, C, Y0, beta=beta, alpha=alpha, emulated=False)
    e_emu, e_fp = _rel_err(emu, ex, scale), _rel_err(fp64, ex, scale)
    assert e_emu < 1e-15, (e_emu, e_fp)
    assert e_fp < 1e-14


def test_lincomb_digits_nan_and_zero_k(gpu_lib):
    G = gpu_lib
    rng = np.random.default_rng(2)
    X = rng.standard_normal((300, 10))
    C = rng.standard_normal((10, 4))
    X[17, 3] = np.nan
    Y = G.dense_lincomb(X, C, np.zeros((300, 4)), emulated=True)
    assert np.all(np.isnan(Y[17]))
    assert np.all(np.isfinite(np.delete(Y, 17, axis=0)))
    # k = 0: Y diag(beta)
    Y0 = rng.standard_normal((50, 3))
    out = G.dense_lincomb(np.zeros((50, 0)), np.zeros((0, 3)), Y0, beta=np.array([2.0, 0.0, -1.0]),
                          emulated=True)
    np.testing.assert_array_equal(out, Y0 * np.array([2.0, 0.0, -1.0]))
