"""Solver components on the GPU, one at a time: the dense eigensolver of the
Rayleigh-Ritz step, the block-PCG inner solve and the B-orthonormalisation,
against numpy/scipy and the CPU oracle."""
import numpy as np
import pytest

from gcge_gb300 import problems as P
from oracle.gcg_oracle import GCGOracle, GCGParams

pytestmark = pytest.mark.gpu


def sym_with_spectrum(lam, seed):
    rng = np.random.default_rng(seed)
    Q, _ = np.linalg.qr(rng.standard_normal((lam.size, lam.size)))
    M = (Q * lam) @ Q.T
    return 0.5 * (M + M.T)


@pytest.mark.parametrize("s", [1, 2, 7, 40, 64, 87, 88, 160, 230, 337, 400])
def test_dense_eig_random(gpu_lib, s):
    """s < 88: one-CTA Jacobi; s >= 88: the 8-CTA cluster Jacobi (337 and 400
    are beyond the one-CTA kernel's shared memory; 400 is the largest
    projected dimension of the 128^3 variable-coefficient workload)."""
    rng = np.random.default_rng(s)
    lam = np.sort(rng.uniform(0.01, 100.0, s))
    M = sym_with_spectrum(lam, s)
    ev, Z = gpu_lib.dense_eig(M)
    scale = np.abs(lam).max()
    assert np.all(np.diff(ev) >= 0)
    assert np.max(np.abs(ev - np.linalg.eigvalsh(M))) <= 1e-13 * scale
    assert np.abs(Z.T @ Z - np.eye(s)).max() < 1e-11
    assert np.abs(M @ Z - Z * ev).max() < 1e-12 * scale


@pytest.mark.parametrize("gap", [0.0, 1e-14, 1e-10, 1e-7, 1e-4])
def test_dense_eig_clusters(gpu_lib, gap):
    """Exactly and nearly degenerate eigenvalues (the Rayleigh-Ritz matrices of
    symmetric problems have them)."""
    lam = np.concatenate([[1.0, 2.0], 3.0 + gap * np.arange(4), np.linspace(5, 50, 30)])
    M = sym_with_spectrum(lam, 3)
    ev, Z = gpu_lib.dense_eig(M)
    assert np.max(np.abs(ev - np.sort(lam))) < 1e-12 * 50
    assert np.abs(Z.T @ Z - np.eye(lam.size)).max() < 1e-11
    assert np.abs(M @ Z - Z * ev).max() < 1e-12 * 50


def test_dense_eig_rr_structure(gpu_lib):
    """Diagonal X block plus a weak coupling to a P/W block, as in late GCG
    iterations, including a converged double eigenvalue."""
    rng = np.random.default_rng(9)
    d = np.sort(rng.uniform(0.03, 8.0, 24))
    d[3] = d[4]
    M = np.zeros((32, 32))
    M[:24, :24] = np.diag(d)
    C = 1e-6 * rng.standard_normal((24, 8))
    W = rng.standard_normal((8, 8))
    M[:24, 24:] = C
    M[24:, :24] = C.T
    M[24:, 24:] = 10.0 + W @ W.T
    ev, Z = gpu_lib.dense_eig(M)
    ref = np.linalg.eigvalsh(M)
    assert np.max(np.abs(ev - ref)) < 1e-13 * np.abs(ref).max()
    assert np.abs(M @ Z - Z * ev).max() < 1e-13 * np.abs(ref).max()


@pytest.mark.parametrize("fp32", [False, True])
@pytest.mark.parametrize("grid", [30, 170])
def test_block_pcg_matches_oracle(gpu_lib, fp32, grid):
    """n = 900 runs the kernel's cluster form, n = 28900 (904 slices) its
    grid form with the cooperative launch."""
    A = P.laplace2d(grid, grid)
    B = P.diag_matrix(0.5 + 1.5 * P.splitmix_uniform(3, A.n, 0))
    rng = np.random.default_rng(4)
    b = rng.standard_normal((A.n, 5))
    x0 = rng.standard_normal((A.n, 5)) * 0.1
    sigma = 0.25
    x, it = gpu_lib.block_pcg(A, B, sigma, b, x0, max_iter=30, rate=1e-2, tol=1e-14, fp32=fp32)
    o = GCGOracle(A.to_scipy(), B.to_scipy(), GCGParams(nev_init=5, nev_max=5, block_size=5))
    o.sigma = sigma
    xr = np.asfortranarray(x0.copy())
    ito = o.block_pcg(np.asfortranarray(b), xr)
    assert abs(it - ito) <= (0 if not fp32 else 2)
    S = A.to_scipy() + sigma * B.to_scipy()
    r0 = np.linalg.norm(b - S @ x0, axis=0)
    r = np.linalg.norm(b - S @ x, axis=0)
    assert np.all(r <= 1.05e-2 * r0)
    tol = 1e-9 if not fp32 else 2e-4
    assert np.abs(x - xr).max() <= tol * np.abs(xr).max()


@pytest.mark.parametrize("withB", [False, True])
def test_b_orth_against_prefix_and_self(gpu_lib, withB):
    A = P.laplace2d(40, 25)
    n = A.n
    B = P.diag_matrix(0.5 + 1.5 * P.splitmix_uniform(8, n, 0)) if withB else None
    Bs = B.to_scipy() if withB else None
    rng = np.random.default_rng(2)
    X = rng.standard_normal((n, 12))
    Q0 = gpu_lib.b_orth(B, X[:, :5], 0, A_for_size=A)
    X[:, :5] = Q0
    X[:, 9] = X[:, 7] + 1e-3 * rng.standard_normal(n)   # nearly dependent: kept
    Q = gpu_lib.b_orth(B, X, 5, A_for_size=A)
    BQ = Q if not withB else Bs @ Q
    assert Q.shape[1] == 12
    assert np.abs(Q.T @ BQ - np.eye(12)).max() < 1e-12
    np.testing.assert_allclose(Q[:, :5], X[:, :5], rtol=0, atol=0)
    # the span of the new block is kept
    proj = X[:, 5:] - Q @ (BQ.T @ X[:, 5:])
    assert np.abs(proj).max() < 1e-10 * np.abs(X).max()


def test_b_orth_drops_zero_columns(gpu_lib):
    A = P.laplace2d(20, 20)
    X = np.random.default_rng(1).standard_normal((A.n, 6))
    X[:, 3] = 0.0
    Q = gpu_lib.b_orth(None, X, 0, A_for_size=A)
    assert Q.shape[1] == 5
    assert np.abs(Q.T @ Q - np.eye(5)).max() < 1e-13
