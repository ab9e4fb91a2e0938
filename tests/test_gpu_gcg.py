"""End-to-end parity of the GPU GCG with the reference GCGE CPU path on the
same seeded inputs: eigenvalues within 1e-10 relative of the reference's
(golden fixtures made by its own C sources), eigenvector subspaces within
1e-6 rad per cluster, every residual under the requested tolerance."""
import numpy as np
import pytest

from conftest import build_case, cluster_subspace_angle, cluster_subspace_sine
from gcge_gb300 import problems as P
from oracle.gcg_oracle import gcg_solve, residuals

pytestmark = pytest.mark.gpu

CASES = ["laplace2d_24x24_nev8", "laplace2d_24x24_noshift", "laplace2d_20x20_abstol",
         "laplace2d_128x128_nev20_bs20", "laplace2d_128x128_nev20_rule", "laplace3d_mass_16",
         "laplace3d_mass_24", "vardiff3d_12", "vardiff3d_12_nev200", "aniso2d_40x30_eps10_diagB",
         "rgg_2000_deg10"]


def run_gpu(G, case, g, precision=0):
    A, B = build_case(case)
    X0 = P.initial_block(A.n, g["nev_init"], seed=g["x0_seed"])
    r = G.solve(A, B, g["nev"], g["block_size"], g["nev_init"], g["nev_max"], X0=X0,
                tol=tuple(g["tol"]), max_iter=g["max_iter"], gap_min=g["gap_min"],
                auto_shift=g["auto_shift"], precision=precision)
    return A, B, r


@pytest.mark.parametrize("case", CASES)
def test_gcg_matches_reference(gpu_lib, golden, golden_vectors, case):
    g = golden[case]
    A, B, r = run_gpu(gpu_lib, case, g)
    nev = g["nev"]
    ref = np.array(g["eval"][:nev])
    assert r.status == gpu_lib.GCGE_OK
    assert r.nconv >= nev
    rel = np.abs(r.eval[:nev] - ref) / np.abs(ref)
    assert rel.max() < 1e-10, rel.max()
    Bs = None if B is None else B.to_scipy()
    res, relres = residuals(A.to_scipy(), Bs, r.eval[:nev], r.evec[:, :nev])
    tol0, tol1 = g["tol"]
    assert np.all(res <= tol0 * 1.001) and np.all(relres <= tol1 * 1.001)
    if case in golden_vectors:
        ang = cluster_subspace_angle(r.eval[:nev], r.evec[:, :nev], golden_vectors[case], Bs)
        assert ang < 1e-6, ang
    # B-orthonormal eigenvectors
    V = r.evec[:, :nev]
    BV = V if Bs is None else Bs @ V
    assert np.abs(V.T @ BV - np.eye(nev)).max() < 1e-9
    # iteration count close to the reference's
    assert abs(r.niter - g["niter"]) <= max(4, g["niter"] // 4), (r.niter, g["niter"])


# The benchmarked workloads: the generalized 64^3 stiffness + Kronecker-mass
# problem (nev 100) at full size and at 32^3, and the generator of the 128^3
# variable-coefficient problem with its nev-200 block rule at 32^3, each against
# the compiled reference on the same seeded inputs.
LARGE = ["laplace3d_mass_32", "vardiff3d_32_nev200", "laplace3d_mass_64"]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("case", LARGE)
def test_benchmarked_sizes_match_reference(gpu_lib, golden, golden_vectors_large, case,
                                           precision):
    """Eigenvalues within 1e-10 relative of the reference's, every residual
    under the tolerance, the leading eigenvector clusters within 1e-6 rad of
    the reference's (where stored), the returned vectors B-orthonormal."""
    g = golden[case]
    prec = gpu_lib.PREC_FP64 if precision == "fp64" else gpu_lib.PREC_MIXED
    A, B, r = run_gpu(gpu_lib, case, g, precision=prec)
    nev = g["nev"]
    ref = np.array(g["eval"][:nev])
    assert r.status == gpu_lib.GCGE_OK and r.nconv >= nev, (r.status, r.nconv)
    rel = np.abs(r.eval[:nev] - ref) / np.abs(ref)
    assert rel.max() < 1e-10, rel.max()
    Bs = None if B is None else B.to_scipy()
    res, relres = residuals(A.to_scipy(), Bs, r.eval[:nev], r.evec[:, :nev])
    assert np.all(relres <= g["tol"][1] * 1.001), relres.max()
    if case in golden_vectors_large:
        Vref = golden_vectors_large[case]
        m = Vref.shape[1]
        sine = cluster_subspace_sine(r.eval[:m], r.evec[:, :m], Vref, Bs)
        assert sine < 1e-6, sine
    V = r.evec[:, :nev]
    BV = V if Bs is None else Bs @ V
    assert np.abs(V.T @ BV - np.eye(nev)).max() < 1e-9
    if precision == "fp64":
        assert abs(r.niter - g["niter"]) <= max(4, g["niter"] // 4), (r.niter, g["niter"])


def test_analytic_spectrum_config1(gpu_lib, golden):
    g = golden["laplace2d_128x128_nev20_bs20"]
    A, B, r = run_gpu(gpu_lib, "laplace2d_128x128_nev20_bs20", g)
    k = np.arange(1, 129)
    lam1 = 2 - 2 * np.cos(k * np.pi / 129)
    exact = np.sort((lam1[:, None] + lam1[None, :]).ravel())[:20]
    assert np.max(np.abs(r.eval[:20] - exact) / exact) < 1e-10


@pytest.mark.parametrize("case", ["laplace3d_mass_16", "vardiff3d_12", "laplace2d_128x128_nev20_bs20"])
def test_mixed_precision_same_eigenvalues(gpu_lib, golden, case):
    """FP32 inner solve, FP64 everything else: same eigenvalues, same tolerance."""
    g = golden[case]
    A, B, r = run_gpu(gpu_lib, case, g, precision=gpu_lib.PREC_MIXED)
    nev = g["nev"]
    ref = np.array(g["eval"][:nev])
    assert r.status == gpu_lib.GCGE_OK and r.nconv >= nev
    assert np.max(np.abs(r.eval[:nev] - ref) / np.abs(ref)) < 1e-10
    Bs = None if B is None else B.to_scipy()
    res, relres = residuals(A.to_scipy(), Bs, r.eval[:nev], r.evec[:, :nev])
    assert np.all(relres <= g["tol"][1] * 1.001)
    # the returned vectors are B-orthonormal (the projected-space products of
    # the mixed solve stay FP64, so its basis keeps FP64-level orthonormality)
    V = r.evec[:, :nev]
    BV = V if Bs is None else Bs @ V
    assert np.abs(V.T @ BV - np.eye(nev)).max() < 1e-9


def test_matches_live_oracle_on_unseen_input(gpu_lib):
    """A problem the fixtures do not hold, against the oracle run here."""
    A = P.aniso2d(33, 21, 2.5)
    B = P.diag_matrix(0.5 + 1.5 * P.splitmix_uniform(42, A.n, 0))
    X0 = P.initial_block(A.n, 12, seed=3)
    r = gpu_lib.solve(A, B, 10, 4, 12, 22, X0=X0)
    o = gcg_solve(A.to_scipy(), B.to_scipy(), X0, 10, 4, 12, 22)
    assert r.nconv >= 10 and o.nconv >= 10
    assert np.max(np.abs(r.eval[:10] - o.eval[:10]) / o.eval[:10]) < 1e-10


def test_prepared_solve_is_repeatable(gpu_lib):
    c = P.config1()
    X0 = P.initial_block(c["A"].n, 40, seed=1)
    prep = gpu_lib.Prepared(c["A"], None, 20, 20, 40, 40, X0=X0)
    try:
        r1 = prep.solve(want_evec=True)
        r2 = prep.solve(want_evec=True)
    finally:
        prep.close()
    assert np.array_equal(r1.eval, r2.eval) and r1.niter == r2.niter
    assert np.array_equal(r1.evec, r2.evec)
    assert r1.info["kernel_launches"] > 0 and r1.info["spmm_calls"] > 0


def test_mixed_escalates_to_fp64_inner_solve_when_fp32_stalls(gpu_lib):
    """A shifted random-geometric-graph Laplacian (eigenvalues from 1e-3, |A| ~ 20)
    at relative tolerance 4.6e-10: the FP32 inner solve's operator rounding,
    amplified by the near-singular shift, and the digit products stall the
    residuals just above the tolerance; the mixed solve must notice, finish in
    FP64 and converge like the FP64 solve (the reference converges in ~100
    iterations on this input)."""
    G = gpu_lib
    import scipy.sparse.linalg as sla
    c = P.serving_requests(3, seed=5, rate=8.0, max_n=100_000)[1]
    assert c["name"].startswith("rgg_9745") and c["B"] is None
    X0 = P.initial_block(c["A"].n, c["nev_init"], seed=1)
    kw = dict(X0=X0, tol=c["tol"], want_evec=False)
    mixed = G.solve(c["A"], c["B"], c["nev"], c["block_size"], c["nev_init"], c["nev_max"],
                    precision=G.PREC_MIXED, **kw)
    fp64 = G.solve(c["A"], c["B"], c["nev"], c["block_size"], c["nev_init"], c["nev_max"],
                   precision=G.PREC_FP64, **kw)
    nev = c["nev"]
    assert fp64.status == G.GCGE_OK and mixed.status == G.GCGE_OK, (fp64.status, mixed.status)
    assert mixed.nconv >= nev and mixed.info["precision_escalation_iter"] > 20
    assert fp64.info["precision_escalation_iter"] == 0
    w = np.sort(sla.eigsh(c["A"].to_scipy().tocsc(), k=nev, sigma=0, which="LM",
                          return_eigenvectors=False))
    np.testing.assert_allclose(mixed.eval[:nev], w, rtol=1e-9, atol=0)
    np.testing.assert_allclose(mixed.eval[:nev], fp64.eval[:nev], rtol=1e-10, atol=0)


def test_nev200_projected_dimension_400(gpu_lib):
    """The block rule of the 128^3 variable-coefficient workload (nev 200:
    bs 40, nevInit 120, nevMax 320) at 16^3: projected dimensions up to 400,
    the cluster Jacobi's range beyond the one-CTA kernel's.  Mixed and FP64
    solves agree with each other and with the dense generalized eigenvalues,
    and every returned pair meets the relative residual tolerance."""
    import scipy.linalg as sl
    c = P.config3(16)
    A, B, nev = c["A"], c["B"], c["nev"]
    kw = dict(nev=nev, block_size=c["block_size"], nev_init=c["nev_init"], nev_max=c["nev_max"],
              max_iter=2000)
    assert (c["block_size"], c["nev_init"], c["nev_max"]) == (40, 120, 320)
    r64 = gpu_lib.solve(A, B, precision=gpu_lib.PREC_FP64, **kw)
    rmx = gpu_lib.solve(A, B, precision=gpu_lib.PREC_MIXED, **kw)
    for r in (r64, rmx):
        assert r.status == gpu_lib.GCGE_OK and r.nconv >= nev
    d = B.diagonal()
    s = 1.0 / np.sqrt(d)
    H = (A.to_scipy().toarray() * s[:, None]) * s[None, :]
    ref = sl.eigh(H, eigvals_only=True, subset_by_index=[0, nev - 1])
    for r in (r64, rmx):
        assert np.max(np.abs(r.eval[:nev] - ref) / np.abs(ref)) < 1e-10
        X = r.evec[:, :nev]
        R = A.to_scipy() @ X - (d[:, None] * X) * r.eval[:nev]
        rel = np.linalg.norm(R, axis=0) / np.abs(r.eval[:nev])
        assert rel.max() < 1e-8 * 1.05
    assert np.max(np.abs(rmx.eval[:nev] - r64.eval[:nev]) / np.abs(r64.eval[:nev])) < 1e-10
