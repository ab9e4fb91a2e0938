"""The CPU oracle (numpy restatement of the reference GCG) pinned against the
golden fixtures produced by the reference's own C sources, and against the
analytic Dirichlet spectrum."""
import numpy as np
import pytest

from conftest import build_case
from gcge_gb300 import problems as P
from oracle import ref_lib
from oracle.gcg_oracle import GCGOracle, GCGParams, gcg_solve, residuals

FAST_CASES = ["laplace2d_24x24_nev8", "laplace2d_24x24_noshift", "laplace2d_20x20_abstol",
              "vardiff3d_12", "vardiff3d_12_nev200", "aniso2d_40x30_eps10_diagB",
              "rgg_2000_deg10"]


def run_oracle(case, g):
    A, B = build_case(case)
    X0 = P.initial_block(A.n, g["nev_init"], seed=g["x0_seed"])
    return A, B, gcg_solve(A.to_scipy(), None if B is None else B.to_scipy(), X0, g["nev"],
                           g["block_size"], g["nev_init"], g["nev_max"], tol=tuple(g["tol"]),
                           max_iter=g["max_iter"], gap_min=g["gap_min"], auto_shift=g["auto_shift"])


@pytest.mark.parametrize("case", FAST_CASES)
def test_oracle_matches_reference_fixture(case, golden):
    g = golden[case]
    A, B, r = run_oracle(case, g)
    nev = g["nev"]
    ref = np.array(g["eval"][:nev])
    assert r.nconv >= nev
    # same algorithm: eigenvalues agree far below the solver tolerance
    assert np.max(np.abs(r.eval[:nev] - ref) / np.abs(ref)) < 1e-10
    # iteration counts agree up to summation-order effects
    assert abs(r.niter - g["niter"]) <= max(3, g["niter"] // 5)
    res, rel = residuals(A.to_scipy(), None if B is None else B.to_scipy(), r.eval[:nev],
                         r.evec[:, :nev])
    tol0, tol1 = g["tol"]
    assert np.all((res <= tol0 * 1.0001) & (rel <= tol1 * 1.0001))


def test_oracle_analytic_laplace2d():
    A = P.laplace2d(24, 24)
    X0 = P.initial_block(A.n, 12, seed=1)
    r = gcg_solve(A.to_scipy(), None, X0, 8, 4, 12, 20)
    k = np.arange(1, 25)
    lam1 = 2 - 2 * np.cos(k * np.pi / 25)
    exact = np.sort((lam1[:, None] + lam1[None, :]).ravel())[:8]
    assert np.max(np.abs(r.eval[:8] - exact) / exact) < 1e-11


def test_oracle_mgs_orthonormalises():
    A = P.laplace2d(10, 10).to_scipy()
    Bd = P.diag_matrix(np.linspace(0.5, 2.0, 100)).to_scipy()
    o = GCGOracle(A, Bd, GCGParams(nev_init=6, nev_max=6, block_size=2))
    rng = np.random.default_rng(3)
    X = np.asfortranarray(rng.standard_normal((100, 8)))
    X[:, 5] = 0.0                        # a zero column is dropped (src/ops_orth.c:64-74)
    end = o.mgs(X, 0, 8, Bd)
    assert end == 7
    G = X[:, :end].T @ (Bd @ X[:, :end])
    assert np.abs(G - np.eye(end)).max() < 1e-12


def test_oracle_block_pcg_stops_at_rate():
    A = P.laplace2d(16, 16).to_scipy()
    o = GCGOracle(A, None, GCGParams(nev_init=4, nev_max=4, block_size=4))
    o.sigma = 0.3
    rng = np.random.default_rng(4)
    b = np.asfortranarray(rng.standard_normal((256, 3)))
    x = np.zeros((256, 3), order="F")
    it = o.block_pcg(b, x)
    r = b - (A @ x + 0.3 * x)
    assert it <= 30
    assert np.all(np.linalg.norm(r, axis=0) <= 1e-2 * np.linalg.norm(b, axis=0) * 1.0001)


@pytest.mark.skipif(not ref_lib.available(), reason="reference build (oracle/_ref) not present")
def test_oracle_matches_live_reference_on_new_input():
    A = P.aniso2d(17, 23, 3.0)
    B = P.diag_matrix(0.5 + 1.5 * P.splitmix_uniform(99, A.n, 0))
    X0 = P.initial_block(A.n, 9, seed=7)
    ev, evec, nc, it, _ = ref_lib.ref_solve(A, B, X0, 10, 3, 9, 19)
    r = gcg_solve(A.to_scipy(), B.to_scipy(), X0, 10, 3, 9, 19)
    assert nc >= 10 and r.nconv >= 10
    assert np.max(np.abs(ev[:10] - r.eval[:10]) / np.abs(ev[:10])) < 1e-10


# ---------------------------------------------------------------------------
# Binary Gram-Schmidt (src/ops_orth.c:416-641) and ComputeW12
# (src/ops_eig_sol_gcg.c:703-929) against the reference's outputs
# ---------------------------------------------------------------------------
ORTH_CASES = ["mleaf_plain", "mleaf_prefix_diagB_zero", "mleaf_near_prefix", "mleaf_prefix_dep",
              "evp_plain", "evp_prefix_diagB_dep", "evp_wide_massB_zero", "evp_prefix_zero"]


@pytest.mark.parametrize("case", ORTH_CASES)
def test_oracle_bgs_matches_reference_fixture(case, golden_orth):
    import scipy.sparse as sp
    from conftest import b_projector, orth_case
    x, start, end, bs, B = orth_case(case)
    meta = golden_orth["orth"][f"{case}/bgs"]
    ref = golden_orth["arrays"][f"{case}/bgs"]
    Bs = None if B is None else B.to_scipy()
    o = GCGOracle(sp.identity(x.shape[0], format="csr"), Bs,
                  GCGParams(nev_init=1, nev_max=1, block_size=1, orth_method="bgs",
                            orth_block_size=bs))
    got_end = o.bgs(x, start, end, Bs)
    assert got_end == meta["end"]
    X = x[:, :got_end]
    G = X.T @ (X if Bs is None else Bs @ X)
    assert np.abs(G - np.eye(got_end)).max() < 1e-13
    # the same subspace; leaves of OrthSelf (blocks under 16 columns) also the same basis
    tol = 5e-9 if "near" in case else 1e-13
    assert np.abs(b_projector(X, Bs) - b_projector(ref, Bs)).max() < tol
    if case.startswith("mleaf"):
        assert np.abs(X - ref).max() < tol


SOLVE_CASES_CPU = ["laplace2d_24x24_nev8_bgs", "aniso2d_40x30_eps10_diagB_bgs",
                   "laplace2d_24x24_nev8_w12", "aniso2d_40x30_eps10_diagB_w12",
                   "aniso2d_40x30_eps10_diagB_w12_bgs"]


@pytest.mark.parametrize("case", SOLVE_CASES_CPU)
def test_oracle_orth_and_w12_solves_match_reference_fixture(case, golden_orth):
    from conftest import orth_solve_case
    g = golden_orth["solve"][case]
    A, B = orth_solve_case(case)
    X0 = P.initial_block(A.n, g["nev_init"], seed=g["x0_seed"])
    r = gcg_solve(A.to_scipy(), None if B is None else B.to_scipy(), X0, g["nev"], g["block_size"],
                  g["nev_init"], g["nev_max"], tol=tuple(g["tol"]), max_iter=g["max_iter"],
                  gap_min=g["gap_min"], auto_shift=g["auto_shift"],
                  orth=None if g["orth"] is None else tuple(g["orth"]),
                  w_order=2 if "-gcge_compW_cg_order" in g["args"] else 1)
    nev = g["nev"]
    ref = np.array(g["eval"][:nev])
    assert r.nconv >= nev
    assert np.max(np.abs(r.eval[:nev] - ref) / np.abs(ref)) < 1e-10
    assert abs(r.niter - g["niter"]) <= max(3, g["niter"] // 5)


def _pcg_cases():
    """(name, A, b, x0, sb, sx, k, max_iter, rate, tol, tol_type, user_norms)."""
    A = P.laplace2d(40, 30)
    n = A.n
    rng = np.random.default_rng(0)
    B = rng.standard_normal((n, 14))
    X0 = 0.1 * rng.standard_normal((n, 13))
    # columns whose right-hand sides are eigenvectors leave after one step
    sx_ = np.sin(np.pi * np.arange(1, 41) / 41)
    sy_ = np.sin(np.pi * 2 * np.arange(1, 31) / 31)
    Be = B.copy()
    Be[:, 2] = np.kron(sy_, sx_)
    Be[:, 3] = 3.0 * np.kron(sy_, sx_)
    Z = np.zeros_like(X0)
    return [
        ("abs_ranges", A, B, X0, 2, 1, 6, 30, 1e-2, 1e-6, "abs", None),
        ("rel_early_leavers", A, Be, Z, 2, 0, 12, 25, 0.0, 1e-10, "rel", None),
        ("user_norms", A, B, X0, 0, 0, 5, 40, 1e-3, 1e-7, "user",
         np.array([2.0, -1.0, 0.5, 4.0, 1.0])),
        ("all_converge", A, B, Z, 1, 3, 7, 400, 0.0, 1e-8, "abs", None),
        ("no_iteration", A, B, X0, 0, 0, 4, 30, 1e-2, 1e30, "abs", None),
    ]


@pytest.mark.skipif(not ref_lib.available(), reason="reference build (oracle/_ref) not present")
@pytest.mark.parametrize("idx", range(5))
def test_block_pcg_restatements_match_live_reference(idx):
    """Both CPU restatements of BlockPCG (the GCG oracle's, which the GPU
    linear-solver tests compare with, and the block AMG oracle's, which also
    keeps the solver record's fields) against the compiled reference's
    BlockPCG: the solution, the iteration count and the residual field
    (src/ops_lin_sol.c:406-410), on column ranges, early leavers, "rel" and
    "user" norms, convergence of every column, and no iteration at all."""
    from oracle.amg_oracle import block_pcg
    name, A, B, X0, sb, sx, k, mi, rate, tol, tt, un = _pcg_cases()[idx]
    xr, itr, resr = ref_lib.ref_block_pcg(A, B, X0, sb, sx, k, mi, rate, tol, tt, un)
    As = A.to_scipy()
    b = np.asfortranarray(B[:, sb:sb + k])
    # the block AMG oracle's BlockPCG
    x1 = np.array(X0[:, sx:sx + k], order="F", copy=True)
    st = block_pcg(lambda v: As @ v, b, x1, mi, rate, tol, tt, user_norms=un)
    assert np.abs(x1 - xr[:, sx:sx + k]).max() <= 1e-12 * max(1.0, np.abs(xr).max())
    assert st.niter == itr
    assert st.residual == pytest.approx(resr, rel=1e-6, abs=1e-14 * np.linalg.norm(b))
    # columns outside the range are untouched
    keep = [c for c in range(X0.shape[1]) if not sx <= c < sx + k]
    assert np.array_equal(xr[:, keep], X0[:, keep])
    # the GCG oracle's BlockPCG
    if tt != "user":
        p = GCGParams(nev_init=1, nev_max=1, block_size=1, cg_max_iter=mi, cg_rate=rate,
                      cg_tol=tol, cg_tol_type=tt)
        o = GCGOracle(As, None, p)
        x2 = np.array(X0[:, sx:sx + k], order="F", copy=True)
        it2 = o.block_pcg(b, x2)
        assert it2 == itr
        assert np.abs(x2 - xr[:, sx:sx + k]).max() <= 1e-12 * max(1.0, np.abs(xr).max())
    if name == "rel_early_leavers":
        assert itr == mi and resr > 1e-6          # a random column's residual
    if name == "no_iteration":
        assert itr == 0
        r0 = np.linalg.norm(B[:, sb] - As @ X0[:, sx])
        assert resr == pytest.approx(r0, rel=1e-12)
