"""MultiVecOrth on the GPU (MultiVecOrthSetup_BinaryGramSchmidt /
_ModifiedGramSchmidt, src/ops_orth.c:395-641), GCG solves with binary
Gram-Schmidt or ComputeW12 (compW_cg_order 2, src/ops_eig_sol_gcg.c:703-929)
selected, and the user-defined MultiLinearSolver hook, against the reference's
own outputs on the same inputs (tests/golden/golden_orth.*, made by
tests/golden/make_golden_orth.py).

What must agree for MultiVecOrth: the number of columns kept (the dependent
ones dropped), the subspace (B-orthogonal projector), B-orthonormality, and
for the binary variant with OrthSelf leaves (blocks under 16 columns) the
basis itself.  The eigen-decomposition leaves fix the basis only up to a
rotation inside each leaf, so there the subspace is compared."""
import ctypes

import numpy as np
import pytest

from conftest import b_projector, orth_case, orth_solve_case
from gcge_gb300 import problems as P

pytestmark = pytest.mark.gpu

ORTH_CASES = ["mleaf_plain", "mleaf_prefix_diagB_zero", "mleaf_near_prefix", "mleaf_prefix_dep",
              "evp_plain", "evp_prefix_diagB_dep", "evp_wide_massB_zero", "evp_prefix_zero"]


def gpu_orth(G, case, method):
    x, start, end, bs, B = orth_case(case)
    ops = G.CudaOps()
    try:
        hB = ops.mat(B) if B is not None else None
        hM = hB if hB is not None else ops.mat(P.identity_diag(x.shape[0]))
        hx = ops.multivec(hM, x.shape[1], x)
        ops.orth_setup(method, bs, 2, 2 * np.finfo(float).eps)
        new_end = ops.orth(hx, start, end, hB)
        return ops.download(hx, 0, new_end), new_end, B
    finally:
        ops.close()


@pytest.mark.parametrize("method", ["bgs", "mgs"])
@pytest.mark.parametrize("case", ORTH_CASES)
def test_multivec_orth_matches_reference(gpu_lib, golden_orth, case, method):
    G = gpu_lib
    meta = golden_orth["orth"][f"{case}/{method}"]
    ref = golden_orth["arrays"][f"{case}/{method}"]
    X, end, B = gpu_orth(G, case, method)
    assert end == meta["end"], (end, meta["end"])
    Bs = None if B is None else B.to_scipy()
    BX = X if Bs is None else Bs @ X
    assert np.abs(X.T @ BX - np.eye(end)).max() < 1e-13
    tol = 5e-9 if "near" in case else 1e-13
    assert np.abs(b_projector(X, Bs) - b_projector(ref, Bs)).max() < tol
    if method == "bgs" and case.startswith("mleaf"):
        assert np.abs(X - ref).max() < tol


def test_multivec_orth_requires_setup(gpu_lib):
    G = gpu_lib
    a, b = G.CudaOps(), G.CudaOps()
    try:
        a.orth_setup("bgs")
        assert a.ptr.contents.MultiVecOrth and a.ptr.contents.orth_workspace
        assert not b.ptr.contents.MultiVecOrth   # a second ops has none installed
    finally:
        b.close()
        a.close()


SOLVES = ["laplace2d_24x24_nev8_bgs", "aniso2d_40x30_eps10_diagB_bgs", "laplace3d_mass_16_bgs",
          "laplace3d_mass_16_bgs_leaf8", "laplace2d_24x24_nev8_w12", "aniso2d_40x30_eps10_diagB_w12",
          "aniso2d_40x30_eps10_diagB_w12_bgs", "laplace3d_mass_16_w12"]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("case", SOLVES)
def test_orth_and_w12_solves_match_reference(gpu_lib, golden_orth, case, precision):
    G = gpu_lib
    g = golden_orth["solve"][case]
    A, B = orth_solve_case(case)
    X0 = P.initial_block(A.n, g["nev_init"], seed=g["x0_seed"])
    r = G.solve_ops(A, B, g["nev"], g["block_size"], g["nev_init"], g["nev_max"], X0=X0,
                    tol=tuple(g["tol"]), max_iter=g["max_iter"], gap_min=g["gap_min"],
                    auto_shift=g["auto_shift"],
                    precision=G.PREC_MIXED if precision == "mixed" else G.PREC_FP64,
                    orth=None if g["orth"] is None else tuple(g["orth"]), args=tuple(g["args"]))
    nev = g["nev"]
    assert r.status == G.GCGE_OK and r.nconv >= nev, (r.status, r.nconv)
    ref = np.array(g["eval"][:nev])
    assert np.max(np.abs(r.eval[:nev] - ref) / np.abs(ref)) < 1e-10
    if precision == "fp64":
        assert abs(r.niter - g["niter"]) <= max(3, g["niter"] // 5)
    X = r.evec[:, :nev]
    As, Bs = A.to_scipy(), None if B is None else B.to_scipy()
    BX = X if Bs is None else Bs @ X
    # the mixed solve's basis drifts from B-orthonormality (digit-plane
    # products, FP32 inner solve) to ~1e-10; ComputeW12's two nearly parallel
    # directions per pair amplify it to ~1e-9 on these cases
    orth_tol = 1e-10 if precision == "fp64" else (1e-8 if "w12" in case else 1e-9)
    assert np.abs(X.T @ BX - np.eye(nev)).max() < orth_tol
    res = np.linalg.norm(As @ X - BX * r.eval[:nev], axis=0)
    assert np.all(res <= g["tol"][1] * np.abs(r.eval[:nev]) * 1.0001)


def test_ops_path_solve_equals_one_call_solve(gpu_lib, golden):
    """The OPS entry points driven slot by slot give the GCGE_Solve result."""
    G = gpu_lib
    A = P.laplace2d(24, 24)
    X0 = P.initial_block(A.n, 12, seed=1)
    a = G.solve_ops(A, None, 8, 4, 12, 20, X0=X0)
    b = G.solve(A, None, 8, 4, 12, 20, X0=X0)
    assert a.nconv >= 8 and b.nconv >= 8 and a.niter == b.niter
    np.testing.assert_allclose(a.eval[:8], b.eval[:8], rtol=1e-13, atol=0)
    ref = np.array(golden["laplace2d_24x24_nev8"]["eval"][:8])
    assert np.max(np.abs(a.eval[:8] - ref) / ref) < 1e-10


def test_user_defined_linear_solver_hook(gpu_lib):
    """user_defined_multi_linear_solver 2 (src/ops_eig_sol_gcg.c:590-592):
    the caller's MultiLinearSolver runs on b = (lambda + sigma) B x in the
    Ritz-vector columns [offset[1], ...) with x in V[:, startW:endW], then
    BlockPCG from its result.  A solver that leaves x alone gives the plain
    solve.  With 1 the caller's solver alone builds W: five Richardson steps
    run through the backend's own OPS slots still converge, more slowly."""
    G = gpu_lib
    A = P.laplace2d(24, 24)
    X0 = P.initial_block(A.n, 12, seed=1)
    base = G.solve_ops(A, None, 8, 4, 12, 20, X0=X0, auto_shift=0)
    calls = []

    def noop(mat, b, x, start, end, ops):
        calls.append((start[0], end[0], start[1], end[1]))

    args = ("-gcge_user_defined_multi_lin_sol", "2")
    r = G.solve_ops(A, None, 8, 4, 12, 20, X0=X0, auto_shift=0, args=args, linear_solver=noop)
    assert r.nconv >= 8 and r.niter == base.niter
    np.testing.assert_array_equal(r.eval[:8], base.eval[:8])
    assert abs(len(calls) - r.niter) <= 1   # one ComputeW per outer iteration
    for s0, e0, s1, e1 in calls:
        assert e0 - s0 == e1 - s1 > 0 and s1 >= 12   # W after X (and P)

    ops_lib = G.load()
    n, omega = A.n, 0.125   # 1 / (largest Gershgorin bound of the 5-point operator)

    def richardson(mat, b, x, start, end, ops):
        """Five Richardson steps x <- x + omega (b - A x) through the backend's slots."""
        o = ctypes.cast(ops, ctypes.POINTER(G.OPSStruct)).contents
        create = ctypes.cast(o.MultiVecCreateByMat, G._FT["MultiVecCreateByMat"])
        destroy = ctypes.cast(o.MultiVecDestroy, G._FT["MultiVecDestroy"])
        matvec = ctypes.cast(o.MatDotMultiVec, G._FT["MatDotMultiVec"])
        axpby = ctypes.cast(o.MultiVecAxpby, G._FT["MultiVecAxpby"])
        I2 = ctypes.c_int * 2
        k = end[1] - start[1]
        tmp = ctypes.c_void_p()
        create(ctypes.byref(tmp), k, mat, ops)
        for _ in range(5):
            matvec(mat, x, tmp, I2(start[1], 0), I2(end[1], k), ops)
            axpby(1.0, b, -1.0, tmp, I2(start[0], 0), I2(end[0], k), ops)
            axpby(omega, tmp, 1.0, x, I2(0, start[1]), I2(k, end[1]), ops)
        destroy(ctypes.byref(tmp), k, ops)

    # user_defined_multi_linear_solver 1: the caller's solver alone builds W
    z = G.solve_ops(A, None, 8, 4, 12, 20, X0=X0, auto_shift=0, max_iter=2000,
                    args=("-gcge_user_defined_multi_lin_sol", "1"), linear_solver=richardson)
    assert ops_lib.ops_cuda_last_error() == 0
    assert z.status == G.GCGE_OK and z.nconv >= 8 and z.niter > base.niter
    np.testing.assert_allclose(z.eval[:8], base.eval[:8], rtol=1e-10, atol=0)
    assert n == 576
