"""Level transfers (CUDA_TransferCreateFromCCS + the MultiVecFromItoJ slot)
against scipy, and the block AMG solver (MultiLinearSolverSetup_BlockAMG,
src/ops_lin_sol.c:466-715) through the OPS surface against the reference's
own BlockAMG run on the same hierarchies (fixtures of
tests/golden/make_golden_amg.py) and against the CPU restatement; and the
BlockPCG residual field those cycles stop on."""
import ctypes
import json
import os

import numpy as np
import pytest

from gcge_gb300 import problems as P
from oracle.amg_oracle import block_amg as oracle_block_amg
from oracle.amg_oracle import block_pcg as oracle_block_pcg

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_transfers_match_scipy(gpu_lib):
    G = gpu_lib
    A, T = P.multigrid_2d(31, 31, 3)          # 961 -> 225 -> 49
    Ps = [t.to_scipy() for t in T]
    rng = np.random.default_rng(3)
    X = rng.standard_normal((A[0].n, 5))
    Y = rng.standard_normal((A[2].n, 4))
    ops = G.CudaOps()
    try:
        mats = [ops.mat(a) for a in A]
        trans = [ops.transfer(t) for t in T]
        x0 = ops.multivec(mats[0], 5, X)
        y1 = ops.multivec(mats[1], 6)
        ops.from_i_to_j(trans, 0, 1, x0, y1, (1, 2), (4, 5))        # restriction
        got = ops.download(y1, 0, 6)
        np.testing.assert_allclose(got[:, 2:5], Ps[0].T @ X[:, 1:4], rtol=0, atol=1e-13)
        assert np.all(got[:, :2] == 0) and np.all(got[:, 5:] == 0)
        y2 = ops.multivec(mats[2], 4, Y)
        x2 = ops.multivec(mats[0], 4)
        ws = [None, ops.multivec(mats[1], 5), None]            # intermediate level 1
        ops.from_i_to_j(trans, 2, 0, y2, x2, (0, 0), (4, 4), ws)   # two levels up
        np.testing.assert_allclose(ops.download(x2, 0, 4), Ps[0] @ (Ps[1] @ Y), rtol=0,
                                   atol=1e-13)
        z2 = ops.multivec(mats[2], 5)
        ops.from_i_to_j(trans, 0, 2, x0, z2, (0, 0), (5, 5), ws)   # two levels down
        np.testing.assert_allclose(ops.download(z2, 0, 5), Ps[1].T @ (Ps[0].T @ X), rtol=0,
                                   atol=1e-12)
    finally:
        ops.close()


def _fixtures():
    import sys
    if GOLDEN not in sys.path:
        sys.path.insert(0, GOLDEN)
    import make_golden_amg
    with open(os.path.join(GOLDEN, "golden_amg.json")) as f:
        meta = json.load(f)
    return make_golden_amg, meta, dict(np.load(os.path.join(GOLDEN, "golden_amg.npz")))


@pytest.mark.parametrize("name", ["lap2d_63_L3_fixed", "lap2d_31_L2_wide", "lap2d_63_L3_abs",
                                  "lap2d_127_L4_rel"])
def test_block_amg_matches_reference(gpu_lib, name):
    mg, meta, xs = _fixtures()
    c = meta[name]
    A, T, b, x0 = mg.inputs(c)
    x, res, cycles = gpu_lib.block_amg(A, T, b, x0, c["max_iter"], c["rate"], c["tol"],
                                       c["tol_type"])
    xr = xs[name]
    scale = np.abs(xr).max()
    if c["tol"][0] == 0:
        # rate 0 and tol 0: every level solve runs its full iteration cap, so
        # the result is a fixed polynomial in b and matches to rounding
        assert cycles == c["max_iter"][0]
        assert np.abs(x - xr).max() <= 1e-9 * scale
        assert res == pytest.approx(c["residual"], rel=1e-6)
    else:
        assert np.abs(x - xr).max() <= 1e-7 * scale
        As = A[0].to_scipy()
        r_gpu = np.linalg.norm(b - As @ x, axis=0)
        r_ref = np.linalg.norm(b - As @ xr, axis=0)
        assert np.all(r_gpu <= 10 * r_ref + 1e-12 * np.linalg.norm(b, axis=0))
        # the same stopping decision as the CPU restatement
        xo = np.array(x0, order="F", copy=True)
        res_o, cyc_o = oracle_block_amg([a.to_scipy() for a in A], [t.to_scipy() for t in T], b,
                                        xo, c["max_iter"], c["rate"], c["tol"], c["tol_type"])
        assert cycles == cyc_o
        assert res == pytest.approx(res_o, rel=1e-3)


class _BlockPCGSolver(ctypes.Structure):
    """src/ops_lin_sol.h:29-40 as include/gcge_ops.h declares it."""
    _fields_ = [("max_iter", ctypes.c_int), ("rate", ctypes.c_double), ("tol", ctypes.c_double),
                ("tol_type", ctypes.c_char * 8), ("mv_ws", ctypes.c_void_p * 3),
                ("dbl_ws", ctypes.c_void_p), ("int_ws", ctypes.c_void_p), ("pc", ctypes.c_void_p),
                ("MatDotMultiVec", ctypes.c_void_p), ("niter", ctypes.c_int),
                ("residual", ctypes.c_double)]


def test_block_pcg_residual_field_follows_the_reference_list(gpu_lib):
    """The residual field that BlockAMG's cycles stop on, from the persistent
    route on 45 columns (two launches): columns 0-39 are Laplacian
    eigenvectors and leave after one step, columns 40-44 are random and still
    iterate after 20 steps.  The reference reports the last residual of the
    first column left in its list (src/ops_lin_sol.c:406-410): column 40's,
    as the restatement does."""
    G = gpu_lib
    nx, k, steps = 40, 45, 20
    A = P.laplace2d(nx, nx)
    n = A.n

    def mode(m):
        return np.sin(np.pi * m * np.arange(1, nx + 1) / (nx + 1))

    B = np.zeros((n, k), order="F")
    for j in range(40):
        B[:, j] = np.kron(mode(1 + j // 5), mode(1 + j % 5))
    B[:, 40:] = (P.splitmix_uniform(9, n * 5, 0) - 0.5).reshape((n, 5), order="F")
    X0 = np.zeros((n, k), order="F")
    ops = G.CudaOps()
    try:
        h = ops.mat(A)
        b = ops.multivec(h, k, B)
        x = ops.multivec(h, k, X0)
        ops.lib.MultiLinearSolverSetup_BlockPCG(ctypes.c_int(steps), ctypes.c_double(0.0),
                                                ctypes.c_double(1e-9), b"abs", None, None, None,
                                                None, None, ops.ptr)
        ops.check("MultiLinearSolverSetup_BlockPCG")
        fn = ctypes.cast(ops.ptr.contents.MultiLinearSolver, G._LINSOL)
        fn(h, b, x, G._I2(0, 0), G._I2(k, k), ctypes.cast(ops.ptr, ctypes.c_void_p))
        ops.check("MultiLinearSolver")
        ws = ctypes.cast(ops.ptr.contents.multi_linear_solver_workspace,
                         ctypes.POINTER(_BlockPCGSolver)).contents
        niter, residual = ws.niter, ws.residual
    finally:
        ops.close()
    As = A.to_scipy()
    st = oracle_block_pcg(lambda v: As @ v, B, X0.copy(order="F"), steps, 0.0, 1e-9, "abs")
    assert niter == st.niter == steps
    assert residual == pytest.approx(st.residual, rel=1e-6)
    assert residual > 1e-6          # a random column's, not an eigenvector column's
