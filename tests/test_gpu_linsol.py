"""The linear-solver hook of the OPS surface: MultiLinearSolverSetup_BlockPCG
(src/ops_lin_sol.c:439-465) and the block CG it installs as
ops->MultiLinearSolver, on both of its routes (the persistent kernel on a CUDA
matrix; the reference's host-driven loop with an operator callback or "user"
norms), against the CPU restatement of BlockPCG (src/ops_lin_sol.c:140-437).
Also: the OPS slots that stage data through host buffers, called from two host
threads at once."""
import ctypes
import threading

import numpy as np
import pytest

from gcge_gb300 import problems as P
from oracle.gcg_oracle import GCGOracle, GCGParams

pytestmark = pytest.mark.gpu

_VP = ctypes.c_void_p
_IP = ctypes.POINTER(ctypes.c_int)
_OPERATOR = ctypes.CFUNCTYPE(None, _VP, _VP, _IP, _IP, _VP, ctypes.c_int, _VP)
_LINSOL = ctypes.CFUNCTYPE(None, _VP, _VP, _VP, _IP, _IP, _VP)
_I2 = ctypes.c_int * 2


class BlockPCGSolver(ctypes.Structure):
    """src/ops_lin_sol.h:29-40 as include/gcge_ops.h declares it."""
    _fields_ = [("max_iter", ctypes.c_int), ("rate", ctypes.c_double), ("tol", ctypes.c_double),
                ("tol_type", ctypes.c_char * 8), ("mv_ws", _VP * 3), ("dbl_ws", _VP),
                ("int_ws", _VP), ("pc", _VP), ("MatDotMultiVec", _VP), ("niter", ctypes.c_int),
                ("residual", ctypes.c_double)]


@pytest.fixture()
def ops(gpu_lib):
    o = gpu_lib.CudaOps()
    yield o
    o.close()


def oracle_pcg(A, b, x0, max_iter, rate, tol, tol_type):
    p = GCGParams(nev_init=1, nev_max=1, block_size=1, cg_max_iter=max_iter, cg_rate=rate,
                  cg_tol=tol, cg_tol_type=tol_type)
    o = GCGOracle(A.to_scipy(), None, p)
    x = np.array(x0, order="F", copy=True)
    it = o.block_pcg(np.asfortranarray(b), x)
    return x, it


def setup(ops, max_iter, rate, tol, tol_type, ws=None, dbl_ws=None, callback=None):
    mv_ws = None if ws is None else (_VP * 3)(*[w.value for w in ws])
    dbl = None if dbl_ws is None else dbl_ws.ctypes.data_as(_VP)
    ops.lib.MultiLinearSolverSetup_BlockPCG(
        ctypes.c_int(max_iter), ctypes.c_double(rate), ctypes.c_double(tol),
        tol_type.encode(), mv_ws, dbl, None, None, callback, ops.ptr)
    ops.check("MultiLinearSolverSetup_BlockPCG")


def solve(ops, mat, b, x, start, end):
    fn = ctypes.cast(ops.ptr.contents.MultiLinearSolver, _LINSOL)
    fn(mat, b, x, _I2(*start), _I2(*end), ctypes.cast(ops.ptr, _VP))
    ops.check("MultiLinearSolver")
    ws = ctypes.cast(ops.ptr.contents.multi_linear_solver_workspace,
                     ctypes.POINTER(BlockPCGSolver)).contents
    return ws


def problem(k, seed=0, nx=70, ny=61):
    A = P.laplace2d(nx, ny)
    rng = np.random.default_rng(seed)
    return A, rng.standard_normal((A.n, k + 3)), 0.1 * rng.standard_normal((A.n, k + 2))


@pytest.mark.parametrize("k,tol_type", [(7, "abs"), (45, "abs"), (12, "rel")])
def test_persistent_route_matches_reference_block_pcg(ops, k, tol_type):
    """No operator callback, a CUDA matrix: one persistent launch per 40
    columns (45 columns: two), b columns [2, 2+k) into x columns [1, 1+k)."""
    A, Bh, Xh = problem(k)
    hA = ops.mat(A)
    b = ops.multivec(hA, k + 3, Bh)
    x = ops.multivec(hA, k + 2, Xh)
    tol = 1e-6 if tol_type == "abs" else 1e-5
    setup(ops, 30, 1e-2, tol, tol_type)
    ws = solve(ops, hA, b, x, (2, 1), (2 + k, 1 + k))
    xr, it = oracle_pcg(A, Bh[:, 2:2 + k], Xh[:, 1:1 + k], 30, 1e-2, tol, tol_type)
    got = ops.download(x, 0, k + 2)
    np.testing.assert_array_equal(got[:, 0], Xh[:, 0])          # outside the range: kept
    np.testing.assert_array_equal(got[:, 1 + k], Xh[:, 1 + k])
    err = np.linalg.norm(got[:, 1:1 + k] - xr, axis=0) / np.linalg.norm(xr, axis=0)
    assert err.max() < 1e-9, err.max()
    assert abs(ws.niter - it) <= 1, (ws.niter, it)
    assert ws.tol_type == tol_type.encode() and ws.max_iter == 30


def test_callback_route_matches_and_calls_the_operator(ops, gpu_lib):
    """With an operator callback the reference's loop runs on the device
    multivectors and calls the callback on runs of unconverged columns: the
    callback here is the backend's own MatDotMultiVec of A, so the result must
    equal the persistent route's and the restatement's."""
    k = 9
    A, Bh, Xh = problem(k, seed=1)
    hA = ops.mat(A)
    b = ops.multivec(hA, k + 3, Bh)
    x = ops.multivec(hA, k + 2, Xh)
    ws = [ops.multivec(hA, k) for _ in range(3)]
    calls = []
    mat_dot = ops._fn("MatDotMultiVec")

    def op(xp, yp, start, end, z, s, opsp):
        calls.append((start[0], end[0], start[1], end[1], s))
        mat_dot(hA, xp, yp, _I2(start[0], start[1]), _I2(end[0], end[1]), opsp)

    cb = _OPERATOR(op)
    setup(ops, 30, 1e-2, 1e-6, "abs", ws=ws, callback=cb)
    res = solve(ops, None, b, x, (2, 1), (2 + k, 1 + k))
    xr, it = oracle_pcg(A, Bh[:, 2:2 + k], Xh[:, 1:1 + k], 30, 1e-2, 1e-6, "abs")
    got = ops.download(x, 1, 1 + k)
    err = np.linalg.norm(got - xr, axis=0) / np.linalg.norm(xr, axis=0)
    assert err.max() < 1e-9, err.max()
    assert res.niter == it
    # first call: the initial residual, x columns [1, 1+k) -> r columns [0, k)
    assert calls[0] == (1, 1 + k, 0, k, 0)
    # then one call per iteration and run, p -> w on the same columns, b as scratch from 2
    assert all(c[4] == 2 and c[0] == c[2] and c[1] == c[3] for c in calls[1:])
    assert len(calls) >= 1 + it


def test_user_norms_route(ops):
    """tol_type "user": norm_b[i] = |dbl_ws[i]| (here ||b_i||, so the result
    equals the "rel" solve of the restatement)."""
    k = 6
    A, Bh, Xh = problem(k, seed=2)
    hA = ops.mat(A)
    b = ops.multivec(hA, k + 3, Bh)
    x = ops.multivec(hA, k + 2, Xh)
    ws = [ops.multivec(hA, k) for _ in range(3)]
    norms = -np.linalg.norm(Bh[:, 0:k], axis=0)   # the sign is dropped
    dbl = np.concatenate([norms, np.zeros(6 * k)])
    setup(ops, 30, 1e-2, 1e-5, "user", ws=ws, dbl_ws=dbl)
    res = solve(ops, hA, b, x, (0, 0), (k, k))
    xr, it = oracle_pcg(A, Bh[:, 0:k], Xh[:, 0:k], 30, 1e-2, 1e-5, "rel")
    got = ops.download(x, 0, k)
    err = np.linalg.norm(got - xr, axis=0) / np.linalg.norm(xr, axis=0)
    assert err.max() < 1e-9 and res.niter == it


def test_solver_without_setup_reports_an_error(ops, gpu_lib):
    """ops->MultiLinearSolver of another ops' setup: a status, no crash."""
    A, Bh, Xh = problem(3)
    other = gpu_lib.CudaOps()
    try:
        setup(other, 30, 1e-2, 1e-6, "abs")
        hA = ops.mat(A)
        b = ops.multivec(hA, 6, Bh)
        x = ops.multivec(hA, 5, Xh)
        fn = ctypes.cast(other.ptr.contents.MultiLinearSolver, _LINSOL)
        fn(hA, b, x, _I2(0, 0), _I2(3, 3), ctypes.cast(ops.ptr, _VP))
        assert ops.lib.ops_cuda_last_error() == gpu_lib.GCGE_ERR_ARG
    finally:
        other.close()


def test_slots_from_two_threads_at_once(gpu_lib):
    """MultiVecLinearComb and MultiVecInnerProd stage coefficients and results
    through host and device buffers; each host thread (and device) has its
    own, so two threads calling the slots at once of different sizes get their
    own correct results."""
    errors = []

    def worker(seed, n1, ncx, ncy):
        ops = gpu_lib.CudaOps()
        try:
            A = P.laplace2d(n1, 17)
            rng = np.random.default_rng(seed)
            X = rng.standard_normal((A.n, ncx))
            Y = rng.standard_normal((A.n, ncy))
            hA = ops.mat(A)
            x = ops.multivec(hA, ncx, X)
            y = ops.multivec(hA, ncy, Y)
            for it in range(40):
                C = rng.standard_normal((ncx, ncy))
                beta = rng.standard_normal(ncy)
                ops.upload(y, Y)
                ops.linear_comb(x, y, (0, 0), (ncx, ncy), coef=C, ldc=ncx, beta=beta, incb=1)
                want = X @ C + Y * beta
                got = ops.download(y, 0, ncy)
                g = ops.inner_prod("N", x, y, (0, 0), (ncx, ncy))
                if np.abs(got - want).max() > 1e-10 * np.abs(want).max():
                    errors.append((seed, it, "lincomb"))
                if np.abs(g - X.T @ want).max() > 1e-9 * np.abs(X.T @ want).max():
                    errors.append((seed, it, "inner"))
        except Exception as e:  # reported by the main thread
            errors.append((seed, repr(e)))
        finally:
            ops.close()

    ts = [threading.Thread(target=worker, args=(1, 300, 24, 31)),
          threading.Thread(target=worker, args=(2, 41, 5, 3))]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert not errors, errors[:5]
