"""Failure reporting without faulting the GPU: bad inputs and non-convergence
come back as status codes; a poisoned (NaN) matrix is detected on the host
from the residual norms and the solve stops with GCGE_ERR_NUMERIC; a grid
barrier of the persistent block-PCG kernel whose wait runs out returns an
error status and leaves the device usable."""
import ctypes

import numpy as np
import pytest

from gcge_gb300 import problems as P

pytestmark = pytest.mark.gpu


def test_not_converged_status(gpu_lib):
    A = P.laplace2d(24, 24)
    X0 = P.initial_block(A.n, 12, seed=1)
    r = gpu_lib.solve(A, None, 8, 4, 12, 20, X0=X0, max_iter=3)
    assert r.status == gpu_lib.GCGE_ERR_NOT_CONVERGED
    assert r.niter == 3 and r.nconv < 8


def test_nan_matrix_is_reported(gpu_lib):
    A = P.laplace2d(16, 16)
    A.data = A.data.copy()
    A.data[5] = np.nan
    X0 = P.initial_block(A.n, 12, seed=1)
    with pytest.raises(gpu_lib.GCGEError) as e:
        gpu_lib.solve(A, None, 4, 4, 12, 16, X0=X0, max_iter=20)
    assert e.value.status == 5


@pytest.mark.parametrize("args", [
    dict(nev=4, block_size=4, nev_init=20, nev_max=12),     # nevInit > nevMax
    dict(nev=4, block_size=8, nev_init=10, nev_max=12),     # nevInit < 3 bs and != nevMax
    dict(nev=4, block_size=100, nev_init=300, nev_max=300), # bs beyond the block-PCG width
])
def test_invalid_arguments(gpu_lib, args):
    A = P.laplace2d(20, 20)
    with pytest.raises(gpu_lib.GCGEError) as e:
        gpu_lib.solve(A, None, args["nev"], args["block_size"], args["nev_init"], args["nev_max"])
    assert e.value.status == 2


def test_library_recovers_after_errors(gpu_lib):
    A = P.laplace2d(24, 24)
    X0 = P.initial_block(A.n, 12, seed=1)
    with pytest.raises(gpu_lib.GCGEError):
        gpu_lib.solve(A, None, 8, 4, 30, 20)
    r = gpu_lib.solve(A, None, 8, 4, 12, 20, X0=X0)
    assert r.status == gpu_lib.GCGE_OK and r.nconv >= 8


def test_block_pcg_barrier_timeout_returns_status_and_device_stays_usable(gpu_lib):
    """One block of the persistent kernel leaves before its first grid
    barrier, so the others' bounded waits (100 ms here) run out: the call
    returns GCGE_ERR_CUDA; then the same solve without the fault, and a whole
    GCG solve, succeed."""
    G = gpu_lib
    A = P.laplace2d(200, 200)            # 1250 slices: the grid form in FP64
    rng = np.random.default_rng(3)
    b = rng.standard_normal((A.n, 8))
    ops = G.CudaOps()
    try:
        hA = ops.mat(A)
        hb = ops.multivec(hA, 8, b)
        hx = ops.multivec(hA, 8)
        st = ops.lib.GCGE_TestBlockPCGBarrierTimeout(hA, hb, hx, ctypes.c_int(8),
                                                     ctypes.c_double(100.0))
        assert st == G.GCGE_ERR_CUDA
        it = ctypes.c_int()
        st = ops.lib.GCGE_BlockPCG(hA, None, ctypes.c_double(0.0), hb, hx, ctypes.c_int(8),
                                   ctypes.c_int(30), ctypes.c_double(1e-2),
                                   ctypes.c_double(1e-14), ctypes.c_int(0), ctypes.byref(it))
        assert st == G.GCGE_OK and it.value > 0
    finally:
        ops.close()
    X0 = P.initial_block(576, 12, seed=1)
    r = G.solve(P.laplace2d(24, 24), None, 8, 4, 12, 20, X0=X0)
    assert r.status == G.GCGE_OK and r.nconv >= 8
