"""Failure reporting without faulting the GPU: bad inputs and non-convergence
come back as status codes; a poisoned (NaN) matrix is detected on the host
from the residual norms and the solve stops with GCGE_ERR_NUMERIC."""
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
