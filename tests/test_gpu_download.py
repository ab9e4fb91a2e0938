"""Device-to-host reads of multivector columns (CUDA_MultiVecGetToHost, the
counterpart of the reference's MultiVecView-style host access used by
GCGE_Solve's eigenvector output): into page-locked memory the columns are
stored by a kernel, into pageable memory by a 2D copy; both must give the
stored values for any row count, column range, host leading dimension and
host alignment."""
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


@pytest.mark.parametrize("nx,ny", [(33, 31), (32, 32)])          # n odd (1023) and even (1024)
@pytest.mark.parametrize("start,end,pad,shift", [(0, 6, 0, 0), (2, 5, 3, 1), (1, 6, 1, 0)])
def test_columns_to_pinned_and_pageable_host(ops, gpu_lib, nx, ny, start, end, pad, shift):
    G = gpu_lib
    A = P.laplace2d(nx, ny)
    n, k = A.n, 6
    rng = np.random.default_rng(nx + 7 * start + pad)
    V = rng.standard_normal((n, k))
    hA = ops.mat(A)
    mv = ops.multivec(hA, k, V)
    ldh = n + pad
    want = V[:, start:end]
    # page-locked destination, possibly starting one element into the block
    # (8-byte aligned only) and with a leading dimension other than n
    blk = G.pinned_empty(ldh * (end - start) + shift + 1)
    blk[:] = -7.0
    ptr = ctypes.c_void_p(blk.ctypes.data + 8 * shift)
    st = ops.lib.CUDA_MultiVecGetToHost(mv, start, end, ptr, ldh)
    assert st == G.GCGE_OK
    got = blk[shift:shift + ldh * (end - start)].reshape((ldh, end - start), order="F")
    np.testing.assert_array_equal(got[:n], want)
    if pad:
        assert np.all(got[n:] == -7.0)          # rows past n untouched
    assert blk[-1] == -7.0 and (shift == 0 or blk[0] == -7.0)
    # pageable destination
    out = np.full((ldh, end - start), -7.0, order="F")
    st = ops.lib.CUDA_MultiVecGetToHost(mv, start, end, out.ctypes.data_as(ctypes.c_void_p), ldh)
    assert st == G.GCGE_OK
    np.testing.assert_array_equal(out[:n], want)
