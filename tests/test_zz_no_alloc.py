"""GCGE_GramNoAlloc - the Gram product for callers that may not allocate device
memory (their memory belongs to another allocator or a fixed pool, or they run
loops where an allocation's device synchronisation is not acceptable).  The
entry point takes device pointers and uses a fixed scratch array inside the
library instead of allocating.

Checked through the C ABI against the library's existing inner-product entry
point (the OPS MultiVecInnerProd slot, mode 'N') on two calls in a row with
different data, plus the size limit.  Device buffers for the caller side are
made with PyTorch (test plumbing only).  The file name makes pytest collect it
last."""
import ctypes

import numpy as np
import pytest

from gcge_gb300 import problems as P

pytestmark = pytest.mark.gpu


def _reference_gram(G, Q, Pm):
    """Q^T P through the existing entry point (OPS MultiVecInnerProd, 'N')."""
    ops = G.CudaOps()
    try:
        n = Q.shape[0]
        h = ops.mat(P.identity_diag(n))
        q = ops.multivec(h, Q.shape[1], Q)
        p = ops.multivec(h, Pm.shape[1], Pm)
        return ops.inner_prod("N", q, p, (0, 0), (Q.shape[1], Pm.shape[1]))
    finally:
        ops.close()


def _no_alloc_gram(lib, torch, Q, Pm):
    n, m = Q.shape
    w = Pm.shape[1]
    # column-major n x m == row-major (m, n)
    dq = torch.tensor(np.ascontiguousarray(Q.T), dtype=torch.float64, device="cuda")
    dp = torch.tensor(np.ascontiguousarray(Pm.T), dtype=torch.float64, device="cuda")
    dc = torch.full((w, m), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    st = lib.GCGE_GramNoAlloc(ctypes.c_int(n), ctypes.c_int(m), ctypes.c_int(w),
                              ctypes.c_void_p(dq.data_ptr()), ctypes.c_int(n),
                              ctypes.c_void_p(dp.data_ptr()), ctypes.c_int(n),
                              ctypes.c_void_p(dc.data_ptr()), ctypes.c_int(m), None)
    torch.cuda.synchronize()
    return st, dc.cpu().numpy().T


def test_gram_no_alloc_matches_inner_prod_twice(gpu_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device for the caller-side buffers")
    lib = gpu_lib.load()
    rng = np.random.default_rng(11)
    for n, m, w in [(70001, 37, 12), (40000, 120, 20)]:   # two calls in a row, new data each
        Q = rng.standard_normal((n, m))
        Pm = rng.standard_normal((n, w))
        st, C = _no_alloc_gram(lib, torch, Q, Pm)
        assert st == gpu_lib.GCGE_OK
        ref = _reference_gram(gpu_lib, Q, Pm)
        scale = np.sqrt(n)  # |Q|_col |P|_col for unit-variance entries
        assert np.all(np.isfinite(C))
        assert np.abs(C - ref).max() <= 1e-13 * scale * np.abs(ref).max() + 1e-12 * scale


def test_gram_no_alloc_rejects_oversize(gpu_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device for the caller-side buffers")
    lib = gpu_lib.load()
    d = torch.zeros((8,), dtype=torch.float64, device="cuda")
    # m * w = 1024 * 1024 > 524288 doubles of scratch: refused before any launch
    st = lib.GCGE_GramNoAlloc(ctypes.c_int(4), ctypes.c_int(1024), ctypes.c_int(1024),
                              ctypes.c_void_p(d.data_ptr()), ctypes.c_int(4),
                              ctypes.c_void_p(d.data_ptr()), ctypes.c_int(4),
                              ctypes.c_void_p(d.data_ptr()), ctypes.c_int(1024), None)
    assert st == 8  # GCGE_ERR_TOO_LARGE
