"""ctypes binding of the reference GCGE CPU path compiled from its own sources
(``oracle/ref/Makefile`` -> ``oracle/_ref/libgcge_ref.so``).

TEST INFRASTRUCTURE ONLY.  The library exists only where the reference tree
was present at build time; callers check :func:`available` first.
"""
from __future__ import annotations

import ctypes
import os
import time

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))


def reference_dir():
    """The reference source tree (GCGE_REFERENCE_DIR, else the recipe's
    default in oracle/ref/Makefile), or None where it is absent."""
    d = os.environ.get("GCGE_REFERENCE_DIR")
    if d is None:
        with open(os.path.join(_HERE, "ref", "Makefile")) as f:
            for line in f:
                if line.startswith("GCGE_REFERENCE_DIR"):
                    d = line.split("=", 1)[1].strip()
                    break
    return d if d and os.path.isdir(os.path.join(d, "src")) else None
LIB_PATH = os.path.join(_HERE, "_ref", "libgcge_ref.so")
_lib = None


def available() -> bool:
    if not os.path.exists(LIB_PATH):
        return False
    try:
        _load()
        return True
    except OSError:
        return False


def _load():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(LIB_PATH, mode=ctypes.RTLD_LOCAL)
        _lib.ref_gcg_solve.restype = ctypes.c_int
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def ref_solve(A, B, X0, nev, block_size, nev_init, nev_max, tol=(1e300, 1e-8), max_iter=500,
              gap_min=1e-5, auto_shift=1, orth=None, args=()):
    """Run the reference GCG (app_ccs backend) on CSRMatrix inputs.

    A and B are symmetric, so their CSR arrays are also their CCS arrays.
    orth = (method, block_size), e.g. ("bgs", 8), selects the orthogonalisation
    of InitializeX and ComputeW through EigenSolverSetParameters_GCG; args
    (strings, e.g. ("-gcge_compW_cg_order", "2")) go through
    EigenSolverSetParametersFromCommandLine_GCG.
    Returns (eval[nev_max], evec[n, nev_max], nconv, niter, seconds).
    """
    lib = _load()
    n = A.n
    X0 = np.asfortranarray(X0, dtype=np.float64)
    ev = np.zeros(nev_max)
    evec = np.zeros((n, nev_max), order="F")
    nc = ctypes.c_int()
    it = ctypes.c_int()
    t = time.perf_counter()
    argv = (ctypes.c_char_p * max(1, len(args)))(*[a.encode() for a in args])
    lib.ref_gcg_solve_opts(
        ctypes.c_int(n), _ptr(A.indptr), _ptr(A.indices), _ptr(A.data),
        _ptr(None if B is None else B.indptr), _ptr(None if B is None else B.indices),
        _ptr(None if B is None else B.data),
        ctypes.c_int(nev), ctypes.c_int(block_size), ctypes.c_int(nev_init), ctypes.c_int(nev_max),
        ctypes.c_int(max_iter), ctypes.c_double(tol[0]), ctypes.c_double(tol[1]),
        ctypes.c_double(gap_min), ctypes.c_int(auto_shift), _ptr(X0), ctypes.c_int(X0.shape[1]),
        _ptr(ev), _ptr(evec), ctypes.byref(nc), ctypes.byref(it),
        None if orth is None else orth[0].encode(), ctypes.c_int(0 if orth is None else orth[1]),
        ctypes.c_int(len(args)), argv)
    return ev, evec, nc.value, it.value, time.perf_counter() - t


def ref_orth(x, start, end, method, block_size, B=None, max_reorth=2,
             zero_tol=2 * np.finfo(float).eps):
    """The reference's MultiVecOrth ("bgs" or "mgs" setup) on a copy of x
    (n x m); returns (x[:, :new_end], new_end)."""
    lib = _load()
    x = np.array(x, dtype=np.float64, order="F", copy=True)
    e = ctypes.c_int(end)
    arrs = [None, None, None] if B is None else [B.indptr, B.indices, B.data]
    lib.ref_orth(ctypes.c_int(x.shape[0]), ctypes.c_int(x.shape[1]), _ptr(x), ctypes.c_int(start),
                 ctypes.byref(e), method.encode(), ctypes.c_int(block_size),
                 ctypes.c_int(max_reorth), ctypes.c_double(zero_tol), *[_ptr(a) for a in arrs])
    return x[:, :e.value].copy(), e.value


def ref_block_amg(A_list, P_list, b, x0, max_iter, rate, tol, tol_type="abs"):
    """The reference's BlockAMG (MultiLinearSolverSetup_BlockAMG and the
    solver it installs, src/ops_lin_sol.c:466-715) on the app_ccs backend,
    with a MultiVecFromItoJ written for that backend in the driver.  A_list:
    level matrices (problems.CSRMatrix, symmetric); P_list:
    problems.Transfer, P_l of n_l x n_{l+1}; b, x0: n_0 x k.  max_iter has
    2 L entries (cycles, then the pre- and post-smoothing iteration caps of
    each level; the coarsest level's single solve takes entry 2 L - 1), rate
    and tol one per level.  Returns (x, the solver's residual field)."""
    lib = _load()
    L = len(A_list)
    assert len(P_list) == L - 1 and len(max_iter) == 2 * L
    b = np.asfortranarray(b, dtype=np.float64)
    x = np.array(x0, dtype=np.float64, order="F", copy=True)
    k = b.shape[1]
    PT = [p.transpose() for p in P_list]
    keep = []

    def ptrs(arrs):
        keep.extend(arrs)
        return (ctypes.c_void_p * max(1, len(arrs)))(*[a.ctypes.data for a in arrs])

    n = np.array([a.n for a in A_list], dtype=np.int32)
    mi = np.array(max_iter, dtype=np.int32)
    ra = np.array(rate, dtype=np.float64)
    to = np.array(tol, dtype=np.float64)
    res = ctypes.c_double()
    lib.ref_block_amg(
        ctypes.c_int(L), _ptr(n),
        ptrs([a.indptr for a in A_list]), ptrs([a.indices for a in A_list]),
        ptrs([a.data for a in A_list]),
        ptrs([p.colptr for p in P_list]), ptrs([p.rowind for p in P_list]),
        ptrs([p.data for p in P_list]),
        ptrs([p.colptr for p in PT]), ptrs([p.rowind for p in PT]), ptrs([p.data for p in PT]),
        ctypes.c_int(k), _ptr(b), _ptr(x), _ptr(mi), _ptr(ra), _ptr(to), tol_type.encode(),
        ctypes.byref(res))
    return x, res.value


def ref_block_pcg(A, b, x0, sb, sx, k, max_iter, rate, tol, tol_type="abs", user_norms=None):
    """The reference's BlockPCG (src/ops_lin_sol.c:140-465) on the app_ccs
    backend: columns [sb, sb + k) of b into [sx, sx + k) of a copy of x0.
    Returns (x, niter, residual) with the solver record's fields."""
    lib = _load()
    b = np.array(b, dtype=np.float64, order="F", copy=True)
    x = np.array(x0, dtype=np.float64, order="F", copy=True)
    un = None if user_norms is None else np.ascontiguousarray(user_norms, dtype=np.float64)
    it, res = ctypes.c_int(), ctypes.c_double()
    lib.ref_block_pcg(ctypes.c_int(A.n), _ptr(A.indptr), _ptr(A.indices), _ptr(A.data),
                      ctypes.c_int(b.shape[1]), _ptr(b), ctypes.c_int(sb), ctypes.c_int(x.shape[1]),
                      _ptr(x), ctypes.c_int(sx), ctypes.c_int(k), ctypes.c_int(max_iter),
                      ctypes.c_double(rate), ctypes.c_double(tol), tol_type.encode(), _ptr(un),
                      ctypes.byref(it), ctypes.byref(res))
    return x, it.value, res.value
