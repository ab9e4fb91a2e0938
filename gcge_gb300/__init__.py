"""gcge_gb300 - GB300-native (sm_103a) GCG block eigensolver behind GCGE's
OPS plugin surface.

The product is the C-ABI shared library ``libgcge_cuda.so`` (declared in
``include/gcge_ops.h`` and ``include/gcge_cuda.h``).  This module is the thin
Python host side over it, mirroring the reference's call sequence
(OPS_Create / OPS_CUDA_Set / OPS_Setup, MultiVecCreateByMat, GCGE_Create,
EigenSolverSetup_GCG, GCGE_Setparameters, ops->EigenSolver; gcge.c:490-531),
plus one-call helpers.  It needs no PyTorch: device memory, the stream and
timing live in the library.  If the library is missing, every entry point
raises - there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field

import numpy as np

from . import problems  # noqa: F401  (re-export)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgcge_cuda.so")

GCGE_OK = 0
GCGE_ERR_CUDA = 1
GCGE_ERR_ARG = 2
GCGE_ERR_NOT_CONVERGED = 6
PREC_FP64 = 0
PREC_MIXED = 1

# Every symbol include/*.h declares (checked by the CPU tests).
EXPORTED_SYMBOLS = [
    "OPS_Create", "OPS_Setup", "OPS_Destroy", "OPS_CUDA_Set",
    "EigenSolverSetup_GCG", "EigenSolverCreateWorkspace_GCG", "EigenSolverDestroyWorkspace_GCG",
    "EigenSolverSetParameters_GCG", "GCGE_Create", "GCGE_Setparameters", "GCGE_Destroymvws",
    "ops_cuda_last_error", "ops_cuda_error_string", "ops_cuda_last_error_detail",
    "CUDA_MatCreateFromCCS", "CUDA_MatDestroy",
    "CUDA_MatNnz", "CUDA_MultiVecSetFromHost", "CUDA_MultiVecGetToHost", "CUDA_MultiVecSize",
    "GCGE_SetPrecision", "GCGE_Solve", "GCGE_GetSolveInfo", "GCGE_Prepare", "GCGE_PreparedSolve",
    "GCGE_PreparedDestroy", "GCGE_BenchSpMM", "GCGE_DenseEig", "GCGE_BlockPCG", "GCGE_BOrth",
    "GCGE_TimerStart", "GCGE_TimerStop", "GCGE_GramNoAlloc", "GCGE_DenseGram",
    "GCGE_DenseLinComb", "GCGE_HostAlloc", "GCGE_HostFree", "GCGE_ServerCreate",
    "GCGE_ServerSubmit", "GCGE_ServerWait", "GCGE_ServerDestroy", "GCGE_SolveBatch",
    "MultiVecOrthSetup_ModifiedGramSchmidt", "MultiVecOrthSetup_BinaryGramSchmidt",
    "EigenSolverSetParametersFromCommandLine_GCG", "CUDA_MatAxpby",
    "MultiLinearSolverSetup_BlockPCG", "GCGE_TestBlockPCGBarrierTimeout",
    "GCGE_BenchDenseProduct", "GCGE_SetSpMMTuning", "GCGE_SpMMTuneCandidates", "GCGE_SpMMTune",
    "CUDA_TransferCreateFromCCS", "CUDA_TransferDestroy", "CUDA_MultiVecFromItoJ",
    "MultiLinearSolverSetup_BlockAMG",
]

_lib = None


class GCGEError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        msg = _status_string(status) if _lib is not None else str(status)
        detail = ""
        if _lib is not None:
            f = _lib.ops_cuda_last_error_detail
            f.restype = ctypes.c_char_p
            detail = (f() or b"").decode(errors="replace")
        super().__init__(f"{what}: status {status} ({msg}) {detail}")
        self.status = status


def _status_string(s: int) -> str:
    f = _lib.ops_cuda_error_string
    f.restype = ctypes.c_char_p
    return f(ctypes.c_int(s)).decode()


class SolveInfo(ctypes.Structure):
    _fields_ = [("nconv", ctypes.c_int), ("niter", ctypes.c_int), ("status", ctypes.c_int),
                ("pcg_iters", ctypes.c_int), ("spmm_calls", ctypes.c_int),
                ("kernel_launches", ctypes.c_int), ("seconds", ctypes.c_double),
                ("phase_ms", ctypes.c_double * 10), ("pcg_spmm_launches", ctypes.c_int),
                ("pcg_spmm_ms", ctypes.c_double), ("pcg_spmm_bytes", ctypes.c_double),
                ("pcg_kernel_launches", ctypes.c_int), ("pcg_kernel_ms", ctypes.c_double),
                ("pcg_kernel_bytes", ctypes.c_double), ("precision_escalation_iter", ctypes.c_int)]

    PHASES = ("checkconv", "compP", "compRR", "rr_matW", "eig", "compRV", "compW", "linsol",
              "compX", "initX")

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k in ("nconv", "niter", "status", "pcg_iters", "spmm_calls",
                                           "kernel_launches", "seconds", "pcg_spmm_launches",
                                           "pcg_spmm_ms", "pcg_spmm_bytes",
                                           "pcg_kernel_launches", "pcg_kernel_ms",
                                           "pcg_kernel_bytes", "precision_escalation_iter")}
        d["phase_ms"] = {p: self.phase_ms[i] for i, p in enumerate(self.PHASES)}
        return d


def lib_path() -> str:
    return LIB_PATH


def load(build_if_missing: bool = False) -> ctypes.CDLL:
    """Load libgcge_cuda.so (RTLD_GLOBAL is not needed: one library)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if build_if_missing:
            from .build import build
            build()
        else:
            raise ImportError(f"{LIB_PATH} is missing: run gcge_gb300.build.build() (nvcc, sm_103a)")
    lib = ctypes.CDLL(LIB_PATH)
    for name in ("CUDA_MatCreateFromCCS", "CUDA_MultiVecSetFromHost", "CUDA_MultiVecGetToHost",
                 "GCGE_Solve", "GCGE_Prepare", "GCGE_PreparedSolve", "GCGE_SetPrecision",
                 "GCGE_GetSolveInfo", "GCGE_BenchSpMM", "ops_cuda_last_error", "CUDA_MultiVecSize",
                 "CUDA_MatNnz", "GCGE_DenseEig", "GCGE_BlockPCG", "GCGE_BOrth",
                 "GCGE_TimerStart", "GCGE_GramNoAlloc", "GCGE_DenseGram", "GCGE_DenseLinComb",
                 "GCGE_SetSpMMTuning", "GCGE_SpMMTuneCandidates", "GCGE_SpMMTune"):
        getattr(lib, name).restype = ctypes.c_int
    lib.GCGE_TimerStop.restype = ctypes.c_double
    lib.GCGE_HostAlloc.restype = ctypes.c_void_p
    lib.GCGE_HostAlloc.argtypes = [ctypes.c_size_t]
    lib.GCGE_HostFree.argtypes = [ctypes.c_void_p]
    lib.GCGE_ServerCreate.restype = ctypes.c_void_p
    lib.GCGE_ServerCreate.argtypes = [ctypes.c_int, ctypes.c_size_t]
    lib.GCGE_ServerSubmit.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    lib.GCGE_ServerWait.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    lib.GCGE_ServerDestroy.argtypes = [ctypes.c_void_p]
    lib.GCGE_SolveBatch.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_size_t]
    for name in ("GCGE_ServerSubmit", "GCGE_ServerWait", "GCGE_SolveBatch"):
        getattr(lib, name).restype = ctypes.c_int
    _lib = lib
    return lib


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _csr_args(M):
    if M is None:
        return None, None, None
    return (np.ascontiguousarray(M.indptr, dtype=np.int32),
            np.ascontiguousarray(M.indices, dtype=np.int32),
            np.ascontiguousarray(M.data, dtype=np.float64))


@dataclass
class SolveResult:
    eval: np.ndarray
    evec: np.ndarray | None
    nconv: int
    niter: int
    status: int
    info: dict = field(default_factory=dict)


class _HostBlock:
    """Owner of a GCGE_HostAlloc block; frees it when the last view goes."""

    def __init__(self, nbytes):
        self.lib = load()
        self.ptr = self.lib.GCGE_HostAlloc(ctypes.c_size_t(max(int(nbytes), 1)))
        if not self.ptr:
            raise GCGEError(3, "GCGE_HostAlloc")

    def __del__(self):
        if getattr(self, "ptr", None):
            self.lib.GCGE_HostFree(ctypes.c_void_p(self.ptr))
            self.ptr = None


def pinned_empty(shape, dtype=np.float64, order="C"):
    """numpy array in page-locked host memory (GCGE_HostAlloc)."""
    dtype = np.dtype(dtype)
    shape = (shape,) if np.isscalar(shape) else tuple(shape)
    count = int(np.prod(shape)) if shape else 1
    owner = _HostBlock(count * dtype.itemsize)
    buf = (ctypes.c_char * max(count * dtype.itemsize, 1)).from_address(owner.ptr)
    buf._gcge_owner = owner  # the array's base is buf: the block lives as long as the array
    return np.frombuffer(buf, dtype=dtype, count=count).reshape(shape, order=order)


def pinned_copy(a, order="C"):
    """Copy of a numpy array in page-locked host memory."""
    a = np.asarray(a)
    out = pinned_empty(a.shape, a.dtype, order=order)
    out[...] = a
    return out


def solve(A, B, nev, block_size, nev_init, nev_max, X0=None, tol=(1e300, 1e-8), max_iter=500,
          gap_min=1e-5, auto_shift=1, precision=PREC_FP64, want_evec=True, evec_out=None,
          eval_out=None) -> SolveResult:
    """One GCG solve through GCGE_Solve.  A, B: problems.CSRMatrix (symmetric,
    so CSR arrays == CCS arrays); B None = identity.  X0 (n x k) seeds the basis.
    evec_out (n x nev_max, column-major) and eval_out (nev_max) may be given to
    receive the results in caller memory (e.g. pinned_empty buffers)."""
    lib = load()
    n = A.n
    a = _csr_args(A)
    b = _csr_args(B)
    X0 = None if X0 is None else np.asfortranarray(X0, dtype=np.float64)
    ng = 0 if X0 is None else X0.shape[1]
    ev = np.zeros(nev_max) if eval_out is None else eval_out
    if evec_out is not None:
        assert evec_out.shape == (n, nev_max) and evec_out.flags.f_contiguous
        evec = evec_out
    else:
        evec = np.zeros((n, nev_max), order="F") if want_evec else None
    info = SolveInfo()
    t = (ctypes.c_double * 2)(*tol)
    st = lib.GCGE_Solve(ctypes.c_int(n), _p(a[0]), _p(a[1]), _p(a[2]), _p(b[0]), _p(b[1]), _p(b[2]),
                        ctypes.c_int(nev), ctypes.c_int(block_size), ctypes.c_int(nev_init),
                        ctypes.c_int(nev_max), ctypes.c_int(max_iter), t, ctypes.c_double(gap_min),
                        ctypes.c_int(auto_shift), ctypes.c_int(precision), _p(X0), ctypes.c_int(ng),
                        _p(ev), _p(evec), ctypes.byref(info))
    if st not in (GCGE_OK, GCGE_ERR_NOT_CONVERGED):
        raise GCGEError(st, "GCGE_Solve")
    return SolveResult(ev, evec, info.nconv, info.niter, st, info.as_dict())


def solve_ops(A, B, nev, block_size, nev_init, nev_max, X0=None, tol=(1e300, 1e-8), max_iter=500,
              gap_min=1e-5, auto_shift=1, precision=PREC_FP64, orth=None,
              args=(), linear_solver=None) -> SolveResult:
    """One GCG solve driven slot by slot through the OPS entry points, in the
    order of the reference's front end (gcge.c:490-531): OPS_CUDA_Set,
    MultiVecCreateByMat for evec, GCGE_Create, EigenSolverSetup_GCG,
    GCGE_Setparameters, then ops->EigenSolver.  orth = (method, block_size),
    e.g. ("bgs", -1), selects the orthogonalisation of InitializeX and
    ComputeW through EigenSolverSetParameters_GCG (src/ops_eig_sol_gcg.c:1684-1741);
    args, e.g. ("-gcge_compW_cg_order", "2"), then go through
    EigenSolverSetParametersFromCommandLine_GCG (:1743-1862).  linear_solver,
    a Python callable (mat, b, x, start, end, ops) with start/end int[2], is
    installed as ops->MultiLinearSolver for -gcge_user_defined_multi_lin_sol
    1 or 2 (:590-592)."""
    ops = CudaOps()
    lib = ops.lib
    try:
        hA = ops.mat(A)
        hB = ops.mat(B) if B is not None else None
        evec = ops.multivec(hA, nev_max)
        ng = 0
        if X0 is not None:
            ops.upload(evec, X0)
            ng = X0.shape[1]
        mv_ws = (_VP * 4)()
        lib.GCGE_Create(hA, ctypes.c_int(nev_max), ctypes.c_int(block_size), ctypes.c_int(nev_init),
                        mv_ws, None, None, ops.ptr)
        ops.check("GCGE_Create")
        t = (ctypes.c_double * 2)(*tol)
        lib.EigenSolverSetup_GCG(ctypes.c_double(gap_min), ctypes.c_int(nev_init),
                                 ctypes.c_int(nev_max), ctypes.c_int(block_size), t,
                                 ctypes.c_int(max_iter), 0, 0, 0, mv_ws, None, None, ops.ptr)
        lib.GCGE_Setparameters(ctypes.c_double(gap_min), ctypes.c_int(auto_shift), ops.ptr)
        if orth is not None:
            m, bs = orth[0].encode(), ctypes.c_int(orth[1])
            z = ctypes.c_double(0.0)
            lib.EigenSolverSetParameters_GCG(0, m, bs, -1, z, None, -1, -1, z, m, bs, -1, z, 0, z, z,
                                             None, ctypes.c_int(auto_shift), 0, z, z, ops.ptr)
        if args:
            argv = (ctypes.c_char_p * len(args))(*[a.encode() for a in args])
            lib.EigenSolverSetParametersFromCommandLine_GCG(ctypes.c_int(len(args)), argv, ops.ptr)
        st = lib.GCGE_SetPrecision(ops.ptr, ctypes.c_int(precision))
        if st != GCGE_OK:
            raise GCGEError(st, "GCGE_SetPrecision")
        ops.check("GCG setup")
        if linear_solver is not None:
            cb = _LINSOL(linear_solver)
            ops._keep = cb
            ops.ptr.contents.MultiLinearSolver = ctypes.cast(cb, _VP)
        ev = np.zeros(nev_max)
        nconv = ctypes.c_int(nev)
        ops._fn("EigenSolver")(hA, hB, ev.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), evec, ng,
                               ctypes.byref(nconv), ctypes.cast(ops.ptr, _VP))
        err = lib.ops_cuda_last_error()
        if err != GCGE_OK:
            raise GCGEError(err, "ops->EigenSolver")
        info = SolveInfo()
        lib.GCGE_GetSolveInfo(ops.ptr, ctypes.byref(info))
        X = ops.download(evec, 0, nev_max)
        lib.GCGE_Destroymvws(mv_ws, None, None, ctypes.c_int(nev_max), ctypes.c_int(block_size),
                             ops.ptr)
        return SolveResult(ev, X, nconv.value, info.niter, info.status, info.as_dict())
    finally:
        ops.close()


class Prepared:
    """A problem resident in HBM: matrices, initial block and solver state.
    ``solve()`` times device work only (inputs already on the GPU)."""

    def __init__(self, A, B, nev, block_size, nev_init, nev_max, X0=None, tol=(1e300, 1e-8),
                 max_iter=500, gap_min=1e-5, auto_shift=1, precision=PREC_FP64):
        lib = load()
        self.lib = lib
        self.n, self.nev_max = A.n, nev_max
        a = _csr_args(A)
        b = _csr_args(B)
        X0 = None if X0 is None else np.asfortranarray(X0, dtype=np.float64)
        ng = 0 if X0 is None else X0.shape[1]
        self.handle = ctypes.c_void_p()
        t = (ctypes.c_double * 2)(*tol)
        st = lib.GCGE_Prepare(ctypes.byref(self.handle), ctypes.c_int(A.n), _p(a[0]), _p(a[1]),
                              _p(a[2]), _p(b[0]), _p(b[1]), _p(b[2]), ctypes.c_int(nev),
                              ctypes.c_int(block_size), ctypes.c_int(nev_init),
                              ctypes.c_int(nev_max), ctypes.c_int(max_iter), t,
                              ctypes.c_double(gap_min), ctypes.c_int(auto_shift),
                              ctypes.c_int(precision), _p(X0), ctypes.c_int(ng))
        if st != GCGE_OK:
            raise GCGEError(st, "GCGE_Prepare")

    def solve(self, want_evec=False) -> SolveResult:
        ev = np.zeros(self.nev_max)
        evec = np.zeros((self.n, self.nev_max), order="F") if want_evec else None
        info = SolveInfo()
        st = self.lib.GCGE_PreparedSolve(self.handle, _p(ev), _p(evec), ctypes.byref(info))
        if st not in (GCGE_OK, GCGE_ERR_NOT_CONVERGED):
            raise GCGEError(st, "GCGE_PreparedSolve")
        return SolveResult(ev, evec, info.nconv, info.niter, st, info.as_dict())

    def close(self):
        if self.handle:
            self.lib.GCGE_PreparedDestroy(ctypes.byref(self.handle))
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# Many solves on one GPU: batched problems and the serving loop (serve.cu)
# ---------------------------------------------------------------------------
class Request(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int), ("a_colptr", ctypes.c_void_p), ("a_rowind", ctypes.c_void_p),
                ("a_val", ctypes.c_void_p), ("b_colptr", ctypes.c_void_p),
                ("b_rowind", ctypes.c_void_p), ("b_val", ctypes.c_void_p), ("nev", ctypes.c_int),
                ("block_size", ctypes.c_int), ("nev_init", ctypes.c_int), ("nev_max", ctypes.c_int),
                ("max_iter", ctypes.c_int), ("tol", ctypes.c_double * 2), ("gap_min", ctypes.c_double),
                ("auto_shift", ctypes.c_int), ("precision", ctypes.c_int), ("X0", ctypes.c_void_p),
                ("nev_given", ctypes.c_int), ("eval", ctypes.c_void_p), ("evec", ctypes.c_void_p),
                ("info", SolveInfo), ("status", ctypes.c_int), ("done", ctypes.c_int),
                ("t_submit", ctypes.c_double), ("t_start", ctypes.c_double),
                ("t_end", ctypes.c_double)]


class Job:
    """One solve for the server: the request and the arrays it points to."""

    def __init__(self, A, B, nev, block_size, nev_init, nev_max, X0=None, tol=(1e300, 1e-8),
                 max_iter=500, gap_min=1e-5, auto_shift=1, precision=PREC_MIXED, want_evec=False):
        self.arrays = [_csr_args(A), _csr_args(B)]
        a, b = self.arrays
        self.X0 = None if X0 is None else np.asfortranarray(X0, dtype=np.float64)
        self.eval = np.zeros(nev_max)
        self.evec = np.zeros((A.n, nev_max), order="F") if want_evec else None
        r = Request()
        r.n = A.n
        r.a_colptr, r.a_rowind, r.a_val = (x.ctypes.data for x in a)
        if B is not None:
            r.b_colptr, r.b_rowind, r.b_val = (x.ctypes.data for x in b)
        r.nev, r.block_size, r.nev_init, r.nev_max, r.max_iter = nev, block_size, nev_init, nev_max, max_iter
        r.tol[0], r.tol[1] = tol
        r.gap_min, r.auto_shift, r.precision = gap_min, auto_shift, precision
        if self.X0 is not None:
            r.X0, r.nev_given = self.X0.ctypes.data, self.X0.shape[1]
        r.eval = self.eval.ctypes.data
        r.evec = None if self.evec is None else self.evec.ctypes.data
        self.req = r

    @property
    def result(self) -> SolveResult:
        r = self.req
        return SolveResult(self.eval, self.evec, r.info.nconv, r.info.niter, r.status,
                           r.info.as_dict())

    @property
    def latency(self) -> float:
        return self.req.t_end - self.req.t_submit


class Server:
    """Serving loop: requests submitted at any time run on `workers` host
    threads (one CUDA stream each), admitted by device-memory footprint."""

    def __init__(self, workers=4, budget_bytes=0):
        self.lib = load()
        self.h = self.lib.GCGE_ServerCreate(workers, budget_bytes)
        if not self.h:
            raise GCGEError(self.lib.ops_cuda_last_error(), "GCGE_ServerCreate")

    def submit(self, job: Job):
        st = self.lib.GCGE_ServerSubmit(self.h, ctypes.byref(job.req))
        if st != GCGE_OK:
            raise GCGEError(st, "GCGE_ServerSubmit")
        return job

    def wait(self, job: Job) -> SolveResult:
        self.lib.GCGE_ServerWait(self.h, ctypes.byref(job.req))
        return job.result

    def close(self):
        if self.h:
            hp = ctypes.c_void_p(self.h)
            self.lib.GCGE_ServerDestroy(ctypes.byref(hp))
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def solve_batch(jobs, workers=4, budget_bytes=0):
    """Solve a list of Jobs through GCGE_SolveBatch; returns their results."""
    lib = load()
    arr = (Request * len(jobs))()
    for i, j in enumerate(jobs):
        arr[i] = j.req
    lib.GCGE_SolveBatch(arr, len(jobs), workers, budget_bytes)
    for i, j in enumerate(jobs):
        j.req = arr[i]
    return [j.result for j in jobs]


# ---------------------------------------------------------------------------
# OPS vtable access, for callers that drive the backend slot by slot
# ---------------------------------------------------------------------------
_OPS_FIELDS = [
    "Printf", "GetWtime", "GetOptionFromCommandLine", "MatView", "MatAxpby", "VecCreateByMat",
    "VecCreateByVec", "VecDestroy", "VecView", "VecInnerProd", "VecLocalInnerProd",
    "VecSetRandomValue", "VecAxpby", "MatDotVec", "MatTransDotVec", "MultiVecCreateByMat",
    "MultiVecCreateByVec", "MultiVecCreateByMultiVec", "MultiVecDestroy", "GetVecFromMultiVec",
    "RestoreVecForMultiVec", "MultiVecView", "MultiVecLocalInnerProd", "MultiVecInnerProd",
    "MultiVecSetRandomValue", "MultiVecAxpby", "MultiVecLinearComb", "MatDotMultiVec",
    "MatTransDotMultiVec", "MultiVecQtAP", "lapack_ops", "DenseMatQtAP", "DenseMatOrth",
    "LinearSolver", "linear_solver_workspace", "MultiLinearSolver",
    "multi_linear_solver_workspace", "MultiVecOrth", "orth_workspace", "MultiGridCreate",
    "MultiGridDestroy", "VecFromItoJ", "MultiVecFromItoJ", "EigenSolver",
    "eigen_solver_workspace", "app_ops",
]


class OPSStruct(ctypes.Structure):
    """Layout of struct OPS_ (src/ops.h:43-152): 46 pointer-sized members."""
    _fields_ = [(f, ctypes.c_void_p) for f in _OPS_FIELDS]


_I2 = ctypes.c_int * 2
_VP = ctypes.c_void_p
_FT = {
    "MultiVecCreateByMat": ctypes.CFUNCTYPE(None, ctypes.POINTER(_VP), ctypes.c_int, _VP, _VP),
    "MultiVecDestroy": ctypes.CFUNCTYPE(None, ctypes.POINTER(_VP), ctypes.c_int, _VP),
    "MultiVecAxpby": ctypes.CFUNCTYPE(None, ctypes.c_double, _VP, ctypes.c_double, _VP, _I2, _I2, _VP),
    "MultiVecLinearComb": ctypes.CFUNCTYPE(None, _VP, _VP, ctypes.c_int, _I2, _I2,
                                           ctypes.POINTER(ctypes.c_double), ctypes.c_int,
                                           ctypes.POINTER(ctypes.c_double), ctypes.c_int, _VP),
    "MultiVecInnerProd": ctypes.CFUNCTYPE(None, ctypes.c_char, _VP, _VP, ctypes.c_int, _I2, _I2,
                                          ctypes.POINTER(ctypes.c_double), ctypes.c_int, _VP),
    "MatDotMultiVec": ctypes.CFUNCTYPE(None, _VP, _VP, _VP, _I2, _I2, _VP),
    "MultiVecQtAP": ctypes.CFUNCTYPE(None, ctypes.c_char, ctypes.c_char, _VP, _VP, _VP,
                                     ctypes.c_int, _I2, _I2, ctypes.POINTER(ctypes.c_double),
                                     ctypes.c_int, _VP, _VP),
    "MultiVecSetRandomValue": ctypes.CFUNCTYPE(None, _VP, ctypes.c_int, ctypes.c_int, _VP),
    "MultiVecOrth": ctypes.CFUNCTYPE(None, _VP, ctypes.c_int, ctypes.POINTER(ctypes.c_int), _VP,
                                     _VP),
    "EigenSolver": ctypes.CFUNCTYPE(None, _VP, _VP, ctypes.POINTER(ctypes.c_double), _VP,
                                    ctypes.c_int, ctypes.POINTER(ctypes.c_int), _VP),
    "MultiVecFromItoJ": ctypes.CFUNCTYPE(None, _VP, ctypes.c_int, ctypes.c_int, _VP, _VP, _I2, _I2,
                                         _VP, _VP),
}


class BlockAMGSolver(ctypes.Structure):
    """src/ops_lin_sol.h:41-47 as include/gcge_ops.h declares it."""
    _fields_ = [("max_iter", _VP), ("rate", _VP), ("tol", _VP), ("tol_type", ctypes.c_char * 8),
                ("A_array", _VP), ("P_array", _VP), ("num_levels", ctypes.c_int),
                ("mv_array_ws", _VP * 5), ("dbl_ws", _VP), ("int_ws", _VP), ("pc", _VP),
                ("niter", ctypes.c_int), ("residual", ctypes.c_double)]


class AMGArrays:
    """The argument arrays of MultiLinearSolverSetup_BlockAMG (the library
    keeps pointers to them, so they live as long as the solver is used):
    level matrix handles, transfer handles, per-level workspace handles
    (ws[i][l], i < 5), iteration caps, rates, tolerances and the BlockPCG
    double / int workspaces for blocks of up to k columns."""

    def __init__(self, mats, transfers, ws, max_iter, rate, tol, k):
        L = len(mats)
        if len(transfers) != L - 1 or len(ws) != 5 or any(len(w) != L for w in ws):
            raise ValueError("hierarchy: L matrices, L - 1 transfers, 5 x L workspaces")
        if len(max_iter) != 2 * L or len(rate) != L or len(tol) != L:
            raise ValueError("max_iter needs 2 L entries, rate and tol L each")
        self.L = L
        self.A = (_VP * L)(*[_handle(m) for m in mats])
        self.P = (_VP * max(1, L - 1))(*[_handle(t) for t in transfers])
        self.levels = [(_VP * L)(*[_handle(w) for w in row]) for row in ws]
        self.ws = (_VP * 5)(*[ctypes.addressof(a) for a in self.levels])
        self.max_iter = (ctypes.c_int * (2 * L))(*[int(v) for v in max_iter])
        self.rate = (ctypes.c_double * L)(*[float(v) for v in rate])
        self.tol = (ctypes.c_double * L)(*[float(v) for v in tol])
        self.dbl = (ctypes.c_double * (8 * k + 64))()
        self.int = (ctypes.c_int * (4 * k + 64))()

    def setup(self, lib, ops_ptr, tol_type="abs"):
        """MultiLinearSolverSetup_BlockAMG(max_iter, rate, tol, tol_type,
        A_array, P_array, L, mv_array_ws, dbl_ws, int_ws, NULL, ops)."""
        lib.MultiLinearSolverSetup_BlockAMG(self.max_iter, self.rate, self.tol, tol_type.encode(),
                                            self.A, self.P, ctypes.c_int(self.L), self.ws,
                                            self.dbl, self.int, None, ops_ptr)


def _handle(h):
    return h.value if isinstance(h, ctypes.c_void_p) else h


# ops->MultiLinearSolver (src/ops.h:121-122)
_LINSOL = ctypes.CFUNCTYPE(None, _VP, _VP, _VP, ctypes.POINTER(ctypes.c_int),
                           ctypes.POINTER(ctypes.c_int), _VP)


class CudaOps:
    """OPS filled by OPS_CUDA_Set, with numpy-friendly wrappers of its slots
    (the same slot names and argument meaning as the reference's OPS)."""

    def __init__(self):
        lib = load()
        self.lib = lib
        self.ptr = ctypes.POINTER(OPSStruct)()
        lib.OPS_Create(ctypes.byref(self.ptr))
        lib.OPS_CUDA_Set(self.ptr)
        lib.OPS_Setup(self.ptr)
        self._mats, self._mvs, self._transfers = [], [], []

    def _fn(self, name):
        return ctypes.cast(getattr(self.ptr.contents, name), _FT[name])

    def check(self, what=""):
        st = self.lib.ops_cuda_last_error()
        if st != GCGE_OK:
            raise GCGEError(st, what)

    def mat(self, M):
        h = ctypes.c_void_p()
        a = _csr_args(M)
        st = self.lib.CUDA_MatCreateFromCCS(ctypes.byref(h), ctypes.c_int(M.n), ctypes.c_int(M.n),
                                            _p(a[0]), _p(a[1]), _p(a[2]))
        if st != GCGE_OK:
            raise GCGEError(st, "CUDA_MatCreateFromCCS")
        self._mats.append(h)
        return h

    def transfer(self, T):
        """CUDA_TransferCreateFromCCS of a problems.Transfer (P_l: n_l fine rows
        by n_{l+1} coarse columns), for the P_array of the block AMG solver."""
        h = ctypes.c_void_p()
        cp = np.ascontiguousarray(T.colptr, dtype=np.int32)
        ri = np.ascontiguousarray(T.rowind, dtype=np.int32)
        va = np.ascontiguousarray(T.data, dtype=np.float64)
        st = self.lib.CUDA_TransferCreateFromCCS(ctypes.byref(h), ctypes.c_int(T.nrows),
                                                 ctypes.c_int(T.ncols), _p(cp), _p(ri), _p(va))
        if st != GCGE_OK:
            raise GCGEError(st, "CUDA_TransferCreateFromCCS")
        self._transfers.append(h)
        return h

    def from_i_to_j(self, P_array, level_i, level_j, x, y, start, end, ws=None):
        """ops->MultiVecFromItoJ: P_array a sequence of transfer handles, ws
        (per-level multivector handles) for jumps over several levels."""
        parr = (_VP * max(1, len(P_array)))(*[h.value for h in P_array])
        warr = None if ws is None else (_VP * len(ws))(*[w.value if w else None for w in ws])
        self._fn("MultiVecFromItoJ")(parr, level_i, level_j, x, y, _I2(*start), _I2(*end), warr,
                                     ctypes.cast(self.ptr, _VP))
        self.check("MultiVecFromItoJ")

    def mat_axpby(self, alpha, X, beta, Y):
        """CUDA_MatAxpby: Y = alpha X + beta Y (the OPS MatAxpby slot)."""
        self.lib.CUDA_MatAxpby(ctypes.c_double(alpha), X, ctypes.c_double(beta), Y, self.ptr)
        self.check("CUDA_MatAxpby")

    def multivec(self, mat, ncols, host=None):
        h = _VP()
        self._fn("MultiVecCreateByMat")(ctypes.byref(h), ncols, mat, ctypes.cast(self.ptr, _VP))
        self.check("MultiVecCreateByMat")
        if host is not None:
            self.upload(h, host)
        self._mvs.append((h, ncols))
        return h

    def upload(self, mv, host, start=0):
        host = np.asfortranarray(host, dtype=np.float64)
        st = self.lib.CUDA_MultiVecSetFromHost(mv, start, start + host.shape[1], _p(host),
                                               host.shape[0])
        if st != GCGE_OK:
            raise GCGEError(st, "CUDA_MultiVecSetFromHost")

    def download(self, mv, start, end):
        nr, nc = ctypes.c_int(), ctypes.c_int()
        self.lib.CUDA_MultiVecSize(mv, ctypes.byref(nr), ctypes.byref(nc))
        out = np.zeros((nr.value, end - start), order="F")
        st = self.lib.CUDA_MultiVecGetToHost(mv, start, end, _p(out), nr.value)
        if st != GCGE_OK:
            raise GCGEError(st, "CUDA_MultiVecGetToHost")
        return out

    # slots -------------------------------------------------------------
    def axpby(self, alpha, x, beta, y, start, end):
        self._fn("MultiVecAxpby")(alpha, x, beta, y, _I2(*start), _I2(*end), ctypes.cast(self.ptr, _VP))
        self.check("MultiVecAxpby")

    def linear_comb(self, x, y, start, end, coef=None, ldc=0, beta=None, incb=0):
        c = None if coef is None else np.asfortranarray(coef, dtype=np.float64)
        b = None if beta is None else np.ascontiguousarray(beta, dtype=np.float64)
        cp = None if c is None else c.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        bp = None if b is None else b.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        self._fn("MultiVecLinearComb")(x, y, 0, _I2(*start), _I2(*end), cp, ldc, bp, incb,
                                       ctypes.cast(self.ptr, _VP))
        self.check("MultiVecLinearComb")

    def inner_prod(self, mode, x, y, start, end, ldip=None):
        nr, nc = end[0] - start[0], end[1] - start[1]
        if mode == "D":
            out = np.zeros(nc)
            ld = 1
        else:
            ld = ldip or nr
            out = np.zeros((ld, nc), order="F")
        self._fn("MultiVecInnerProd")(mode.encode(), x, y, 0, _I2(*start), _I2(*end),
                                      out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ld,
                                      ctypes.cast(self.ptr, _VP))
        self.check("MultiVecInnerProd")
        return out

    def mat_dot(self, mat, x, y, start, end):
        self._fn("MatDotMultiVec")(mat, x, y, _I2(*start), _I2(*end), ctypes.cast(self.ptr, _VP))
        self.check("MatDotMultiVec")

    def qtap(self, ntsA, mode, Q, A, P, start, end, ws, ld=None):
        nr, nc = end[0] - start[0], end[1] - start[1]
        shape = (nc, nr) if mode == "T" else (nr, nc)
        ld = ld or shape[0]
        out = np.zeros((ld, shape[1]), order="F")
        self._fn("MultiVecQtAP")(ntsA.encode(), mode.encode(), Q, A, P, 0, _I2(*start), _I2(*end),
                                 out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ld, ws,
                                 ctypes.cast(self.ptr, _VP))
        self.check("MultiVecQtAP")
        return out

    def orth_setup(self, method="bgs", block_size=-1, max_reorth=2,
                   zero_tol=2 * np.finfo(float).eps):
        """MultiVecOrthSetup_BinaryGramSchmidt / _ModifiedGramSchmidt
        (src/ops_orth.c:395-414, :625-641): installs ops->MultiVecOrth."""
        fn = {"bgs": self.lib.MultiVecOrthSetup_BinaryGramSchmidt,
              "mgs": self.lib.MultiVecOrthSetup_ModifiedGramSchmidt}[method]
        fn(ctypes.c_int(block_size), ctypes.c_int(max_reorth), ctypes.c_double(zero_tol), None,
           None, self.ptr)
        self.check("MultiVecOrthSetup")

    def orth(self, x, start, end, B=None):
        """ops->MultiVecOrth(x, start, &end, B): returns the new end."""
        e = ctypes.c_int(end)
        self._fn("MultiVecOrth")(x, start, ctypes.byref(e), B, ctypes.cast(self.ptr, _VP))
        self.check("MultiVecOrth")
        return e.value

    def set_random(self, x, start, end):
        self._fn("MultiVecSetRandomValue")(x, start, end, ctypes.cast(self.ptr, _VP))
        self.check("MultiVecSetRandomValue")

    def close(self):
        for h, nc in self._mvs:
            self._fn("MultiVecDestroy")(ctypes.byref(h), nc, ctypes.cast(self.ptr, _VP))
        for h in self._mats:
            self.lib.CUDA_MatDestroy(ctypes.byref(h))
        for h in self._transfers:
            self.lib.CUDA_TransferDestroy(ctypes.byref(h))
        self._mvs, self._mats, self._transfers = [], [], []
        if self.ptr:
            self.lib.OPS_Destroy(ctypes.byref(self.ptr))


def bench_spmm(A, k: int, fp32: bool, reps: int = 20):
    """Average ms per SpMM launch of k columns and its algorithmic bytes."""
    lib = load()
    ops = CudaOps()
    try:
        h = ops.mat(A)
        ms, by = ctypes.c_double(), ctypes.c_double()
        st = lib.GCGE_BenchSpMM(h, ctypes.c_int(k), ctypes.c_int(1 if fp32 else 0), ctypes.c_int(reps),
                                ctypes.byref(ms), ctypes.byref(by))
        if st != GCGE_OK:
            raise GCGEError(st, "GCGE_BenchSpMM")
        return ms.value, by.value
    finally:
        ops.close()


def block_amg(A_list, P_list, b, x0, max_iter, rate, tol, tol_type="abs"):
    """The block AMG solver through the OPS surface: level matrices
    (problems.CSRMatrix), transfers (problems.Transfer, P_l of n_l x n_{l+1}),
    MultiLinearSolverSetup_BlockAMG with the reference's parameter arrays
    (max_iter: cycles, then each level's pre- and post-smoothing caps; rate and
    tol per level), then ops->MultiLinearSolver on b (n_0 x k) from x0.
    Returns (x, the solver's residual field, cycles run)."""
    load()
    b = np.asfortranarray(b, dtype=np.float64)
    k = b.shape[1]
    ops = CudaOps()
    try:
        mats = [ops.mat(a) for a in A_list]
        trans = [ops.transfer(t) for t in P_list]
        ws = [[ops.multivec(m, k) for m in mats] for _ in range(5)]
        arr = AMGArrays(mats, trans, ws, max_iter, rate, tol, k)
        arr.setup(ops.lib, ops.ptr, tol_type)
        ops.check("MultiLinearSolverSetup_BlockAMG")
        bv = ops.multivec(mats[0], k, b)
        xv = ops.multivec(mats[0], k, x0)
        fn = ctypes.cast(ops.ptr.contents.MultiLinearSolver, _LINSOL)
        fn(mats[0], bv, xv, _I2(0, 0), _I2(k, k), ctypes.cast(ops.ptr, _VP))
        ops.check("MultiLinearSolver (BlockAMG)")
        g = ctypes.cast(ops.ptr.contents.multi_linear_solver_workspace,
                        ctypes.POINTER(BlockAMGSolver)).contents
        residual, cycles = g.residual, g.niter
        return ops.download(xv, 0, k), residual, cycles
    finally:
        ops.close()


def set_spmm_tuning(on: int):
    """1: tune the column split of SpMMs; 0: fixed 40-column launches;
    -1: off, and forget the tuned choices."""
    st = load().GCGE_SetSpMMTuning(ctypes.c_int(on))
    if st != GCGE_OK:
        raise GCGEError(st, "GCGE_SetSpMMTuning")


def spmm_tune_candidates(k: int) -> list:
    """Candidate launch widths of an SpMM of k columns, fewest launches first."""
    lib = load()
    buf = (ctypes.c_int * 16)()
    cnt = ctypes.c_int()
    st = lib.GCGE_SpMMTuneCandidates(ctypes.c_int(k), buf, ctypes.c_int(16), ctypes.byref(cnt))
    if st != GCGE_OK:
        raise GCGEError(st, "GCGE_SpMMTuneCandidates")
    return list(buf[:min(cnt.value, 16)])


def spmm_tune(A, k: int, fp32: bool):
    """Time every candidate column split of an SpMM of k columns of A; the
    choice is kept for later SpMMs of A's shape.  Returns (chosen width,
    {width: ms})."""
    lib = load()
    ops = CudaOps()
    try:
        h = ops.mat(A)
        chunk, cnt = ctypes.c_int(), ctypes.c_int()
        ms = (ctypes.c_double * 16)()
        st = lib.GCGE_SpMMTune(h, ctypes.c_int(k), ctypes.c_int(1 if fp32 else 0),
                               ctypes.byref(chunk), ms, ctypes.c_int(16), ctypes.byref(cnt))
        if st != GCGE_OK:
            raise GCGEError(st, "GCGE_SpMMTune")
        widths = spmm_tune_candidates(k)
        return chunk.value, dict(zip(widths, ms[:min(cnt.value, 16)]))
    finally:
        ops.close()


def dense_eig(M: np.ndarray):
    """Eigen-decomposition of a symmetric matrix with the solver's dense
    eigensolver (FP32 Jacobi + FP64 refinement on the GPU)."""
    lib = load()
    M = np.asfortranarray(M, dtype=np.float64)
    s = M.shape[0]
    ev = np.zeros(s)
    Z = np.zeros((s, s), order="F")
    st = lib.GCGE_DenseEig(ctypes.c_int(s), _p(M), ctypes.c_int(s), _p(ev), _p(Z), ctypes.c_int(s))
    if st != GCGE_OK:
        raise GCGEError(st, "GCGE_DenseEig")
    return ev, Z


def block_pcg(A, B, sigma, b, x0, max_iter=30, rate=1e-2, tol=1e-14, fp32=False):
    """Block CG on (A + sigma B) x = b through GCGE_BlockPCG; returns (x, iters)."""
    ops = CudaOps()
    try:
        hA = ops.mat(A)
        hB = ops.mat(B) if B is not None else None
        k = b.shape[1]
        hb = ops.multivec(hA, k, b)
        hx = ops.multivec(hA, k, x0)
        it = ctypes.c_int()
        st = ops.lib.GCGE_BlockPCG(hA, hB, ctypes.c_double(sigma), hb, hx, ctypes.c_int(k),
                                   ctypes.c_int(max_iter), ctypes.c_double(rate),
                                   ctypes.c_double(tol), ctypes.c_int(1 if fp32 else 0),
                                   ctypes.byref(it))
        if st != GCGE_OK:
            raise GCGEError(st, "GCGE_BlockPCG")
        return ops.download(hx, 0, k), it.value
    finally:
        ops.close()


def bench_dense_product(kind, n, m, w, emulated=True, reps=5):
    """Average ms of one long-dimension product on generated device data:
    kind "gram" (Q^T P, Q n x m, P n x w) or "lincomb" (X C, X n x m, C m x w)."""
    lib = load()
    ms = ctypes.c_double()
    st = lib.GCGE_BenchDenseProduct(ctypes.c_int(0 if kind == "gram" else 1), ctypes.c_int(n),
                                    ctypes.c_int(m), ctypes.c_int(w),
                                    ctypes.c_int(1 if emulated else 0), ctypes.c_int(reps),
                                    ctypes.byref(ms))
    if st != GCGE_OK:
        raise GCGEError(st, "GCGE_BenchDenseProduct")
    return ms.value


def dense_gram(Q, P, emulated=False):
    """Q^T P through GCGE_DenseGram (FP64 kernel, or the tensor-core digit
    kernel when emulated)."""
    lib = load()
    Q = np.asfortranarray(Q, dtype=np.float64)
    P = np.asfortranarray(P, dtype=np.float64)
    n, m = Q.shape
    w = P.shape[1]
    C = np.zeros((m, w), dtype=np.float64, order="F")
    st = lib.GCGE_DenseGram(ctypes.c_int(n), ctypes.c_int(m), ctypes.c_int(w),
                            Q.ctypes.data_as(ctypes.c_void_p), ctypes.c_int(max(n, 1)),
                            P.ctypes.data_as(ctypes.c_void_p), ctypes.c_int(max(n, 1)),
                            C.ctypes.data_as(ctypes.c_void_p), ctypes.c_int(1 if emulated else 0))
    if st != GCGE_OK:
        raise GCGEError(st, "GCGE_DenseGram")
    return C


def dense_lincomb(X, C, Y, beta=None, alpha=1.0, emulated=False):
    """alpha X C + Y diag(beta) (beta None: overwrite) through GCGE_DenseLinComb."""
    lib = load()
    X = np.asfortranarray(X, dtype=np.float64)
    C = np.asfortranarray(C, dtype=np.float64)
    Y = np.array(Y, dtype=np.float64, order="F", copy=True)
    n, k = X.shape
    m = C.shape[1]
    b = None if beta is None else np.ascontiguousarray(beta, dtype=np.float64)
    st = lib.GCGE_DenseLinComb(ctypes.c_int(n), ctypes.c_int(k), ctypes.c_int(m),
                               X.ctypes.data_as(ctypes.c_void_p), ctypes.c_int(n),
                               C.ctypes.data_as(ctypes.c_void_p), ctypes.c_int(max(k, 1)),
                               Y.ctypes.data_as(ctypes.c_void_p), ctypes.c_int(n),
                               None if b is None else b.ctypes.data_as(ctypes.c_void_p),
                               ctypes.c_double(alpha), ctypes.c_int(1 if emulated else 0))
    if st != GCGE_OK:
        raise GCGEError(st, "GCGE_DenseLinComb")
    return Y


def b_orth(B, X, start, n=None, zero_tol=2 * np.finfo(float).eps, max_reorth=2, A_for_size=None):
    """B-orthonormalise columns [start, end) of X against [0, start) via
    GCGE_BOrth; returns the orthonormalised block (columns [0, new_end))."""
    ops = CudaOps()
    try:
        M = B if B is not None else A_for_size
        hB = ops.mat(B) if B is not None else None
        hM = hB if hB is not None else ops.mat(M)
        k = X.shape[1]
        hx = ops.multivec(hM, k, X)
        end = ctypes.c_int(k)
        st = ops.lib.GCGE_BOrth(hB, hx, ctypes.c_int(start), ctypes.byref(end),
                                ctypes.c_double(zero_tol), ctypes.c_int(max_reorth))
        if st != GCGE_OK:
            raise GCGEError(st, "GCGE_BOrth")
        return ops.download(hx, 0, end.value)
    finally:
        ops.close()


class DeviceTimer:
    """CUDA events on the library stream around a region (GCGE_TimerStart/Stop)."""

    def __enter__(self):
        st = load().GCGE_TimerStart()
        if st != GCGE_OK:
            raise GCGEError(st, "GCGE_TimerStart")
        return self

    def __exit__(self, *exc):
        self.ms = load().GCGE_TimerStop()
        return False
