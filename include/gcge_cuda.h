/*
 * gcge_cuda.h - CUDA (sm_103a) backend and solver entry points of the GB300
 * GCGE library (libgcge_cuda.so).  Plain C ABI: pointers, sizes, status codes.
 *
 * Drop-in map (reference interface each entry replaces):
 *   OPS_CUDA_Set                 <- OPS_CCS_Set            app/app_ccs.c:213-249
 *   CUDA_MatCreateFromCCS        <- filling a CCSMAT        app/app_ccs.h:20-24
 *   CUDA_MultiVecSetFromHost /
 *   CUDA_MultiVecGetToHost       <- direct LAPACKVEC.data access (app/app_lapack.h:17-20);
 *                                   device multivectors are opaque
 *   GCGE_Solve                   <- the EigenSolverSetup_GCG + GCGE_Setparameters +
 *                                   ops->EigenSolver sequence of gcge.c:490-531
 *                                   (the reference has no single GCGE_Solve symbol)
 * OPS slots filled by OPS_CUDA_Set (semantics of app_ccs + app_lapack):
 *   MatDotMultiVec, MatTransDotMultiVec   app/app_ccs.c:50-150 (mat NULL -> copy)
 *   MultiVecAxpby                         app/app_lapack.c:334-395
 *   MultiVecLinearComb                    app/app_lapack.c:463-534
 *   MultiVecInnerProd / LocalInnerProd    app/app_lapack.c:299-321 + DenseMatQtAP :64-183
 *   MultiVecQtAP                          src/ops_multi_vec.c:351-411 (fused on device)
 *   MultiVecCreateByMat/ByVec/ByMultiVec, MultiVecDestroy, MultiVecView,
 *   MultiVecSetRandomValue, Get/RestoreVecFromMultiVec, Vec* single-vector ops
 *                                         app/app_lapack.c:230-650
 */
#ifndef GCGE_CUDA_H
#define GCGE_CUDA_H

#include <stddef.h>
#include "gcge_ops.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes returned by every int-valued entry point and recorded as the
 * sticky status of the void OPS slots. */
enum {
    GCGE_OK = 0,
    GCGE_ERR_CUDA = 1,        /* a CUDA runtime call failed */
    GCGE_ERR_ARG = 2,         /* invalid argument (size, range, NULL) */
    GCGE_ERR_ALLOC = 3,       /* device or host allocation failed */
    GCGE_ERR_HANDLE = 4,      /* handle is not a CUDA matrix / multivector */
    GCGE_ERR_NUMERIC = 5,     /* NaN/Inf detected in residuals or projections */
    GCGE_ERR_NOT_CONVERGED = 6, /* numIterMax reached before nev pairs converged */
    GCGE_ERR_NO_DEVICE = 7,   /* no CUDA device visible */
    GCGE_ERR_TOO_LARGE = 8    /* projected problem exceeds the dense-solver capacity */
};

/* Sticky error of the OPS slots and setup calls on this thread (0 = none);
 * reading it clears it. */
int ops_cuda_last_error(void);
const char *ops_cuda_error_string(int status);
/* Text of the most recent error recorded by any entry point (where it was
 * raised and the CUDA message, if any); not cleared by ops_cuda_last_error. */
const char *ops_cuda_last_error_detail(void);

/* ---- backend --------------------------------------------------------- */
void OPS_CUDA_Set(struct OPS_ *ops);

/* Device matrix from host CCS arrays of an n x n matrix (int32 indices, FP64
 * values; j_col[n+1], i_row[nnz], data[nnz]).  The data are copied to HBM.
 * Like app_ccs, MatTransDotMultiVec assumes the matrix is symmetric
 * (app/app_ccs.c:140-150). */
int CUDA_MatCreateFromCCS(void **mat, int nrows, int ncols, const int *j_col, const int *i_row,
                          const double *data);
void CUDA_MatDestroy(void **mat);
int CUDA_MatNnz(void *mat, long long *nnz);

/* Y = alpha X + beta Y for device matrices: the OPS MatAxpby slot
 * (src/ops.h:52, used by src/ops_eig_sol_gcg.c:600-631 and :730-744 for the
 * in-place shift A + sigma B).  Y takes the union pattern of X and Y.
 * OPS_CUDA_Set leaves ops->MatAxpby NULL, as app_ccs does; install this
 * function there to provide the slot.  Failures go to ops_cuda_last_error(). */
void CUDA_MatAxpby(double alpha, void *matX, double beta, void *matY, struct OPS_ *ops);

/* Transfer operator P between adjacent multigrid levels (nrows fine rows x
 * ncols coarse columns) from host CCS arrays (j_col[ncols+1], i_row[nnz],
 * data[nnz]), copied to HBM; for P_array of MultiLinearSolverSetup_BlockAMG
 * and MultiVecFromItoJ.  No counterpart in app_ccs (its matrices are square
 * operators; the reference's hierarchies come from ops->MultiGridCreate). */
int CUDA_TransferCreateFromCCS(void **P, int nrows, int ncols, const int *j_col,
                               const int *i_row, const double *data);
void CUDA_TransferDestroy(void **P);
/* The OPS MultiVecFromItoJ slot (src/ops.h:142-144; NULL in every backend
 * the reference ships, src/ops.c:78): columns [startIJ[0], endIJ[0]) of the
 * level-i block to [startIJ[1], endIJ[1]) of the level-j block, one level at
 * a time: restriction x_{l+1} = P_l^T x_l going down, prolongation x_l =
 * P_l x_{l+1} going up, P_array[l] from CUDA_TransferCreateFromCCS; between
 * non-adjacent levels through columns [0, k) of multi_vec_ws[l].
 * OPS_CUDA_Set installs it.  Failures go to ops_cuda_last_error(). */
void CUDA_MultiVecFromItoJ(void **P_array, int level_i, int level_j, void **multi_vec_i,
                           void **multi_vec_j, int *startIJ, int *endIJ, void ***multi_vec_ws,
                           struct OPS_ *ops);

/* Copy columns [start, end) between a device multivector and a host
 * column-major array with leading dimension ldh >= nrows. */
int CUDA_MultiVecSetFromHost(void **mv, int start, int end, const double *host, int ldh);
int CUDA_MultiVecGetToHost(void **mv, int start, int end, double *host, int ldh);
int CUDA_MultiVecSize(void **mv, int *nrows, int *ncols);

/* ---- GCG solve -------------------------------------------------------- */
enum { GCGE_PREC_FP64 = 0, GCGE_PREC_MIXED = 1 };

/* Precision of the GPU GCG installed on this ops (default GCGE_PREC_FP64).
 * MIXED runs the block-PCG inner solve and its SpMM with FP32 values, int32
 * indices and FP32 accumulation; residuals, B-orthogonalisation, Rayleigh-Ritz
 * and the dense eigensolve stay FP64. */
int GCGE_SetPrecision(struct OPS_ *ops, int precision);

typedef struct gcge_solve_info {
    int nconv;          /* locked (converged) pairs, may exceed nev */
    int niter;          /* outer GCG iterations */
    int status;         /* GCGE_OK / GCGE_ERR_NOT_CONVERGED / ... */
    int pcg_iters;      /* total inner block-PCG iterations */
    int spmm_calls;     /* SpMM launches */
    int kernel_launches;/* all kernels launched by the solve */
    double seconds;     /* wall time of the solve on the host clock */
    double phase_ms[10];/* checkconv, compP, compRR, rr_matW, eig, compRV, compW, linsol,
                           compX, initX (CUDA events on the solver stream) */
    int pcg_spmm_launches;   /* SpMM phases inside the block-PCG iterations (one per iteration) */
    double pcg_spmm_ms;      /* their summed device time (device clock at the grid barriers
                                that open and close each SpMM phase) */
    double pcg_spmm_bytes;   /* their summed algorithmic bytes: nnz (v + 4) + 4 (n + 1)
                                + 2 n k_active v, v = value size (8 FP64, 4 mixed),
                                k_active = columns in 16-byte groups with an active column */
    int pcg_kernel_launches; /* block-PCG solves (one persistent kernel launch each) */
    double pcg_kernel_ms;    /* their summed device time (CUDA events around each launch) */
    double pcg_kernel_bytes; /* their summed algorithmic bytes: per iteration the matrix once
                                + 12 n k_active v (p update, SpMM, x/r update), plus the setup */
    int precision_escalation_iter; /* mixed solve: outer iteration from which the solve
                                      ran in FP64 because its residuals stalled just
                                      above the tolerance (0: never) */
} gcge_solve_info;

/* One-call solve of A x = lambda B x for the nev smallest pairs from host
 * CCS arrays (B may be NULL = identity).  X0 (n x nev_given, column-major,
 * may be NULL when nev_given = 0) seeds the first columns of the basis.
 * tol = {abs, rel}; convergence is ||A x - lambda B x||_2 <= tol[0] and
 * <= |lambda| tol[1] with x B-normalised (src/ops_eig_sol_gcg.c:239-240).
 * gap_min and auto_shift are the GCGE_Setparameters arguments.
 * eval[nev_max], evec[n x nev_max] (column-major) receive the solver's
 * eval/evec arrays; info may be NULL. */
int GCGE_Solve(int n, const int *a_colptr, const int *a_rowind, const double *a_val,
               const int *b_colptr, const int *b_rowind, const double *b_val, int nev,
               int block_size, int nev_init, int nev_max, int max_iter, const double tol[2],
               double gap_min, int auto_shift, int precision, const double *X0, int nev_given,
               double *eval, double *evec, gcge_solve_info *info);

/* Page-locked host memory for GCGE_Solve's inputs and outputs (the CCS
 * arrays, X0, eval, evec): copies from and to it run as DMA at link speed,
 * while pageable buffers are staged by the driver.  NULL on failure. */
void *GCGE_HostAlloc(size_t bytes);
void GCGE_HostFree(void *p);

/* ---- many solves on one GPU (batched problems, serving) ----------------
 * A request is one GCGE_Solve call (same inputs and outputs) plus its state.
 * A server runs requests on `workers` host threads, each with its own CUDA
 * stream, so solves overlap on the device; a request starts when its estimated
 * device footprint fits the memory budget (0: 80% of the free memory at
 * creation), or when nothing else runs.  Results are the same alone and in a
 * mix up to the rounding of the block-PCG reductions, whose grid is shared
 * between the workers.  No counterpart in the reference (one solve per
 * process, file-static solver state). */
typedef struct gcge_request {
    int n;
    const int *a_colptr, *a_rowind;
    const double *a_val;
    const int *b_colptr, *b_rowind; /* B may be NULL = identity */
    const double *b_val;
    int nev, block_size, nev_init, nev_max, max_iter;
    double tol[2];
    double gap_min;
    int auto_shift, precision;
    const double *X0;
    int nev_given;
    double *eval;  /* nev_max */
    double *evec;  /* n x nev_max or NULL */
    gcge_solve_info info;
    int status;    /* set when done */
    int done;      /* 1 when the outputs are final */
    double t_submit, t_start, t_end; /* host clock, seconds */
} gcge_request;
typedef struct gcge_server gcge_server;
gcge_server *GCGE_ServerCreate(int workers, size_t device_budget_bytes);
int GCGE_ServerSubmit(gcge_server *s, gcge_request *r);  /* returns at once */
int GCGE_ServerWait(gcge_server *s, gcge_request *r);    /* waits for r; returns its status */
void GCGE_ServerDestroy(gcge_server **s);                 /* runs the queue out, joins */
/* Submit all, wait for all; returns the first error other than NOT_CONVERGED. */
int GCGE_SolveBatch(gcge_request *reqs, int count, int workers, size_t device_budget_bytes);

/* Statistics of the last ops->EigenSolver call on this ops. */
int GCGE_GetSolveInfo(struct OPS_ *ops, gcge_solve_info *info);

/* ---- device-resident benchmarking helpers ------------------------------
 * A prepared problem keeps A, B, the initial block and all solver state in
 * HBM so repeated solves time only the device work. */
typedef struct gcge_prepared gcge_prepared;
int GCGE_Prepare(gcge_prepared **prep, int n, const int *a_colptr, const int *a_rowind,
                 const double *a_val, const int *b_colptr, const int *b_rowind,
                 const double *b_val, int nev, int block_size, int nev_init, int nev_max,
                 int max_iter, const double tol[2], double gap_min, int auto_shift,
                 int precision, const double *X0, int nev_given);
/* Solve with device-resident inputs; eval (host, nev_max) is copied back,
 * eigenvectors stay on the device unless evec is non-NULL. */
int GCGE_PreparedSolve(gcge_prepared *prep, double *eval, double *evec, gcge_solve_info *info);
void GCGE_PreparedDestroy(gcge_prepared **prep);

/* ---- kernel-level entry points used by the measurement harness ---------
 * SpMM of k columns, Y = M X, on device buffers owned by the library.
 * Timed with CUDA events on the library stream; returns average ms/launch. */
int GCGE_BenchSpMM(void *mat, int k, int fp32, int reps, double *ms_per_launch,
                   double *bytes_per_launch);

/* ---- SpMM column-split autotuner ----------------------------------------
 * An SpMM of k columns (MatDotMultiVec and the solver's own products; the
 * reference's app_ccs multiplies one column at a time, app/app_ccs.c:120-131)
 * runs as p launches of ceil(k / p) columns: each launch streams the matrix
 * once and keeps its columns' sums in registers, so few wide launches read
 * the matrix least and narrow ones keep more warps resident.  With tuning
 * on, the first SpMM of a matrix shape (rows, stored entries, value type) and
 * column class (k rounded up to a multiple of 8) on a device times every
 * candidate split with CUDA events on the calling stream and keeps the
 * fastest for the process.  Results are bitwise the same for every split.
 * Off until GCGE_SetSpMMTuning(1) or the environment variable
 * GCGE_SPMM_TUNE=1 at the first SpMM.  No counterpart in the reference. */
/* on = 1: tune; 0: fixed 40-column launches; -1: off and forget the choices. */
int GCGE_SetSpMMTuning(int on);
/* The candidate launch widths for k columns, fewest launches first:
 * chunks[0 .. min(*count, cap)).  Host only (needs no device). */
int GCGE_SpMMTuneCandidates(int k, int *chunks, int cap, int *count);
/* Time every candidate split of an SpMM of k columns of a CUDA matrix (FP32
 * values and columns when fp32) on seeded device columns owned by the call,
 * keep the choice for later SpMMs of that shape, and return the chosen
 * launch width and each candidate's average ms (ms[0 .. min(*count, cap))). */
int GCGE_SpMMTune(void *mat, int k, int fp32, int *chunk, double *ms, int cap, int *count);

/* One long-dimension dense product on device data the call generates
 * (seeded uniform values), timed with CUDA events on the library stream
 * after one untimed call: kind 0 = Gram C (m x w) = Q^T P with Q n x m and
 * P n x w; kind 1 = linear combination Y (n x w) = X C with X n x m and
 * C m x w; emulated selects the tensor-core digit kernels of the mixed solve
 * instead of the FP64 ones.  Returns the average ms per call. */
int GCGE_BenchDenseProduct(int kind, int n, int m, int w, int emulated, int reps,
                           double *ms_per_call);

/* CUDA-event timer on the library stream: GCGE_TimerStart records the start
 * event; GCGE_TimerStop records the stop event, waits for it and returns the
 * elapsed milliseconds (negative on error). */
int GCGE_TimerStart(void);
double GCGE_TimerStop(void);

/* ---- component entry points (each step of the solver on its own) -------
 * Dense symmetric eigensolve of the Rayleigh-Ritz step (replaces dsyevx,
 * src/ops_eig_sol_gcg.c:1145-1150): host M (s x s, ldm) -> ascending eval[s]
 * and orthonormal eigenvectors Z (s x s, ldz). */
int GCGE_DenseEig(int s, const double *M, int ldm, double *eval, double *Z, int ldz);
/* Block CG on (A + sigma B) x = b for columns [0, k) of device multivectors
 * b and x (x holds the initial guess), with the stopping rule of BlockPCG
 * (src/ops_lin_sol.c:383-394, absolute tolerance); fp32 selects the mixed
 * precision path. */
int GCGE_BlockPCG(void *A, void *B, double sigma, void **b, void **x, int k, int max_iter,
                  double rate, double tol, int fp32, int *iters);
/* Failure-detection test of the persistent block-PCG kernel's grid barrier:
 * GCGE_BlockPCG (FP64, sigma 0, 30 steps) with every barrier wait bounded by
 * timeout_ms and the grid's last block leaving before its first barrier, so
 * the other blocks' waits run out.  Expected result: GCGE_ERR_CUDA, with the
 * device context intact (the next solve succeeds).  Needs an operator large
 * enough for the grid form (FP64: more slices than a 16-CTA cluster has
 * warps, n > 4096 or so).  No counterpart in the reference. */
int GCGE_TestBlockPCGBarrierTimeout(void *A, void **b, void **x, int k, double timeout_ms);
/* B-orthonormalise columns [start, *end) of x against [0, start) (B NULL =
 * identity), as MultiVecOrth does (src/ops_orth.c:203-394); *end shrinks by
 * the number of dependent columns dropped. */
int GCGE_BOrth(void *B, void **x, int start, int *end, double zero_tol, int max_reorth);

/* Long-dimension dense products from host arrays, through the FP64 kernels
 * (emulated = 0) or the FP64-accurate tensor-core digit kernels of the mixed
 * solve (emulated = 1).  GCGE_DenseGram: C (m x w, leading dimension m) =
 * Q^T P for Q n x m and P n x w, as DenseMatQtAP with matA = NULL
 * (app/app_lapack.c:64-183).  GCGE_DenseLinComb: Y (n x m) = alpha X C +
 * Y diag(beta) for X n x k and C k x m (beta NULL: Y overwritten), as
 * MultiVecLinearComb (app/app_lapack.c:463-534). */
int GCGE_DenseGram(int n, int m, int w, const double *Q, int ldq, const double *P, int ldp,
                   double *C, int emulated);
int GCGE_DenseLinComb(int n, int k, int m, const double *X, int ldx, const double *C, int ldc,
                      double *Y, int ldy, const double *beta, double alpha, int emulated);

/* ---- allocation-free Gram product ---------------------------------------
 * No counterpart in the reference: an addition for callers that may not
 * allocate device memory (their memory belongs to another allocator or a
 * pre-sized pool, or they run latency-critical loops where an allocation's
 * device synchronisation is not acceptable).
 * C (m x w, ldc) = Q^T P for device arrays Q (n x m, ldq) and P (n x w, ldp),
 * column-major, launched on `stream` (a cudaStream_t; NULL = default stream).
 * Calls no cudaMalloc/cudaFree: the split-K partial sums live in a 4 MiB
 * device array fixed in the library, so m * w <= 524288 (larger requests
 * return GCGE_ERR_TOO_LARGE).  The array's device address is looked up by
 * the first call on each device (make that call before any stream capture);
 * all calls on a device share the array, so calls that overlap on the GPU
 * race - order them on one stream. */
#define GCGE_NOALLOC_SCRATCH_BYTES (4u << 20)
int GCGE_GramNoAlloc(int n, int m, int w, const double *Q, int ldq, const double *P, int ldp,
                     double *C, int ldc, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* GCGE_CUDA_H */
