// GPU GCG solver context (gcg.cu) shared with the OPS backend (app_cuda.cu).
#pragma once
#include "common.cuh"
#include "eig.cuh"
#include "pcg.cuh"

namespace gcge {

struct SolverCtx {
    GCGSolver pub;  // first member: ops->eigen_solver_workspace points here
    bool pub_init = false;  // pub holds the EigenSolverSetup_GCG defaults
    int precision = GCGE_PREC_FP64;
    // mixed solve that fell back to FP64 for its remaining iterations (reset
    // at the start of every solve)
    bool escalated = false;
    int refine_steps = 8;  // upper bound; the refinement stops on convergence
    gcge_solve_info info{};
    int last_status = GCGE_OK;

    // union-pattern operator data, rebuilt when (A, B) change
    unsigned long long keyA = 0, keyB = 0;
    bool has_union = false;
    SellPattern upat;
    DevBuf<double> ua, ub, us64;
    DevBuf<float> us32;

    // work buffers
    int n = 0, ld = 0, cap_cols = 0, cap_s = 0, cap_bs = 0;
    DevBuf<double> T1, T2, bbuf, r64;
    // slice-blocked block-PCG vectors (n x 40 at most)
    DevBuf<double> xr64, br64, rr64, pr64, wr64;
    DevBuf<float> xr32, br32, rr32, pr32, wr32;
    DevBuf<double> M0, M1, evec, work, coefP, ptap, dC, dtmp, gscr, part, dvec, dmax, one;
    // A x and B x of the Ritz vectors CheckConvergence tested (n x numCheck),
    // reused by ComputeW for its right-hand side and initial residual
    DevBuf<double> chkA, chkB;
    // right-operand digit planes of the mixed solve's linear combinations
    DevBuf<unsigned char> ozb;
    DevBuf<int> dmask, didx;
    PinnedBuf<double> hbuf, hmax;
    // host staging of small uploads that no later host write touches before
    // the stream has passed them (ComputeP's column lists, the Ritz values of
    // the projected matrix), so their copies need no wait
    PinnedBuf<double> hup;
    EigWork eig;
    PcgWork pcg;

    void reserve(int n, int nev_max, int nev_init, int bs, int spmm_nblocks);
};

// Registry of solver contexts, one per OPS object.
SolverCtx *ctx_for(OPS *ops, bool create);
void ctx_release(OPS *ops);

// Per-ops state of MultiLinearSolverSetup_BlockPCG (linsol.cu), freed by
// OPS_Destroy.
void linsol_release(OPS *ops);
// Per-ops state of MultiLinearSolverSetup_BlockAMG (amg.cu), freed by
// OPS_Destroy.
void amg_release(OPS *ops);

// The GPU GCG installed as ops->EigenSolver.
void gcg_eigensolver(void *A, void *B, double *eval, void **evec, int nevGiven, int *nevConv,
                     OPS *ops);

unsigned long long mat_serial(const SparseMat *m);

// B-orthonormalisation of columns [start, end) of x against [0, start)
// (blocked CGS with re-orthogonalisation + Cholesky-QR2 with dropping).
int borth(SolverCtx &c, SparseMat *B, double *x, int ldx, int nrows, int start, int end,
          bool useB, double zero_tol, int max_reorth, int *spmm_calls);
// Binary Gram-Schmidt of src/ops_orth.c:416-623 (CGS against the prefix, then
// recursive halving with OrthSelf / OrthSelfEVP leaves); same arguments as
// borth plus the leaf size (<= 0: the reference's default choice).
int bgs_orth(SolverCtx &c, SparseMat *B, double *x, int ldx, int nrows, int start, int end,
             bool useB, double zero_tol, int max_reorth, int block_size, int *spmm_calls);
// Union pattern of A, B (B NULL = identity) and the diagonal, with A's and B's
// values on it; cached on the context by matrix identity.
void prepare_union(SolverCtx &c, SparseMat *A, SparseMat *B, cudaStream_t st);

}  // namespace gcge
