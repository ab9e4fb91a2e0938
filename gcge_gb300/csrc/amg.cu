// Block algebraic multigrid solver and the level transfers of the CUDA
// backend: MultiLinearSolverSetup_BlockAMG installs the reference's V-cycle
// (src/ops_lin_sol.c:466-715) as ops->MultiLinearSolver over a hierarchy the
// caller builds (level matrices A_l as CUDA matrices, transfers P_l from
// CUDA_TransferCreateFromCCS); CUDA_MultiVecFromItoJ is the OPS slot that
// moves blocks between levels, which the reference declares
// (src/ops.h:142-144) and leaves NULL in every backend it ships.
//
// The V-cycle runs on the host through the OPS slots, as in the reference:
// at level l, BlockPCG smoothing with that level's iteration cap, rate and
// tolerance (installed by MultiLinearSolverSetup_BlockPCG, so the smoothing
// is the persistent block-PCG kernel of pcg.cu on the level's matrix), the
// residual b - A_l x, its restriction P_l^T r, the coarse solve from zero,
// the prolongation P_l e added to x, and the post-smoothing; the coarsest
// level is one BlockPCG solve.  Cycles repeat until the residual field of the
// last level-0 smoothing is below tol[0] or max_iter[0] cycles ran.
#include <cstring>
#include <mutex>
#include <unordered_map>
#include <vector>

#include "gcg.cuh"

namespace gcge {

constexpr uint32_t kTransferMagic = 0x54524755u;  // transfer operator

// P (fine rows x coarse columns) in CSR, and P^T in CSR (= P's CCS).
struct Transfer {
    uint32_t magic = kTransferMagic;
    int nrows = 0, ncols = 0;
    long long nnz = 0;
    DevBuf<int> p_ptr, p_ind, t_ptr, t_ind;
    DevBuf<double> p_val, t_val;
};

Transfer *as_transfer(void *h) {
    Transfer *t = static_cast<Transfer *>(h);
    return (t != nullptr && t->magic == kTransferMagic) ? t : nullptr;
}

namespace {

// Y(:, c) = M X(:, c) for a CSR matrix M of `rows` rows and columns c < k:
// one thread per row and column, the row's entries summed in stored order.
// Column indices were checked against X's rows when M was created.
__global__ void k_csr_mm(int rows, const int *__restrict__ ptr, const int *__restrict__ ind,
                         const double *__restrict__ val, const double *__restrict__ X, int ldx,
                         double *__restrict__ Y, int ldy, int k) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int c = blockIdx.y;
    if (i >= rows || c >= k) return;
    const double *x = X + (size_t)c * ldx;
    double s = 0.0;
    for (int e = ptr[i]; e < ptr[i + 1]; ++e) s = fma(val[e], x[ind[e]], s);
    Y[i + (size_t)c * ldy] = s;
}

void csr_mm(int rows, const int *ptr, const int *ind, const double *val, const double *X, int ldx,
            double *Y, int ldy, int k, cudaStream_t st) {
    if (rows <= 0 || k <= 0) return;
    GCGE_REQUIRE(k <= 65535, GCGE_ERR_ARG, "MultiVecFromItoJ: more than 65535 columns");
    k_csr_mm<<<dim3((rows + 255) / 256, k), 256, 0, st>>>(rows, ptr, ind, val, X, ldx, Y, ldy, k);
    GCGE_CHECK_LAUNCH();
    count_launch();
}

MultiVec *mv_checked(void **h, const char *what) {
    MultiVec *m = as_mv(h);
    GCGE_REQUIRE(m != nullptr, GCGE_ERR_HANDLE, std::string(what) + ": not a CUDA multivector");
    return m;
}

// Throws the status a slot left behind (the slots report through set_error).
void check_slot(const char *what) {
    const int e = take_error();
    if (e != GCGE_OK) throw CudaError{e, std::string("BlockAMG: ") + what};
}

// Per-ops state: the reference keeps one static BlockAMGSolver per process
// (src/ops_lin_sol.c:690-693); here every ops has its own.  The smoothing
// solves of each level run on an OPS object of that level: the block-PCG
// setup keeps its operator (the level matrix on its union pattern) per OPS,
// so one per level builds each level's operator once instead of at every
// switch between levels.
struct AmgRecord {
    BlockAMGSolver pub;  // ops->multi_linear_solver_workspace points here
    std::vector<OPS *> level_ops;
    ~AmgRecord() {
        for (OPS *&o : level_ops) OPS_Destroy(&o);
    }
    OPS *level(int l) {
        while ((int)level_ops.size() <= l) {
            OPS *o = nullptr;
            OPS_Create(&o);
            GCGE_REQUIRE(o != nullptr, GCGE_ERR_ALLOC, "BlockAMG: level solver");
            OPS_CUDA_Set(o);
            OPS_Setup(o);
            level_ops.push_back(o);
        }
        return level_ops[l];
    }
};

std::mutex g_amg_mu;
std::unordered_map<OPS *, AmgRecord *> g_amg;

AmgRecord *amg_record(OPS *ops, bool create) {
    std::lock_guard<std::mutex> lk(g_amg_mu);
    auto it = g_amg.find(ops);
    if (it != g_amg.end()) return it->second;
    if (!create) return nullptr;
    AmgRecord *r = new AmgRecord();
    g_amg[ops] = r;
    return r;
}

// One V-cycle from `level` down (src/ops_lin_sol.c:466-642): columns
// [start_bx[0], end_bx[0]) of b, [start_bx[1], end_bx[1]) of x.  The
// residual, the transfers and the correction go through the caller's slots;
// the smoothing solves (BlockPCG with the level's parameters) through the
// level's own OPS object.
void amg_cycle(AmgRecord &r, int level, void **mv_b, void **mv_x, int *start_bx, int *end_bx,
               OPS *ops) {
    BlockAMGSolver &g = r.pub;
    OPS *lops = r.level(level);
    const int coarsest = g.num_levels - 1;
    const int bs = end_bx[1] - start_bx[1];
    void *A = g.A_array[level];
    void **ws[3] = {g.mv_array_ws[2][level], g.mv_array_ws[3][level], g.mv_array_ws[4][level]};
    // pre-smoothing (the whole solve at the coarsest level), :485-502
    MultiLinearSolverSetup_BlockPCG(g.max_iter[2 * level + 1], g.rate[level], g.tol[level],
                                    g.tol_type, ws, g.dbl_ws, g.int_ws, nullptr, nullptr, lops);
    check_slot("MultiLinearSolverSetup_BlockPCG");
    lops->MultiLinearSolver(A, mv_b, mv_x, start_bx, end_bx, lops);
    check_slot("smoothing");
    if (level < coarsest) {
        int start[2], end[2];
        // r = b - A x into columns [0, bs) of ws[0], :516-530
        void **mv_r = g.mv_array_ws[2][level];
        start[0] = start_bx[1], end[0] = end_bx[1], start[1] = 0, end[1] = bs;
        ops->MatDotMultiVec(A, mv_x, mv_r, start, end, ops);
        check_slot("MatDotMultiVec");
        start[0] = start_bx[0], end[0] = end_bx[0], start[1] = 0, end[1] = bs;
        ops->MultiVecAxpby(1.0, mv_b, -1.0, mv_r, start, end, ops);
        check_slot("MultiVecAxpby");
        // restriction and the coarse problem from zero, :544-570
        const int coarse = level + 1;
        void **coarse_b = g.mv_array_ws[0][coarse], **coarse_x = g.mv_array_ws[1][coarse];
        start[0] = start[1] = 0, end[0] = end[1] = bs;
        ops->MultiVecFromItoJ(g.P_array, level, coarse, mv_r, coarse_b, start, end,
                              g.mv_array_ws[4], ops);
        check_slot("MultiVecFromItoJ (restriction)");
        ops->MultiVecAxpby(0.0, nullptr, 0.0, coarse_x, start, end, ops);
        check_slot("MultiVecAxpby");
        amg_cycle(r, coarse, coarse_b, coarse_x, start, end, ops);
        // prolongation into ws[0] and x += P e, :577-600
        ops->MultiVecFromItoJ(g.P_array, coarse, level, coarse_x, mv_r, start, end,
                              g.mv_array_ws[4], ops);
        check_slot("MultiVecFromItoJ (prolongation)");
        start[0] = 0, end[0] = bs, start[1] = start_bx[1], end[1] = end_bx[1];
        ops->MultiVecAxpby(1.0, mv_r, 1.0, mv_x, start, end, ops);
        check_slot("MultiVecAxpby");
        // post-smoothing, :611-627
        MultiLinearSolverSetup_BlockPCG(g.max_iter[2 * level + 2], g.rate[level], g.tol[level],
                                        g.tol_type, ws, g.dbl_ws, g.int_ws, nullptr, nullptr,
                                        lops);
        check_slot("MultiLinearSolverSetup_BlockPCG");
        lops->MultiLinearSolver(A, mv_b, mv_x, start_bx, end_bx, lops);
        check_slot("smoothing");
    }
    // the residual field of the last smoothing solve, :637; the caller's ops
    // keeps the AMG solver installed throughout (the reference re-installs
    // it after each level, :638-641)
    g.residual = static_cast<BlockPCGSolver *>(lops->multi_linear_solver_workspace)->residual;
}

// Sizes of the hierarchy and of the workspaces a cycle of bs columns uses,
// checked before the first launch.
void check_hierarchy(const BlockAMGSolver &g, int bs) {
    GCGE_REQUIRE(g.num_levels >= 1 && g.A_array != nullptr && (g.num_levels == 1 || g.P_array),
                 GCGE_ERR_ARG, "BlockAMG: hierarchy arrays");
    for (int i = 0; i < 5; ++i)
        GCGE_REQUIRE(g.mv_array_ws[i] != nullptr, GCGE_ERR_ARG, "BlockAMG: mv_array_ws");
    for (int l = 0; l < g.num_levels; ++l) {
        SparseMat *A = as_mat(g.A_array[l]);
        GCGE_REQUIRE(A != nullptr, GCGE_ERR_HANDLE, "BlockAMG: A_array holds a non-CUDA matrix");
        for (int i = 0; i < 5; ++i) {
            if (l == 0 && i < 2) continue;  // level 0's coarse_b / coarse_x are unused
            MultiVec *m = mv_checked(g.mv_array_ws[i][l], "BlockAMG workspace");
            GCGE_REQUIRE(m->nrows == A->n && m->ncols >= bs, GCGE_ERR_ARG,
                         "BlockAMG: a workspace has the wrong rows or too few columns");
        }
        if (l + 1 < g.num_levels) {
            Transfer *t = as_transfer(g.P_array[l]);
            SparseMat *Ac = as_mat(g.A_array[l + 1]);
            GCGE_REQUIRE(t != nullptr, GCGE_ERR_HANDLE,
                         "BlockAMG: P_array holds no transfer (CUDA_TransferCreateFromCCS)");
            GCGE_REQUIRE(Ac != nullptr && t->nrows == A->n && t->ncols == Ac->n, GCGE_ERR_ARG,
                         "BlockAMG: P_l must be n_l x n_{l+1}");
        }
    }
}

// ops->MultiLinearSolver installed by the setup (src/ops_lin_sol.c:643-685).
void cuda_block_amg(void *mat, void **mv_b, void **mv_x, int *start_bx, int *end_bx, OPS *ops) {
    (void)mat;  // the cycle uses A_array[0], as the reference does
    AmgRecord *r = nullptr;
    try {
        r = amg_record(ops, false);
        GCGE_REQUIRE(r && ops->multi_linear_solver_workspace == (void *)&r->pub, GCGE_ERR_ARG,
                     "MultiLinearSolver: MultiLinearSolverSetup_BlockAMG was not called on this ops");
        GCGE_REQUIRE(end_bx[0] - start_bx[0] == end_bx[1] - start_bx[1], GCGE_ERR_ARG,
                     "BlockAMG: b and x ranges differ");
        GCGE_REQUIRE(ops->MatDotMultiVec && ops->MultiVecAxpby && ops->MultiVecFromItoJ,
                     GCGE_ERR_ARG, "BlockAMG: ops lacks MatDotMultiVec, MultiVecAxpby or "
                                   "MultiVecFromItoJ");
        const int bs = end_bx[1] - start_bx[1];
        if (bs <= 0) return;
        check_hierarchy(r->pub, bs);
        take_error();
        BlockAMGSolver &g = r->pub;
        g.niter = 0;
        for (int it = 0; it < g.max_iter[0]; ++it) {
            amg_cycle(*r, 0, mv_b, mv_x, start_bx, end_bx, ops);
            ++g.niter;
            if (g.residual < g.tol[0]) break;
        }
    } catch (const CudaError &e) {
        if (r) {
            // leave the AMG solver installed, as a completed solve does
            ops->multi_linear_solver_workspace = (void *)&r->pub;
            ops->MultiLinearSolver = cuda_block_amg;
        }
        set_error(e.status, e.where.c_str());
    } catch (const std::bad_alloc &) {
        set_error(GCGE_ERR_ALLOC, "BlockAMG: host allocation");
    }
}

}  // namespace

void amg_release(OPS *ops) {
    AmgRecord *r = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_amg_mu);
        auto it = g_amg.find(ops);
        if (it == g_amg.end()) return;
        r = it->second;
        g_amg.erase(it);
    }
    delete r;
}

}  // namespace gcge

using namespace gcge;

extern "C" {

int CUDA_TransferCreateFromCCS(void **P, int nrows, int ncols, const int *j_col,
                               const int *i_row, const double *data) {
    try {
        GCGE_REQUIRE(P && j_col && nrows > 0 && ncols > 0, GCGE_ERR_ARG,
                     "CUDA_TransferCreateFromCCS: sizes or column pointers");
        GCGE_REQUIRE(j_col[0] == 0, GCGE_ERR_ARG, "CUDA_TransferCreateFromCCS: j_col[0] must be 0");
        for (int j = 0; j < ncols; ++j)
            GCGE_REQUIRE(j_col[j] <= j_col[j + 1], GCGE_ERR_ARG,
                         "CUDA_TransferCreateFromCCS: column pointers must not decrease");
        const long long nnz = j_col[ncols];
        GCGE_REQUIRE(nnz == 0 || (i_row && data), GCGE_ERR_ARG, "CUDA_TransferCreateFromCCS: arrays");
        // CSR of P by a counting sort of the row indices (entries of a row in
        // column order); P^T's CSR is P's CCS as given
        std::vector<int> rp((size_t)nrows + 1, 0), ri((size_t)std::max<long long>(nnz, 1));
        std::vector<double> rv((size_t)std::max<long long>(nnz, 1));
        for (long long e = 0; e < nnz; ++e) {
            GCGE_REQUIRE(i_row[e] >= 0 && i_row[e] < nrows, GCGE_ERR_ARG,
                         "CUDA_TransferCreateFromCCS: row index out of range");
            ++rp[(size_t)i_row[e] + 1];
        }
        for (int i = 0; i < nrows; ++i) rp[(size_t)i + 1] += rp[i];
        std::vector<int> fill(rp.begin(), rp.end() - 1);
        for (int j = 0; j < ncols; ++j)
            for (int e = j_col[j]; e < j_col[j + 1]; ++e) {
                const int at = fill[i_row[e]]++;
                ri[at] = j;
                rv[at] = data[e];
            }
        Transfer *t = new Transfer();
        try {
            cudaStream_t st = lib_stream();
            t->nrows = nrows;
            t->ncols = ncols;
            t->nnz = nnz;
            const size_t ne = (size_t)std::max<long long>(nnz, 1);
            t->p_ptr.alloc((size_t)nrows + 1);
            t->t_ptr.alloc((size_t)ncols + 1);
            t->p_ind.alloc(ne);
            t->t_ind.alloc(ne);
            t->p_val.alloc(ne);
            t->t_val.alloc(ne);
            GCGE_CUDA(cudaMemcpyAsync(t->p_ptr.p, rp.data(), sizeof(int) * rp.size(),
                                      cudaMemcpyHostToDevice, st));
            GCGE_CUDA(cudaMemcpyAsync(t->t_ptr.p, j_col, sizeof(int) * ((size_t)ncols + 1),
                                      cudaMemcpyHostToDevice, st));
            if (nnz > 0) {
                GCGE_CUDA(cudaMemcpyAsync(t->p_ind.p, ri.data(), sizeof(int) * nnz,
                                          cudaMemcpyHostToDevice, st));
                GCGE_CUDA(cudaMemcpyAsync(t->p_val.p, rv.data(), sizeof(double) * nnz,
                                          cudaMemcpyHostToDevice, st));
                GCGE_CUDA(cudaMemcpyAsync(t->t_ind.p, i_row, sizeof(int) * nnz,
                                          cudaMemcpyHostToDevice, st));
                GCGE_CUDA(cudaMemcpyAsync(t->t_val.p, data, sizeof(double) * nnz,
                                          cudaMemcpyHostToDevice, st));
            }
            GCGE_CUDA(cudaStreamSynchronize(st));  // the host arrays may go after return
        } catch (...) {
            delete t;
            throw;
        }
        *P = t;
        return GCGE_OK;
    } catch (const CudaError &e) {
        set_error(e.status, e.where.c_str());
        take_error();
        return e.status;
    } catch (const std::bad_alloc &) {
        return GCGE_ERR_ALLOC;
    }
}

void CUDA_TransferDestroy(void **P) {
    if (!P || !*P) return;
    Transfer *t = as_transfer(*P);
    if (!t) {
        set_error(GCGE_ERR_HANDLE, "CUDA_TransferDestroy");
        return;
    }
    cudaStreamSynchronize(lib_stream());
    t->magic = 0;
    delete t;
    *P = nullptr;
}

void CUDA_MultiVecFromItoJ(void **P_array, int level_i, int level_j, void **mv_i, void **mv_j,
                           int *startIJ, int *endIJ, void ***mv_ws, OPS *ops) {
    (void)ops;
    try {
        GCGE_REQUIRE(P_array && startIJ && endIJ, GCGE_ERR_ARG, "MultiVecFromItoJ: arguments");
        const int k = endIJ[0] - startIJ[0];
        GCGE_REQUIRE(k == endIJ[1] - startIJ[1] && k >= 0, GCGE_ERR_ARG,
                     "MultiVecFromItoJ: ranges differ");
        MultiVec *src = mv_checked(mv_i, "MultiVecFromItoJ");
        MultiVec *dstv = mv_checked(mv_j, "MultiVecFromItoJ");
        GCGE_REQUIRE(startIJ[0] >= 0 && endIJ[0] <= src->ncols && startIJ[1] >= 0 &&
                         endIJ[1] <= dstv->ncols,
                     GCGE_ERR_ARG, "MultiVecFromItoJ: column range");
        if (k == 0 || level_i == level_j) {
            if (k > 0) {
                GCGE_REQUIRE(src->nrows == dstv->nrows, GCGE_ERR_ARG, "MultiVecFromItoJ: rows");
                copy_cols(src->nrows, k, src->data + (size_t)startIJ[0] * src->ld, src->ld,
                          dstv->data + (size_t)startIJ[1] * dstv->ld, dstv->ld, lib_stream());
            }
            return;
        }
        cudaStream_t st = lib_stream();
        const int step = level_j > level_i ? 1 : -1;
        int s0 = startIJ[0];
        for (int l = level_i; l != level_j; l += step) {
            const int next = l + step;
            Transfer *t = as_transfer(P_array[step > 0 ? l : next]);
            GCGE_REQUIRE(t != nullptr, GCGE_ERR_HANDLE, "MultiVecFromItoJ: P_array holds no transfer");
            MultiVec *dst;
            int d0;
            if (next == level_j) {
                dst = dstv;
                d0 = startIJ[1];
            } else {
                GCGE_REQUIRE(mv_ws != nullptr, GCGE_ERR_ARG,
                             "MultiVecFromItoJ: workspace needed between levels");
                dst = mv_checked(mv_ws[next], "MultiVecFromItoJ workspace");
                GCGE_REQUIRE(dst->ncols >= k, GCGE_ERR_ARG, "MultiVecFromItoJ: workspace width");
                d0 = 0;
            }
            // restriction: P^T (ncols rows) on fine columns; prolongation: P
            const bool down = step > 0;
            const int rows = down ? t->ncols : t->nrows, cols = down ? t->nrows : t->ncols;
            GCGE_REQUIRE(src->nrows == cols && dst->nrows == rows, GCGE_ERR_ARG,
                         "MultiVecFromItoJ: block rows do not match the transfer");
            csr_mm(rows, down ? t->t_ptr.p : t->p_ptr.p, down ? t->t_ind.p : t->p_ind.p,
                   down ? t->t_val.p : t->p_val.p, src->data + (size_t)s0 * src->ld, src->ld,
                   dst->data + (size_t)d0 * dst->ld, dst->ld, k, st);
            src = dst;
            s0 = d0;
        }
    } catch (const CudaError &e) {
        set_error(e.status, e.where.c_str());
    }
}

void MultiLinearSolverSetup_BlockAMG(int *max_iter, double *rate, double *tol,
                                     const char *tol_type, void **A_array, void **P_array,
                                     int num_levels, void ***mv_array_ws[5], double *dbl_ws,
                                     int *int_ws, void *pc, OPS *ops) {
    if (!ops) return;
    try {
        GCGE_REQUIRE(max_iter && rate && tol && A_array && mv_array_ws && num_levels >= 1,
                     GCGE_ERR_ARG, "MultiLinearSolverSetup_BlockAMG: arguments");
        AmgRecord *r = amg_record(ops, true);
        // the caller's arrays are kept and read at every solve, as the
        // reference does: 2 num_levels iteration caps (cycles, then each
        // level's pre- and post-smoothing caps; the coarsest level's solve
        // takes entry 2 num_levels - 1), num_levels rates and tolerances
        BlockAMGSolver &g = r->pub;
        g.max_iter = max_iter;
        g.rate = rate;
        g.tol = tol;
        std::memset(g.tol_type, 0, sizeof(g.tol_type));
        if (tol_type) std::strncpy(g.tol_type, tol_type, sizeof(g.tol_type) - 1);
        g.A_array = A_array;
        g.P_array = P_array;
        g.num_levels = num_levels;
        for (int i = 0; i < 5; ++i) g.mv_array_ws[i] = mv_array_ws[i];
        g.dbl_ws = dbl_ws;
        g.int_ws = int_ws;
        g.pc = pc;
        g.niter = 0;
        g.residual = -1.0;
        ops->multi_linear_solver_workspace = (void *)&g;
        ops->MultiLinearSolver = cuda_block_amg;
    } catch (const CudaError &e) {
        set_error(e.status, e.where.c_str());
    } catch (const std::bad_alloc &) {
        set_error(GCGE_ERR_ALLOC, "MultiLinearSolverSetup_BlockAMG");
    }
}

}  // extern "C"
