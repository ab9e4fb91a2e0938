// MultiLinearSolverSetup_BlockPCG and the block conjugate gradient it installs
// as ops->MultiLinearSolver: the reference's linear-solver hook
// (src/ops_lin_sol.c:439-465 setup, :140-437 BlockPCG) over CUDA multivectors.
//
// The setup keeps its parameters per ops object (the reference keeps one
// static BlockPCGSolver for the whole process) and points
// ops->multi_linear_solver_workspace at a BlockPCGSolver with the reference's
// layout, whose niter / residual the solve fills in.  The solve takes one of
// two routes with the same iteration:
//  * no operator callback (MatDotMultiVec NULL), a CUDA matrix, and an "abs"
//    or "rel" tolerance: the persistent block-PCG kernel (pcg.cu), one launch
//    per 40 columns (the columns are independent CG solves);
//  * otherwise (the caller's operator callback, e.g. the reference's shifted
//    product MatDotMultiVecShift, or the "user" tolerance with norms from
//    dbl_ws): the reference's host-driven loop step for step - the callback or
//    ops->MatDotMultiVec for the products, on the same column ranges and with
//    the same workspace arguments; per-column updates and dots on the device;
//    the convergence bookkeeping on the host.
#include <cmath>
#include <cstring>
#include <mutex>
#include <unordered_map>
#include <vector>

#include "gcg.cuh"
#include "pcg.cuh"

namespace gcge {
namespace {

constexpr int kChunkCols = 40;  // widest block the persistent kernel takes

struct LinSolRecord {
    BlockPCGSolver pub;  // ops->multi_linear_solver_workspace points here
    SolverCtx ctx;       // union pattern and PCG work of the persistent route
    DevBuf<int> dcols;
    DevBuf<double> dcoef, dots, scr;
    PinnedBuf<double> hstage;
    PinnedBuf<int> hcols;
};

std::mutex g_ls_mu;
std::unordered_map<OPS *, LinSolRecord *> g_ls;

LinSolRecord *record_for(OPS *ops, bool create) {
    std::lock_guard<std::mutex> lk(g_ls_mu);
    auto it = g_ls.find(ops);
    if (it != g_ls.end()) return it->second;
    if (!create) return nullptr;
    LinSolRecord *r = new LinSolRecord();
    g_ls[ops] = r;
    return r;
}

// Y(:, cols[i] + yoff) <- per mode, for i < ncols:
//   0: X(:, cols[i]) + coef[i] Y(:, cols[i])  (coef 0: a copy of X)
//   1: Y + coef[i] X(:, cols[i])
__global__ void k_cols_update(int n, int ncols, const int *__restrict__ cols,
                              const double *__restrict__ coef, const double *__restrict__ X,
                              int ldx, double *__restrict__ Y, int ldy, int yoff, int mode) {
    const int j = blockIdx.y;
    if (j >= ncols) return;
    const int c = cols[j];
    const double a = coef[j];
    const double *x = X + (size_t)c * ldx;
    double *y = Y + (size_t)(c + yoff) * ldy;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (mode == 0) y[i] = a == 0.0 ? x[i] : fma(a, y[i], x[i]);
        else y[i] = fma(a, x[i], y[i]);
    }
}

void cols_update(LinSolRecord &r, int n, const std::vector<int> &cols, const std::vector<double> &coef,
                 const double *X, int ldx, double *Y, int ldy, int yoff, int mode,
                 cudaStream_t st) {
    const int m = (int)cols.size();
    if (m == 0 || n == 0) return;
    // staging is reused by the next call only after this stream has passed
    // the copies (the host loop synchronises once per iteration before it
    // writes the staging again)
    r.hcols.alloc(m);
    r.hstage.alloc(m);
    GCGE_CUDA(cudaStreamSynchronize(st));
    std::memcpy(r.hcols.p, cols.data(), sizeof(int) * m);
    std::memcpy(r.hstage.p, coef.data(), sizeof(double) * m);
    r.dcols.alloc(m);
    r.dcoef.alloc(m);
    GCGE_CUDA(cudaMemcpyAsync(r.dcols.p, r.hcols.p, sizeof(int) * m, cudaMemcpyHostToDevice, st));
    GCGE_CUDA(cudaMemcpyAsync(r.dcoef.p, r.hstage.p, sizeof(double) * m, cudaMemcpyHostToDevice,
                              st));
    const int gx = std::max(1, std::min((n + 255) / 256, 2 * device_sms() / std::max(1, m) + 1));
    k_cols_update<<<dim3(gx, m), 256, 0, st>>>(n, m, r.dcols.p, r.dcoef.p, X, ldx, Y, ldy, yoff,
                                               mode);
    GCGE_CHECK_LAUNCH();
    count_launch();
}

// Column dots X(:, c) . Y(:, c) for c in [lo, hi), to the host.
void col_dots(LinSolRecord &r, int n, int lo, int hi, const double *X, int ldx, const double *Y,
              int ldy, double *out, cudaStream_t st) {
    const int k = hi - lo;
    if (k <= 0) return;
    r.dots.alloc(k);
    r.scr.alloc((size_t)k * 4096);
    coldot(n, k, X + (size_t)lo * ldx, ldx, Y + (size_t)lo * ldy, ldy, r.dots.p, r.scr.p, r.scr.n,
           st);
    r.hstage.alloc(k);
    GCGE_CUDA(cudaMemcpyAsync(r.hstage.p, r.dots.p, sizeof(double) * k, cudaMemcpyDeviceToHost,
                              st));
    GCGE_CUDA(cudaStreamSynchronize(st));
    std::memcpy(out, r.hstage.p, sizeof(double) * k);
}

MultiVec *mv_of(void **h, const char *what) {
    MultiVec *m = as_mv(h);
    GCGE_REQUIRE(m != nullptr, GCGE_ERR_HANDLE, std::string(what) + ": not a CUDA multivector");
    return m;
}

// The persistent route: columns [sb, eb) of b and [sx, sx + k) of x, in
// chunks of at most 40 columns.
void solve_persistent(LinSolRecord &r, SparseMat *A, MultiVec *bv, int sb, MultiVec *xv, int sx,
                      int k, cudaStream_t st) {
    BlockPCGSolver &p = r.pub;
    SolverCtx &c = r.ctx;
    const int n = A->n;
    const bool rel = std::strcmp(p.tol_type, "rel") == 0;
    prepare_union(c, A, nullptr, st);
    c.reserve(n, kChunkCols, kChunkCols, kChunkCols, spmm_blocks(c.upat));
    // S = A (the identity's slots of the union pattern carry zero shift)
    shift_values(c.upat.padded, c.ua.p, c.ub.p, 0.0, c.us64.p, nullptr, st);
    int niter = 0;
    double residual = -1.0;
    // The reference runs one list of unconverged columns over the whole block
    // and reports last_res[unconv[0]] (src/ops_lin_sol.c:406-410): the first
    // column still iterating at the end, else (the list is compacted in place)
    // the first column that entered the last iteration; init_res[0] when no
    // iteration ran.  Chunks iterate independently, so each chunk's candidates
    // are kept until the block's iteration count is known.
    struct Candidate {
        int it;
        double active_res, entered_res, init0;
        bool active, entered;
    };
    std::vector<Candidate> cand;
    for (int c0 = 0; c0 < k; c0 += kChunkCols) {
        const int kc = std::min(kChunkCols, k - c0);
        const int kp = rows_width(kc, 8);
        col_to_rows<double, double>(n, kc, kp, xv->data + (size_t)(sx + c0) * xv->ld, xv->ld,
                                    c.xr64.p, st);
        col_to_rows<double, double>(n, kc, kp, bv->data + (size_t)(sb + c0) * bv->ld, bv->ld,
                                    c.br64.p, st);
        block_pcg_rows<double>(c.pcg, c.upat, c.us64.p, c.br64.p, c.xr64.p, c.rr64.p, c.pr64.p,
                               c.wr64.p, kp, kc, p.max_iter, p.rate, p.tol, rel, false, st);
        rows_to_col<double, double>(n, kc, kp, c.xr64.p, xv->data + (size_t)(sx + c0) * xv->ld,
                                    xv->ld, false, st);
        const int it = pcg_last_iters(c.pcg, st);
        PcgScalars hs;
        GCGE_CUDA(cudaMemcpyAsync(&hs, c.pcg.sc.p, sizeof(PcgScalars), cudaMemcpyDeviceToHost, st));
        GCGE_CUDA(cudaStreamSynchronize(st));
        Candidate cd{it, 0.0, 0.0, hs.init_res[0], false, false};
        for (int j = 0; j < kc; ++j)
            if (hs.active[j]) {
                cd.active = true;
                cd.active_res = hs.last_res[j];
                break;
            }
        for (int j = 0; j < kc && it > 0; ++j)
            if (hs.active[j] || hs.left_at[j] == it) {
                cd.entered = true;
                cd.entered_res = hs.last_res[j];
                break;
            }
        cand.push_back(cd);
        niter = std::max(niter, it);
    }
    if (niter == 0) {
        residual = cand.empty() ? -1.0 : cand[0].init0;
    } else {
        bool found = false;
        for (const Candidate &cd : cand)
            if (cd.it == niter && cd.active) {
                residual = cd.active_res;
                found = true;
                break;
            }
        for (size_t i = 0; i < cand.size() && !found; ++i)
            if (cand[i].it == niter && cand[i].entered) {
                residual = cand[i].entered_res;
                found = true;
            }
    }
    p.niter = niter;
    p.residual = residual;
}

// The host-driven route: src/ops_lin_sol.c:140-437 step for step.
void solve_generic(LinSolRecord &r, void *mat, void **mv_b, void **mv_x, const int *start_bx,
                   const int *end_bx, OPS *ops, cudaStream_t st) {
    BlockPCGSolver &p = r.pub;
    void **mv_r = p.mv_ws[0], **mv_p = p.mv_ws[1], **mv_w = p.mv_ws[2];
    GCGE_REQUIRE(mv_r && mv_p && mv_w, GCGE_ERR_ARG,
                 "BlockPCG: the r, p, w workspaces (mv_ws) are required with an operator "
                 "callback or the \"user\" tolerance");
    MultiVec *R = mv_of(mv_r, "BlockPCG r"), *Pm = mv_of(mv_p, "BlockPCG p"),
             *Wm = mv_of(mv_w, "BlockPCG w"), *Xm = mv_of(mv_x, "BlockPCG x"),
             *Bm = mv_of(mv_b, "BlockPCG b");
    const int k0 = end_bx[0] - start_bx[0];
    const int n = Bm->nrows;
    GCGE_REQUIRE(R->ncols >= k0 && Pm->ncols >= k0 && Wm->ncols >= k0, GCGE_ERR_ARG,
                 "BlockPCG: workspace narrower than the block");
    GCGE_REQUIRE(p.MatDotMultiVec != nullptr || ops->MatDotMultiVec != nullptr, GCGE_ERR_ARG,
                 "BlockPCG: no operator");
    const double rate = p.rate, tol = p.tol;
    std::vector<double> norm_b(k0, 1.0), rho1(k0), rho2(k0), ptw(k0), init_res(k0), last_res(k0),
        tmp(k0);
    std::vector<int> unconv(k0);
    int start[2], end[2];
    if (std::strcmp(p.tol_type, "rel") == 0) {
        col_dots(r, n, start_bx[0], end_bx[0], Bm->data, Bm->ld, Bm->data, Bm->ld, norm_b.data(),
                 st);
        for (double &v : norm_b) v = std::sqrt(v);
    } else if (std::strcmp(p.tol_type, "user") == 0) {
        GCGE_REQUIRE(p.dbl_ws != nullptr, GCGE_ERR_ARG, "BlockPCG: \"user\" norms need dbl_ws");
        for (int i = 0; i < k0; ++i) norm_b[i] = std::fabs(p.dbl_ws[i]);
    }
    // r = b - op(x)
    start[0] = start_bx[1];
    end[0] = end_bx[1];
    start[1] = 0;
    end[1] = k0;
    if (p.MatDotMultiVec) p.MatDotMultiVec(mv_x, mv_r, start, end, mv_p, 0, ops);
    else ops->MatDotMultiVec(mat, mv_x, mv_r, start, end, ops);
    const int e0 = take_error();
    if (e0 != GCGE_OK) throw CudaError{e0, "BlockPCG: operator"};
    axpby(n, k0, 1.0, Bm->data + (size_t)start_bx[0] * Bm->ld, Bm->ld, -1.0, R->data, R->ld, st);
    col_dots(r, n, 0, k0, R->data, R->ld, R->data, R->ld, rho2.data(), st);
    for (int i = 0; i < k0; ++i) init_res[i] = std::sqrt(rho2[i]);
    int nun = 0;
    for (int i = 0; i < k0; ++i)
        if (init_res[i] > tol * norm_b[i]) {
            unconv[nun] = i;
            rho2[nun] = rho2[i];
            ++nun;
        }
    int niter = 0;
    std::vector<int> cols;
    std::vector<double> coef;
    while (niter < p.max_iter && nun > 0) {
        // runs of consecutive unconverged columns
        std::vector<int> block{0};
        for (int i = 1; i < nun; ++i)
            if (unconv[i] - unconv[i - 1] > 1) block.push_back(i);
        block.push_back(nun);
        // p = r + beta p
        cols.assign(unconv.begin(), unconv.begin() + nun);
        coef.resize(nun);
        for (int i = 0; i < nun; ++i) coef[i] = niter == 0 ? 0.0 : rho2[i] / rho1[i];
        cols_update(r, n, cols, coef, R->data, R->ld, Pm->data, Pm->ld, 0, 0, st);
        // w = op(p) and p^T w, run by run
        for (size_t b = 0; b + 1 < block.size(); ++b) {
            const int lo = unconv[block[b]], hi = unconv[block[b + 1] - 1] + 1;
            start[0] = start[1] = lo;
            end[0] = end[1] = hi;
            if (p.MatDotMultiVec) p.MatDotMultiVec(mv_p, mv_w, start, end, mv_b, start_bx[0], ops);
            else ops->MatDotMultiVec(mat, mv_p, mv_w, start, end, ops);
            const int e = take_error();
            if (e != GCGE_OK) throw CudaError{e, "BlockPCG: operator"};
            col_dots(r, n, lo, hi, Pm->data, Pm->ld, Wm->data, Wm->ld, tmp.data(), st);
            for (int i = block[b]; i < block[b + 1]; ++i) ptw[i] = tmp[unconv[i] - lo];
        }
        for (int i = 0; i < nun; ++i) rho1[i] = rho2[i];
        // x += alpha p, r -= alpha w
        for (int i = 0; i < nun; ++i) coef[i] = rho2[i] / ptw[i];
        cols_update(r, n, cols, coef, Pm->data, Pm->ld, Xm->data, Xm->ld, start_bx[1], 1, st);
        for (int i = 0; i < nun; ++i) coef[i] = -coef[i];
        cols_update(r, n, cols, coef, Wm->data, Wm->ld, R->data, R->ld, 0, 1, st);
        for (size_t b = 0; b + 1 < block.size(); ++b) {
            const int lo = unconv[block[b]], hi = unconv[block[b + 1] - 1] + 1;
            col_dots(r, n, lo, hi, R->data, R->ld, R->data, R->ld, tmp.data(), st);
            for (int i = block[b]; i < block[b + 1]; ++i) rho2[i] = tmp[unconv[i] - lo];
        }
        for (int i = 0; i < nun; ++i) last_res[unconv[i]] = std::sqrt(rho2[i]);
        const int pre = nun;
        nun = 0;
        for (int i = 0; i < pre; ++i) {
            const int col = unconv[i];
            if (last_res[col] > rate * init_res[col] && last_res[col] > tol * norm_b[col]) {
                unconv[nun] = col;
                rho1[nun] = rho1[i];
                rho2[nun] = rho2[i];
                ++nun;
            }
        }
        ++niter;
    }
    p.niter = niter;
    p.residual = niter > 0 ? last_res[unconv[0]] : init_res[0];
    GCGE_CUDA(cudaStreamSynchronize(st));
}

void cuda_block_pcg(void *mat, void **mv_b, void **mv_x, int *start_bx, int *end_bx, OPS *ops) {
    try {
        LinSolRecord *r = record_for(ops, false);
        GCGE_REQUIRE(r && ops->multi_linear_solver_workspace == (void *)&r->pub, GCGE_ERR_ARG,
                     "MultiLinearSolver: MultiLinearSolverSetup_BlockPCG was not called on this ops");
        GCGE_REQUIRE(end_bx[0] - start_bx[0] == end_bx[1] - start_bx[1], GCGE_ERR_ARG,
                     "BlockPCG: b and x ranges differ");
        const int k = end_bx[0] - start_bx[0];
        MultiVec *bv = mv_of(mv_b, "BlockPCG b"), *xv = mv_of(mv_x, "BlockPCG x");
        GCGE_REQUIRE(start_bx[0] >= 0 && end_bx[0] <= bv->ncols && start_bx[1] >= 0 &&
                         end_bx[1] <= xv->ncols && bv->nrows == xv->nrows,
                     GCGE_ERR_ARG, "BlockPCG: column range");
        if (k <= 0) {
            r->pub.niter = 0;
            return;
        }
        cudaStream_t st = lib_stream();
        SparseMat *A = mat ? as_mat(mat) : nullptr;
        const bool persistent = r->pub.MatDotMultiVec == nullptr && A != nullptr &&
                                (std::strcmp(r->pub.tol_type, "abs") == 0 ||
                                 std::strcmp(r->pub.tol_type, "rel") == 0);
        if (persistent) solve_persistent(*r, A, bv, start_bx[0], xv, start_bx[1], k, st);
        else solve_generic(*r, mat, mv_b, mv_x, start_bx, end_bx, ops, st);
    } catch (const CudaError &e) {
        set_error(e.status, e.where.c_str());
    } catch (const std::bad_alloc &) {
        set_error(GCGE_ERR_ALLOC, "BlockPCG: host allocation");
    }
}

}  // namespace

void linsol_release(OPS *ops) {
    LinSolRecord *r = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_ls_mu);
        auto it = g_ls.find(ops);
        if (it == g_ls.end()) return;
        r = it->second;
        g_ls.erase(it);
    }
    delete r;
}

}  // namespace gcge

using namespace gcge;

extern "C" void MultiLinearSolverSetup_BlockPCG(
    int max_iter, double rate, double tol, const char *tol_type, void **mv_ws[3], double *dbl_ws,
    int *int_ws, void *pc,
    void (*MatDotMultiVec)(void **x, void **y, int *start, int *end, void **z, int s, OPS *ops),
    OPS *ops) {
    if (!ops) return;
    try {
        LinSolRecord *r = record_for(ops, true);
        BlockPCGSolver &p = r->pub;
        p.max_iter = max_iter;
        p.rate = rate;
        p.tol = tol;
        std::memset(p.tol_type, 0, sizeof(p.tol_type));
        if (tol_type) std::strncpy(p.tol_type, tol_type, sizeof(p.tol_type) - 1);
        for (int i = 0; i < 3; ++i) p.mv_ws[i] = mv_ws ? mv_ws[i] : nullptr;
        p.dbl_ws = dbl_ws;
        p.int_ws = int_ws;
        p.pc = pc;
        p.MatDotMultiVec = MatDotMultiVec;
        p.niter = 0;
        p.residual = -1.0;
        ops->multi_linear_solver_workspace = (void *)&p;
        ops->MultiLinearSolver = cuda_block_pcg;
    } catch (const std::bad_alloc &) {
        set_error(GCGE_ERR_ALLOC, "MultiLinearSolverSetup_BlockPCG");
    }
}
