// GPU GCG eigensolver (reference: GCG and its phases, src/ops_eig_sol_gcg.c).
//
// The host runs the reference's control flow - sizes, offsets, locking,
// X expansion - and sees only O(s) scalars per step (residual norms,
// eigenvalues, small Gram blocks); the basis V = [X P W], the Ritz vectors,
// the projected matrices, the PCG state and the operators stay in HBM.
// Phases follow the reference function by function:
//   InitializeX      :102-159   ComputeRitzVec :160-195   CheckConvergence :196-321
//   ComputeP         :322-463   ComputeX       :464-477   ComputeW         :478-701
//   ComputeRayleighRitz :931-1258   GCG outer loop :1259-1562
// Two departures, both GPU-shaped and within the reference's tolerances:
//   * B-orthonormalisation (ModifiedGramSchmidt, src/ops_orth.c:203-394) is a
//     blocked classical Gram-Schmidt against the locked prefix with
//     re-orthogonalisation (same pass count and 50*eps early exit as the
//     reference) followed by Cholesky-QR2 of the new block, dropping columns
//     whose remaining B-norm falls under the zero tolerance.
//   * the dense eigensolve (dsyevx) is the FP32 Jacobi + FP64 Ogita-Aishima
//     refinement of eig.cu.
#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstring>
#include <mutex>
#include <unordered_map>

#include "gcg.cuh"

namespace gcge {

static inline double *colp(MultiVec *X, int c) { return X->data + (size_t)c * X->ld; }
static inline int round32(int n) { return (n + 31) / 32 * 32; }

// ---------------------------------------------------------------- registry
static std::mutex g_ctx_mu;
static std::unordered_map<OPS *, SolverCtx *> g_ctx;

SolverCtx *ctx_for(OPS *ops, bool create) {
    std::lock_guard<std::mutex> lk(g_ctx_mu);
    auto it = g_ctx.find(ops);
    if (it != g_ctx.end()) return it->second;
    if (!create) return nullptr;
    SolverCtx *c = new SolverCtx();
    g_ctx[ops] = c;
    return c;
}
void ctx_release(OPS *ops) {
    SolverCtx *c = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_ctx_mu);
        auto it = g_ctx.find(ops);
        if (it == g_ctx.end()) return;
        c = it->second;
        g_ctx.erase(it);
    }
    delete c;
}

void SolverCtx::reserve(int n_, int nev_max, int nev_init, int bs, int spmm_nblocks) {
    const int smax = nev_max + 2 * bs;
    n = n_;
    ld = round32(n_);
    const int cols = std::max({smax, nev_init, bs, 1});
    if (cols > cap_cols || (size_t)ld * cols > T1.n) {
        T1.alloc((size_t)ld * cols);
        T2.alloc((size_t)ld * cols);
        cap_cols = cols;
    }
    if (bs > cap_bs || (size_t)ld * bs > bbuf.n) {
        bbuf.alloc((size_t)ld * bs);
        r64.alloc((size_t)ld * bs);
        const size_t nr = pcg_block_elems(n_, rows_width(std::min(bs, 40), 8));
        for (auto *b : {&xr64, &br64, &rr64, &pr64, &wr64}) b->alloc(nr);
        cap_bs = bs;
    }
    if (smax > cap_s) {
        const size_t s2 = (size_t)smax * smax;
        M0.alloc(s2);
        M1.alloc(s2);
        evec.alloc(s2);
        work.alloc(s2 + (size_t)smax * bs);
        coefP.alloc((size_t)smax * std::max(bs, 1));
        ptap.alloc((size_t)std::max(bs, 1) * std::max(bs, 1));
        dC.alloc(s2 + (size_t)cols * cols);
        dtmp.alloc(s2 + (size_t)smax * cols);
        dvec.alloc(std::max(smax, 64) * 2);
        dmask.alloc(std::max(smax, 64));
        didx.alloc(std::max(smax, 64));
        hbuf.alloc(s2 + (size_t)cols * cols + 4096);
        hup.alloc((size_t)4 * smax + 256);
        eig.reserve(smax);
        cap_s = smax;
    }
    gscr.alloc(std::max<size_t>(gram_scratch_elems(std::max(n_, smax), smax, cols) +
                                    gram_scratch_elems(n_, cols, cols),
                                2u << 20));
    part.alloc((size_t)std::max(spmm_nblocks, 1) * 64);
    ozb.alloc(oz_lincomb_scratch_bytes(std::max(smax, cols), std::max(smax, cols)));
    dmax.alloc(4);
    hmax.alloc(4);
    if (one.p == nullptr) {
        one.alloc(1);
        fill_value(1, one.p, 1.0, lib_stream());
    }
    pcg.reserve(n_, std::max(bs, 1));
}

// ---------------------------------------------------------------- phase timer
struct PhaseTimer {
    enum { kMaxEvents = 4096 };
    // events come from a per-thread pool that lives as long as the thread: a
    // solve marks ~12 phases per outer iteration, and creating and destroying
    // thousands of events per solve cost the next synchronising call on the
    // stream about 5 ms per outer iteration
    static std::vector<cudaEvent_t> &pool() {
        static thread_local std::vector<cudaEvent_t> p;
        return p;
    }
    static int &depth() {
        static thread_local int d = 0;
        return d;
    }
    size_t used = 0;
    std::vector<int> ph;
    cudaStream_t st;
    bool active;  // a solve started inside another one's callback records nothing
    explicit PhaseTimer(cudaStream_t s) : st(s), active(depth()++ == 0) {}
    ~PhaseTimer() { --depth(); }
    PhaseTimer(const PhaseTimer &) = delete;
    PhaseTimer &operator=(const PhaseTimer &) = delete;
    void mark(int phase) {
        if (!active || (int)used >= kMaxEvents) return;
        std::vector<cudaEvent_t> &p = pool();
        if (used == p.size()) {
            cudaEvent_t e;
            if (cudaEventCreate(&e) != cudaSuccess) return;
            p.push_back(e);
        }
        cudaEventRecord(p[used], st);
        ph.push_back(phase);
        ++used;
    }
    void collect(double *out10) {
        for (int i = 0; i < 10; ++i) out10[i] = 0.0;
        if (used < 2) return;
        const std::vector<cudaEvent_t> &p = pool();
        cudaEventSynchronize(p[used - 1]);
        for (size_t i = 0; i + 1 < used; ++i) {
            float ms = 0.f;
            if (ph[i] >= 0 && ph[i] < 10 && cudaEventElapsedTime(&ms, p[i], p[i + 1]) == cudaSuccess)
                out10[ph[i]] += ms;
        }
    }
};
enum { PH_CHECK = 0, PH_P, PH_RR, PH_RRW, PH_EIG, PH_RV, PH_W, PH_LINSOL, PH_X, PH_INITX, PH_NONE = -1 };

// Products over the long (vector-length) dimension: FP64 FMA kernels in the
// FP64 solve, FP64-accurate digit products on the tensor cores in the mixed
// solve (same results to FP64 accuracy).  The digit products' error bound is
// relative to the largest |x| |y| of each exponent window: FP64-level for the
// n-row blocks, but not for the coefficient vectors of the projected space
// (ComputeP's orthogonalisation and its P^T A P, contractions over s rows),
// whose entries mix O(1) and ~1e-8 values in one window.  Products over fewer
// than kDigitMinRows rows - every projected-space product, since s stays
// below it for nev up to ~300 - therefore stay FP64; they cost next to
// nothing.
constexpr int kDigitMinRows = 1024;

static void dgram(const SolverCtx &c, int n, int m, int w, const double *Q, int ldq,
                  const double *P, int ldp, double *C, int ldc, double *scratch, size_t elems,
                  cudaStream_t st, TcExpCache *qcache = nullptr) {
    if (c.precision == GCGE_PREC_MIXED && !c.escalated && n >= kDigitMinRows)
        oz_gram(n, m, w, Q, ldq, P, ldp, C, ldc, scratch, elems, st, qcache);
    else
        gram(n, m, w, Q, ldq, P, ldp, C, ldc, scratch, elems, st);
}
static void dlincomb(const SolverCtx &c, int n, int k, int m, const double *X, int ldx,
                     const double *C, int ldc, double *Y, int ldy, const double *beta, int incb,
                     cudaStream_t st, double alpha = 1.0, TcExpCache *xcache = nullptr) {
    if (c.precision == GCGE_PREC_MIXED && !c.escalated && n >= kDigitMinRows)
        oz_lincomb(n, k, m, X, ldx, C, ldc, Y, ldy, beta, incb, st, alpha, c.ozb.p, c.ozb.n,
                   xcache);
    else
        lincomb(n, k, m, X, ldx, C, ldc, Y, ldy, beta, incb, st, alpha);
}

// B-orthonormalise columns [start, end) of x (nrows x ldx) against the
// B-orthonormal prefix [0, start) and among themselves; returns the new end
// (columns whose remaining B-norm is below the zero tolerance are dropped).
int borth(SolverCtx &c, SparseMat *B, double *x, int ldx, int nrows, int start, int end,
          bool useB, double zero_tol, int max_reorth, int *spmm_calls) {
    cudaStream_t st = lib_stream();
    const int ld = c.ld;
    auto applyB = [&](const double *X, int lx, double *Y, int ly, int k) {
        if (k <= 0) return;
        if (B) {
            spmm<double>(B->pat, B->val.p, X, lx, Y, ly, k, st);
            if (spmm_calls) ++*spmm_calls;
        } else {
            copy_cols(nrows, k, X, lx, Y, ly, st);
        }
    };
    auto device_absmax = [&](int m, int w, const double *C, int ldc) {
        absmax(m, w, C, ldc, c.dmax.p, st);
        GCGE_CUDA(cudaMemcpyAsync(c.hmax.p, c.dmax.p, sizeof(double), cudaMemcpyDeviceToHost, st));
        GCGE_CUDA(cudaStreamSynchronize(st));
        return c.hmax.p[0];
    };
    if (end <= start) return end;
    int k = end - start;
    double *X1 = x + (size_t)start * ldx;
    bool upload_pending = false;  // a Cholesky-QR coefficient upload from hbuf in flight
    const double reorth_tol = 50.0 * 2.220446049250313e-16;  // src/ops_orth.c:404
    // the prefix x[:, 0:start) does not change here: the exponent fields of
    // its digit products are computed once for all projection passes
    TcExpCache qcache, xcache;
    // Two rounds at most.  Cholesky-QR multiplies the block by R^-1, which
    // scales the rounding-level remainder of the prefix components by up to
    // kappa(R); when the first factor of a round was ill-conditioned
    // (nearly dependent columns, e.g. the two W directions of ComputeW12 or a
    // W column of a nearly converged pair) the prefix projection and the
    // factorisation run once more on the now well-conditioned block.
    for (int round = 0; round < 2 && k > 0; ++round) {
        // c.T2 holds B x1 of the block before the last projection, which
        // changed it by a coefficient block C below reorth_tol: the Gram
        // matrix of the first Cholesky-QR pass taken with it differs from
        // x1^T B x1 by (X^T B x1)^T C, of order eps * reorth_tol, so that pass
        // needs no product of its own
        bool bx1_kept = false;
        if (start > 0) {
            for (int pass = 0; pass < 1 + max_reorth; ++pass) {
                const double *BX1 = X1;
                if (useB) {
                    applyB(X1, ldx, c.T2.p, ld, k);
                    BX1 = c.T2.p;
                }
                dgram(c, nrows, start, k, x, ldx, BX1, useB ? ld : ldx, c.dC.p, start, c.gscr.p,
                      c.gscr.n, st, &qcache);
                dlincomb(c, nrows, start, k, x, ldx, c.dC.p, start, X1, ldx, c.one.p, 0, st, -1.0,
                         &xcache);
                if (pass >= 1 || max_reorth == 0) {
                    if (device_absmax(start, k, c.dC.p, start) < reorth_tol) {
                        bx1_kept = useB;
                        break;
                    }
                }
            }
        }
        double kappa = 1.0;  // max over kept columns of |x_j| / |new part of x_j| (first pass)
        // Cholesky-QR of the new block with column dropping, repeated until its
        // Gram matrix is the identity to 1e-13
        for (int pass = 0; pass < 4 && k > 0; ++pass) {
            const double *BX1 = X1;
            if (useB) {
                if (!(pass == 0 && bx1_kept)) applyB(X1, ldx, c.T2.p, ld, k);
                BX1 = c.T2.p;
            }
            dgram(c, nrows, k, k, X1, ldx, BX1, useB ? ld : ldx, c.dC.p, k, c.gscr.p, c.gscr.n, st);
            GCGE_CUDA(cudaMemcpyAsync(c.hbuf.p, c.dC.p, sizeof(double) * k * k,
                                      cudaMemcpyDeviceToHost, st));
            GCGE_CUDA(cudaStreamSynchronize(st));
            upload_pending = false;
            const double *G = c.hbuf.p;
            double offmax = 0.0;
            for (int a = 0; a < k; ++a)
                for (int b = 0; b < k; ++b)
                    offmax = std::max(offmax, std::fabs(G[a + (size_t)b * k] - (a == b ? 1.0 : 0.0)));
            if (pass >= 1 && offmax < 1e-13) break;
            // upper Cholesky R^T R = G restricted to the kept columns
            std::vector<int> kept;
            std::vector<double> R((size_t)k * k, 0.0);  // R[a + b*k], a = kept row index
            for (int j = 0; j < k; ++j) {
                GCGE_REQUIRE(std::isfinite(G[j + (size_t)j * k]), GCGE_ERR_NUMERIC,
                             "orth: non-finite Gram matrix");
                const int nk = (int)kept.size();
                std::vector<double> rj(nk);
                double d = G[j + (size_t)j * k];
                for (int a = 0; a < nk; ++a) {
                    double v = G[kept[a] + (size_t)j * k];
                    for (int b = 0; b < a; ++b) v -= R[b + (size_t)a * k] * rj[b];
                    v /= R[a + (size_t)a * k];
                    rj[a] = v;
                    d -= v * v;
                }
                const double gjj = std::max(G[j + (size_t)j * k], 0.0);
                const double thr = std::max(zero_tol, 1e-7 * std::sqrt(gjj));
                if (!(d > thr * thr)) continue;  // dependent column: drop
                if (pass == 0) kappa = std::max(kappa, std::sqrt(gjj / d));
                for (int a = 0; a < nk; ++a) R[a + (size_t)nk * k] = rj[a];
                R[nk + (size_t)nk * k] = std::sqrt(d);
                kept.push_back(j);
            }
            const int kk = (int)kept.size();
            // coefficient matrix Cf (k x kk): Cf[kept[a], b] = (R^{-1})[a, b]
            std::vector<double> Ri((size_t)kk * kk, 0.0);
            for (int b = 0; b < kk; ++b) {
                Ri[b + (size_t)b * kk] = 1.0 / R[b + (size_t)b * k];
                for (int a = b - 1; a >= 0; --a) {
                    double v = 0.0;
                    for (int l = a + 1; l <= b; ++l) v += R[a + (size_t)l * k] * Ri[l + (size_t)b * kk];
                    Ri[a + (size_t)b * kk] = -v / R[a + (size_t)a * k];
                }
            }
            double *Cf = c.hbuf.p + (size_t)k * k;
            std::fill(Cf, Cf + (size_t)k * std::max(kk, 1), 0.0);
            for (int a = 0; a < kk; ++a)
                for (int b = 0; b < kk; ++b) Cf[kept[a] + (size_t)b * k] = Ri[a + (size_t)b * kk];
            if (kk > 0) {
                GCGE_CUDA(cudaMemcpyAsync(c.dC.p, Cf, sizeof(double) * k * kk,
                                          cudaMemcpyHostToDevice, st));
                dlincomb(c, nrows, k, kk, X1, ldx, c.dC.p, k, c.T1.p, ld, nullptr, 0, st);
                copy_cols(nrows, kk, c.T1.p, ld, X1, ldx, st);
            }
            k = kk;
            // the next pass downloads its Gram matrix into hbuf[0, k^2), apart
            // from this upload's source, and waits for that download (so for
            // this upload) before writing hbuf again; the caller may reuse
            // hbuf at once, so the last upload is waited for on return
            upload_pending = kk > 0;
            // two factorisations of a block with kappa < 1e5 leave it orthonormal
            // to rounding (Cholesky-QR2 is stable for kappa^2 eps < 1): its
            // Gram matrix need not be formed again to check
            if (pass == 1 && kappa < 1e5) break;
        }
        if (start == 0 || kappa < 1e3) break;
    }
    if (upload_pending) GCGE_CUDA(cudaStreamSynchronize(st));
    return start + k;
}

// ---------------------------------------------------------------- BGS
// BinaryGramSchmidt (src/ops_orth.c:416-641): classical Gram-Schmidt of the
// new columns against the prefix, then recursive halving; the leaves are
// orthonormalised column by column (OrthSelf, :45-118) when the whole block
// has fewer than 16 columns, else by the eigen-decomposition of their Gram
// matrix (OrthSelfEVP, :122-201).  Tall products run on the device, the leaf
// decisions (drops, eigen-decompositions of k x k Gram matrices) on the host.
struct BgsOrth {
    SolverCtx &c;
    SparseMat *B;
    int nrows;
    bool useB;
    double zero_tol;
    int max_reorth;
    int block_size;
    int *spmm_calls;
    cudaStream_t st;
    bool evp = true;  // leaf method: OrthSelfEVP (true) or OrthSelf
    static constexpr double kReorthTol = 50.0 * 2.220446049250313e-16;  // src/ops_orth.c:631

    void applyB(const double *X, int lx, double *Y, int ly, int k) {
        if (k <= 0) return;
        if (B) {
            spmm<double>(B->pat, B->val.p, X, lx, Y, ly, k, st);
            if (spmm_calls) ++*spmm_calls;
        } else {
            copy_cols(nrows, k, X, lx, Y, ly, st);
        }
    }
    double absmax_dev(int m, int w, const double *C, int ldc) {
        absmax(m, w, C, ldc, c.dmax.p, st);
        GCGE_CUDA(cudaMemcpyAsync(c.hmax.p, c.dmax.p, sizeof(double), cudaMemcpyDeviceToHost, st));
        GCGE_CUDA(cudaStreamSynchronize(st));
        return c.hmax.p[0];
    }
    // X1 -= X0 (X0^T B X1), up to 1 + max_reorth passes, until the
    // coefficients fall below the reorthogonalisation tolerance; B X0 is formed
    // once (:446-481)
    void cgs(double *X0, int n0, double *X1, int n1, int ldx) {
        if (n0 <= 0 || n1 <= 0) return;
        const double *BX0 = X0;
        int ldb = ldx;
        if (useB) {
            applyB(X0, ldx, c.T2.p, c.ld, n0);
            BX0 = c.T2.p;
            ldb = c.ld;
        }
        TcExpCache qcache, xcache;  // B X0 and X0 stay unchanged over the passes
        for (int pass = 0; pass < 1 + max_reorth; ++pass) {
            dgram(c, nrows, n0, n1, BX0, ldb, X1, ldx, c.dC.p, n0, c.gscr.p, c.gscr.n, st,
                  &qcache);
            dlincomb(c, nrows, n0, n1, X0, ldx, c.dC.p, n0, X1, ldx, c.one.p, 0, st, -1.0,
                     &xcache);
            if (absmax_dev(n0, n1, c.dC.p, n0) < kReorthTol) break;
        }
    }
    // OrthSelf: column by column, normalise x_k by its B-norm (drop it, moving
    // the last column into its place, when the norm is below the zero
    // tolerance) and remove it from the later columns
    int self_mgs(double *x, int ldx, int lo, int hi) {
        for (int k = lo; k < hi; ++k) {
            double *xk = x + (size_t)k * ldx;
            const double *Bxk = xk;
            int ldb = ldx;
            if (useB) {
                applyB(xk, ldx, c.T2.p, c.ld, 1);
                Bxk = c.T2.p;
                ldb = c.ld;
            }
            const int len = hi - k;
            dgram(c, nrows, len, 1, xk, ldx, Bxk, ldb, c.dC.p, len, c.gscr.p, c.gscr.n, st);
            GCGE_CUDA(cudaMemcpyAsync(c.hbuf.p, c.dC.p, sizeof(double) * len,
                                      cudaMemcpyDeviceToHost, st));
            GCGE_CUDA(cudaStreamSynchronize(st));
            const double r = std::sqrt(c.hbuf.p[0]);  // NaN (kept) for a negative square
            if (r < zero_tol) {
                if (k < hi - 1) copy_cols(nrows, 1, x + (size_t)(hi - 1) * ldx, ldx, xk, ldx, st);
                --k;
                --hi;
                continue;
            }
            const double inv = 1.0 / r;
            double *hc = c.hbuf.p + len;  // [1/r, coefficients of the later columns]
            hc[0] = inv;
            for (int i = 1; i < len; ++i) hc[i] = c.hbuf.p[i] * -inv;
            GCGE_CUDA(cudaMemcpyAsync(c.dC.p, hc, sizeof(double) * len, cudaMemcpyHostToDevice, st));
            scale_columns(nrows, 1, xk, ldx, c.dC.p, st);
            if (len > 1)
                dlincomb(c, nrows, 1, len - 1, xk, ldx, c.dC.p + 1, 1, xk + ldx, ldx, c.one.p, 0, st);
            // further passes against x_k (:93-113; none for max_reorth <= 2)
            for (int idx = 1; idx < max_reorth - 1 && len > 1; ++idx) {
                if (useB) applyB(xk, ldx, c.T2.p, c.ld, 1);
                dgram(c, nrows, len - 1, 1, xk + ldx, ldx, Bxk, ldb, c.dC.p, len - 1, c.gscr.p,
                      c.gscr.n, st);
                const double amax = absmax_dev(len - 1, 1, c.dC.p, len - 1);
                dlincomb(c, nrows, 1, len - 1, xk, ldx, c.dC.p, 1, xk + ldx, ldx, c.one.p, 0, st,
                         -1.0);
                if (amax < kReorthTol) break;
            }
            GCGE_CUDA(cudaStreamSynchronize(st));  // the host buffer is reused next column
        }
        return hi;
    }
    // OrthSelfEVP: X <- X V diag(w^-1/2) from G = X^T B X = V diag(w) V^T
    // (ascending), eigenvalues of magnitude at most the zero tolerance dropped
    int self_evp(double *x, int ldx, int lo, int hi) {
        for (int pass = 0; pass < 1 + max_reorth; ++pass) {
            const int k = hi - lo;
            if (k <= 0) return hi;
            double *X = x + (size_t)lo * ldx;
            const double *BX = X;
            int ldb = ldx;
            if (useB) {
                applyB(X, ldx, c.T2.p, c.ld, k);
                BX = c.T2.p;
                ldb = c.ld;
            }
            dgram(c, nrows, k, k, X, ldx, BX, ldb, c.dC.p, k, c.gscr.p, c.gscr.n, st);
            GCGE_CUDA(cudaMemcpyAsync(c.hbuf.p, c.dC.p, sizeof(double) * k * k,
                                      cudaMemcpyDeviceToHost, st));
            GCGE_CUDA(cudaStreamSynchronize(st));
            for (int i = 0; i < k * k; ++i)
                GCGE_REQUIRE(std::isfinite(c.hbuf.p[i]), GCGE_ERR_NUMERIC,
                             "orth: non-finite Gram matrix");
            std::vector<double> w(k), V((size_t)k * k);
            host_eigh(k, c.hbuf.p, w.data(), V.data());
            int lin_dep = 0;
            double wsum = 0.0;
            for (int j = 0; j < k; ++j) {
                if (std::fabs(w[j]) > zero_tol)
                    w[j] = 1.0 / std::sqrt(w[j]);
                else
                    ++lin_dep;
                wsum += std::fabs(w[j]);
            }
            const int kk = k - lin_dep;  // ascending: the dropped ones come first
            double *Cf = c.hbuf.p + (size_t)k * k;
            for (int j = 0; j < kk; ++j)
                for (int i = 0; i < k; ++i)
                    Cf[i + (size_t)j * k] = V[i + (size_t)(lin_dep + j) * k] * w[lin_dep + j];
            if (kk > 0) {
                GCGE_CUDA(cudaMemcpyAsync(c.dC.p, Cf, sizeof(double) * k * kk,
                                          cudaMemcpyHostToDevice, st));
                dlincomb(c, nrows, k, kk, X, ldx, c.dC.p, k, c.T1.p, c.ld, nullptr, 0, st);
                copy_cols(nrows, kk, c.T1.p, c.ld, X, ldx, st);
            }
            GCGE_CUDA(cudaStreamSynchronize(st));  // the host buffer is reused next pass
            hi = lo + kk;
            if (lin_dep == 0 && std::fabs(wsum - k) < kReorthTol) break;
        }
        return hi;
    }
    // OrthBinary (:416-518)
    int binary(double *x, int ldx, int lo, int hi) {
        if (hi <= lo) return hi;
        const int ncols = hi - lo;
        if (ncols <= block_size) return evp ? self_evp(x, ldx, lo, hi) : self_mgs(x, ldx, lo, hi);
        const int mid = lo + ncols / 2;
        const int end0 = binary(x, ldx, lo, mid);
        cgs(x + (size_t)lo * ldx, end0 - lo, x + (size_t)mid * ldx, hi - mid, ldx);
        const int end1 = binary(x, ldx, mid, hi);
        const int gap = mid - end0;
        const int len = std::min(gap, end1 - mid);
        if (len > 0) {  // refill the gap with the last columns of the second half
            copy_cols(nrows, len, x + (size_t)(end1 - len) * ldx, ldx, c.T1.p, c.ld, st);
            copy_cols(nrows, len, c.T1.p, c.ld, x + (size_t)end0 * ldx, ldx, st);
        }
        return end1 - gap;
    }
    int run(double *x, int ldx, int start, int end) {
        if (end <= start) return end;
        // against the prefix (:540-561): coefficients checked every pass
        if (start > 0) {
            const int k = end - start;
            double *X1 = x + (size_t)start * ldx;
            TcExpCache qcache, xcache;  // the prefix stays unchanged over the passes
            for (int pass = 0; pass < 1 + max_reorth; ++pass) {
                const double *BX1 = X1;
                int ldb = ldx;
                if (useB) {
                    applyB(X1, ldx, c.T2.p, c.ld, k);
                    BX1 = c.T2.p;
                    ldb = c.ld;
                }
                dgram(c, nrows, start, k, x, ldx, BX1, ldb, c.dC.p, start, c.gscr.p, c.gscr.n, st,
                      &qcache);
                dlincomb(c, nrows, start, k, x, ldx, c.dC.p, start, X1, ldx, c.one.p, 0, st, -1.0,
                         &xcache);
                if (absmax_dev(start, k, c.dC.p, start) < kReorthTol) break;
            }
        }
        // leaf method and size (:575-591): under 16 columns OrthSelf with leaves of
        // 4 (or the given size), else OrthSelfEVP with leaves of at most a quarter
        const int k = end - start;
        if (k < 16) {
            if (block_size <= 0) block_size = 4;
            evp = false;
        } else {
            if (block_size <= 0 || block_size > k / 4) block_size = k / 4;
            evp = true;
        }
        return binary(x, ldx, start, end);
    }
};

int bgs_orth(SolverCtx &c, SparseMat *B, double *x, int ldx, int nrows, int start, int end,
             bool useB, double zero_tol, int max_reorth, int block_size, int *spmm_calls) {
    BgsOrth o{c, B, nrows, useB, zero_tol, max_reorth, block_size, spmm_calls, lib_stream()};
    return o.run(x, ldx, start, end);
}

// ---------------------------------------------------------------- the solve
struct GcgRun {
    SolverCtx &c;
    GCGSolver &g;
    SparseMat *A, *B;
    MultiVec *V, *ritz;
    cudaStream_t st;
    int n, ld;
    PhaseTimer timer;
    // sizes (names of src/ops_eig_sol_gcg.c:44-47)
    int sizeN = 0, startN = 0, endN = 0, sizeP = 0, startP = 0, endP = 0;
    int sizeW = 0, startW = 0, endW = 0, sizeC = 0, sizeX = 0, sizeV = 0, endX = 0;
    std::vector<double> ss_eval;
    double *M = nullptr, *Mold = nullptr;  // projected matrix (current / previous)
    int s_old = 0;
    double sigma = 0.0;
    int pcg_iters = 0, spmm_calls = 0;
    // Ritz-vector columns [chk_lo, chk_lo + chk_n) whose A x and B x
    // CheckConvergence left in c.chkA / c.chkB (the vectors do not change
    // until the next Rayleigh-Ritz step)
    int chk_lo = 0, chk_n = 0;
    // the caller's handles, for a user-defined MultiLinearSolver
    OPS *ops = nullptr;
    void *Ah = nullptr, **Vh = nullptr, **Rh = nullptr;

    GcgRun(SolverCtx &c_, SparseMat *A_, SparseMat *B_, MultiVec *V_, MultiVec *r_)
        : c(c_), g(c_.pub), A(A_), B(B_), V(V_), ritz(r_), st(lib_stream()), n(A_->n),
          ld(V_->ld), timer(lib_stream()) {}

    // ---------------- helpers
    void applyB(const double *X, int ldx, double *Y, int ldy, int k) {
        if (k <= 0) return;
        if (B) {
            spmm<double>(B->pat, B->val.p, X, ldx, Y, ldy, k, st);
            spmm_calls++;
        } else {
            copy_cols(n, k, X, ldx, Y, ldy, st);
        }
    }
    double device_absmax(int m, int w, const double *C, int ldc) {
        absmax(m, w, C, ldc, c.dmax.p, st);
        GCGE_CUDA(cudaMemcpyAsync(c.hmax.p, c.dmax.p, sizeof(double), cudaMemcpyDeviceToHost, st));
        GCGE_CUDA(cudaStreamSynchronize(st));
        return c.hmax.p[0];
    }

    // MultiVecOrth with the method the parameters select ("bgs": binary
    // Gram-Schmidt; anything else: the GPU counterpart of modified
    // Gram-Schmidt, src/ops_eig_sol_gcg.c:119-141, :396-419, :650-668)
    int orth(double *x, int ldx, int nrows, int start, int end, bool useB, double zero_tol,
             int max_reorth, const char *method, int block_size) {
        if (method && std::strcmp(method, "bgs") == 0)
            return bgs_orth(c, useB ? B : nullptr, x, ldx, nrows, start, end, useB, zero_tol,
                            max_reorth, block_size, &spmm_calls);
        return borth(c, useB ? B : nullptr, x, ldx, nrows, start, end, useB, zero_tol, max_reorth,
                     &spmm_calls);
    }

    // ---------------- InitializeX (:102-159)
    void initialize_x(int nevGiven) {
        timer.mark(PH_INITX);
        copy_cols(n, nevGiven, colp(ritz, 0), ritz->ld, colp(V, 0), ld, st);
        nevGiven = orth(colp(V, 0), ld, n, 0, nevGiven, B != nullptr, g.initX_orth_zero_tol,
                        g.initX_orth_max_reorth, g.initX_orth_method, g.initX_orth_block_size);
        int filled = nevGiven;
        for (int attempt = 0; attempt < 4 && filled < sizeX; ++attempt) {
            fill_uniform(n, sizeX - filled, colp(V, filled), ld, 0x5eed + attempt * 7919 + filled, st);
            filled = orth(colp(V, 0), ld, n, filled, sizeX, B != nullptr, g.initX_orth_zero_tol,
                          g.initX_orth_max_reorth, g.initX_orth_method, g.initX_orth_block_size);
        }
        GCGE_REQUIRE(filled == sizeX, GCGE_ERR_NUMERIC, "InitializeX: could not fill the basis");
        endX = sizeX;
    }

    // ---------------- ComputeRitzVec (:160-195)
    void compute_ritz_vec() {
        timer.mark(PH_RV);
        const int s = sizeV - sizeC;
        dlincomb(c, n, s, endX - startN, colp(V, startN), ld, c.evec.p, s, colp(ritz, startN),
                 ritz->ld, nullptr, 0, st);
    }

    // ---------------- CheckConvergence (:196-321)
    int check_convergence(int numCheck, std::vector<int> &offset) {
        timer.mark(PH_CHECK);
        const double *tol = g.tol;
        GCGE_REQUIRE(c.has_union, GCGE_ERR_ARG, "operator not prepared");
        std::vector<double> res(numCheck);
        c.chkA.alloc((size_t)ld * numCheck);
        c.chkB.alloc((size_t)ld * numCheck);
        chk_lo = startN;
        chk_n = numCheck;
        for (int c0 = 0; c0 < numCheck; c0 += 40) {
            const int kc = std::min(40, numCheck - c0);
            GCGE_CUDA(cudaMemcpyAsync(c.dvec.p, &ss_eval[startN + c0], sizeof(double) * kc,
                                      cudaMemcpyHostToDevice, st));
            const int nb = residual_norms(A->pat, A->val.p, B ? &B->pat : nullptr,
                                          B ? B->val.p : nullptr, colp(ritz, startN + c0),
                                          ritz->ld, c.dvec.p, kc, c.part.p, 64, st,
                                          c.chkA.p + (size_t)c0 * ld, c.chkB.p + (size_t)c0 * ld, ld);
            spmm_calls++;
            reduce_partials(c.part.p, nb, 64, kc, c.dvec.p + 64, st);
            GCGE_CUDA(cudaMemcpyAsync(c.hbuf.p + c0, c.dvec.p + 64, sizeof(double) * kc,
                                      cudaMemcpyDeviceToHost, st));
            GCGE_CUDA(cudaStreamSynchronize(st));
        }
        for (int i = 0; i < numCheck; ++i) {
            GCGE_REQUIRE(std::isfinite(c.hbuf.p[i]), GCGE_ERR_NUMERIC, "CheckConvergence: NaN residual");
            res[i] = std::sqrt(std::max(c.hbuf.p[i], 0.0));
        }
        last_res = res;
        int idx;
        for (idx = 0; idx < numCheck; ++idx) {
            const double lam = ss_eval[startN + idx];
            if (res[idx] > tol[0] || res[idx] > std::fabs(lam) * tol[1]) {
                if (g.print)
                    printf("%3d EPS nconv=%d first unconverged value (error(abs,rel)) %6.5e (%6.5e, %6.5e)\n",
                           iter_print + 1, startN, lam, res[idx], res[idx] / std::fabs(lam));
                break;
            }
        }
        const double first_abs = idx < numCheck ? res[idx] : 0.0;
        const double first_rel =
            idx < numCheck ? res[idx] / std::max(std::fabs(ss_eval[startN + idx]), 1e-300) : 0.0;
        for (; idx > 0; --idx) {
            if (std::fabs((ss_eval[startN + idx - 1] - ss_eval[startN + idx]) / ss_eval[startN + idx - 1]) >
                g.gapMin)
                break;
        }
        const int nevConv = sizeC + idx;
        watch_progress(nevConv, first_abs, first_rel);
        offset[0] = 0;
        int state = 1, num_unconv = 0;
        for (idx = 0; idx < numCheck; ++idx) {
            const double lam = ss_eval[startN + idx];
            if (res[idx] > tol[0] || res[idx] > std::fabs(lam) * tol[1]) {
                if (state) {
                    offset[offset[0] * 2 + 1] = startN + idx;
                    state = 0;
                }
                ++num_unconv;
                if (num_unconv == sizeN) {
                    offset[offset[0] * 2 + 2] = startN + idx + 1;
                    ++offset[0];
                    break;
                }
            } else if (!state) {
                offset[offset[0] * 2 + 2] = startN + idx;
                ++offset[0];
                state = 1;
            }
        }
        if (num_unconv < sizeN) {
            if (state == 1) offset[offset[0] * 2 + 1] = startN + numCheck;
            const int e = startN + numCheck + sizeN - num_unconv;
            offset[offset[0] * 2 + 2] = e < endX ? e : endX;
            GCGE_REQUIRE(offset[offset[0] * 2 + 1] < offset[offset[0] * 2 + 2], GCGE_ERR_NUMERIC,
                         "CheckConvergence: empty unconverged range");
            ++offset[0];
        }
        GCGE_REQUIRE(offset[0] > 0, GCGE_ERR_NUMERIC, "CheckConvergence: no offsets");
        return nevConv;
    }
    std::vector<double> last_res;
    int iter_print = 0;
    bool restart_pending = false;

    // At the switch to FP64: the digit-plane products and the FP32 inner solve
    // leave the basis B-orthonormal only to ~1e-11..1e-10, and the Ritz pairs
    // of such a basis cannot reach a relative residual below that error times
    // the spread of the spectrum (1e-8 on anisotropic problems: pairs stall at
    // 1.5e-8 in FP64 too, since the X block is carried from iteration to
    // iteration and never re-orthonormalised).  The unlocked Ritz vectors are
    // therefore B-orthonormalised against the locked ones and among themselves
    // in FP64, re-diagonalised by a Rayleigh-Ritz step on their span, and the
    // next iteration builds no P (the P coefficients refer to the old basis).
    bool restart_active() {
        const int k = sizeX - sizeC;
        if (k <= 0) return false;
        chk_n = 0;  // the Ritz vectors change: CheckConvergence's products no longer apply
        double *Xa = colp(ritz, sizeC);
        const int e = borth(c, B, ritz->data, ritz->ld, n, sizeC, sizeX, B != nullptr,
                            g.compW_orth_zero_tol, g.compW_orth_max_reorth, &spmm_calls);
        GCGE_REQUIRE(e == sizeX, GCGE_ERR_NUMERIC, "restart: Ritz vectors became dependent");
        spmm<double>(A->pat, A->val.p, Xa, ritz->ld, c.T1.p, ld, k, st);
        spmm_calls++;
        gram(n, k, k, Xa, ritz->ld, c.T1.p, ld, c.dtmp.p, k, c.gscr.p, c.gscr.n, st);
        std::vector<double> w(k);
        sym_eig(c.eig, k, c.dtmp.p, k, w.data(), c.evec.p, k, c.refine_steps, st);
        lincomb(n, k, k, Xa, ritz->ld, c.evec.p, k, c.T1.p, ld, nullptr, 0, st);
        copy_cols(n, k, c.T1.p, ld, Xa, ritz->ld, st);
        for (int i = 0; i < k; ++i) ss_eval[sizeC + i] = w[i];
        GCGE_CUDA(cudaStreamSynchronize(st));
        return true;
    }

    // Precision escalation of the mixed solve.  The FP32 inner solve sees the
    // shifted operator with entry errors of about eps32 |S|, which the
    // near-singular shift (0.01 of a gap from the target eigenvalue) amplifies,
    // and the digit products are exact only to 2^-55 of each chunk's largest
    // entries; for tolerances tight against |A| (small eigenvalues, tol ~1e-10)
    // the residuals then stop falling just above the tolerance.  When the
    // first unconverged residual is within 100x of the tolerance and shrinks
    // by less than 2x over 10 outer iterations with no newly converged pair,
    // the rest of the solve runs in FP64 (inner solve and dense products: the
    // reference's arithmetic).
    int escalated_at = 0;
    std::vector<std::pair<int, double>> progress;
    void watch_progress(int nevConv, double first_abs, double first_rel) {
        if (c.precision != GCGE_PREC_MIXED || c.escalated) return;
        progress.push_back({nevConv, first_rel});
        constexpr size_t K = 10;
        if (progress.size() <= K) return;
        const bool near_tol = first_rel <= 100.0 * g.tol[1] && first_abs <= 100.0 * g.tol[0];
        const auto &old = progress[progress.size() - 1 - K];
        const auto &cur = progress.back();
        if (near_tol && cur.first <= old.first && cur.second > 0.5 * old.second) {
            c.escalated = true;
            escalated_at = iter_print + 1;
            restart_pending = true;
            if (g.print)
                printf("%3d mixed precision: residual %6.5e stalled near the tolerance, FP64 from here\n",
                       escalated_at, cur.second);
        }
    }

    // ---------------- ComputeP (:322-463)
    void compute_p(const std::vector<int> &offset) {
        timer.mark(PH_P);
        const int s = sizeV - sizeC;
        const int base = sizeX - sizeC;
        std::vector<int> cols;
        std::vector<int> mask(s, 0);
        for (int i = 0; i < offset[0]; ++i)
            for (int o = offset[2 * i + 1]; o < offset[2 * i + 2]; ++o) {
                cols.push_back(o - sizeC);
                mask[o - sizeC] = 1;
            }
        int np = (int)cols.size();
        // work = [evec(:, 0:base) | evec(:, cols) with the unconverged X rows zeroed]
        double *wk = c.work.p;
        copy_cols(s, base, c.evec.p, s, wk, s, st);
        // c.hup is next written in the next iteration, after several stream
        // synchronisations: the copies need no wait here
        int *hidx = reinterpret_cast<int *>(c.hup.p);
        for (int a = 0; a < np; ++a) hidx[a] = cols[a];
        for (int a = 0; a < s; ++a) hidx[np + a] = mask[a];
        GCGE_CUDA(cudaMemcpyAsync(c.didx.p, hidx, sizeof(int) * np, cudaMemcpyHostToDevice, st));
        GCGE_CUDA(cudaMemcpyAsync(c.dmask.p, hidx + np, sizeof(int) * s, cudaMemcpyHostToDevice, st));
        gather_columns(s, np, c.evec.p, s, c.didx.p, wk + (size_t)base * s, s, st);
        zero_rows(s, np, wk + (size_t)base * s, s, c.dmask.p, st);
        // small-space orthonormalisation against the X coefficients (B = I)
        const int endP_local = orth(wk, s, s, base, base + np, false, g.compP_orth_zero_tol,
                                    g.compP_orth_max_reorth, g.compP_orth_method,
                                    g.compP_orth_block_size);
        np = endP_local - base;
        startP = base + sizeC;
        endP = endP_local + sizeC;
        sizeP = endP - startP;
        copy_cols(s, sizeP, wk + (size_t)base * s, s, c.coefP.p, s, st);
        // P = V(:, startN:endW) coefP, staged through T1 (it overlaps V's range)
        dlincomb(c, n, s, sizeP, colp(V, startN), ld, c.coefP.p, s, c.T1.p, ld, nullptr, 0, st);
        copy_cols(n, sizeP, c.T1.p, ld, colp(V, startP), ld, st);
    }

    // ---------------- ComputeX (:464-477)
    void compute_x() {
        timer.mark(PH_X);
        copy_cols(n, endX - startN, colp(ritz, startN), ritz->ld, colp(V, startN), ld, st);
    }

    // ---------------- ComputeW (:478-701)
    void compute_w(const std::vector<int> &offset) {
        timer.mark(PH_W);
        double sg = 0.0;
        if (g.compW_cg_auto_shift == 1)
            sg = -ss_eval[sizeC] + (ss_eval[sizeC + 1] - ss_eval[sizeC]) * 0.01;
        g.sigma = g.compW_cg_shift + sg;
        sigma = g.sigma;
        startW = endP;
        int bsz = 0;
        double *hscale = c.hbuf.p;
        // B x of each column: CheckConvergence's product where it checked the
        // column, else a product here (the last run of unconverged columns may
        // extend past the checked ones, :285-300); `fresh` lists the latter
        // (W position, Ritz column, count) for S x0 below
        std::vector<std::array<int, 3>> fresh;
        const int chk_hi = chk_lo + chk_n;
        for (int i = 0; i < offset[0]; ++i) {
            const int o1 = offset[2 * i + 1], o2 = offset[2 * i + 2], len = o2 - o1;
            copy_cols(n, len, colp(ritz, o1), ritz->ld, colp(V, startW + bsz), ld, st);
            const int cov = (c.chkB.p != nullptr && o1 >= chk_lo && o1 < chk_hi)
                                ? std::min(o2, chk_hi) - o1
                                : 0;
            if (cov > 0)
                copy_cols(n, cov, c.chkB.p + (size_t)(o1 - chk_lo) * ld, ld,
                          c.bbuf.p + (size_t)bsz * ld, ld, st);
            if (len > cov) {
                applyB(colp(V, o1 + cov), ld, c.bbuf.p + (size_t)(bsz + cov) * ld, ld, len - cov);
                fresh.push_back({bsz + cov, o1 + cov, len - cov});
            }
            for (int j = 0; j < len; ++j) hscale[bsz + j] = ss_eval[o1 + j] + sigma;
            bsz += len;
        }
        endW = startW + bsz;
        const bool mixed = c.precision == GCGE_PREC_MIXED && !c.escalated;
        const int ud = g.user_defined_multi_linear_solver;
        // S x0 = A x0 + sigma B x0 for the mixed inner solve, from the stored
        // products and, for the other columns, A x0 here and the B x0 above
        // (before bbuf is scaled)
        const bool have_sx = mixed && ud == 0;
        if (have_sx) {
            int off = 0;
            for (int i = 0; i < offset[0]; ++i) {
                const int o1 = offset[2 * i + 1], o2 = offset[2 * i + 2], len = o2 - o1;
                const int cov = (c.chkB.p != nullptr && o1 >= chk_lo && o1 < chk_hi)
                                    ? std::min(o2, chk_hi) - o1
                                    : 0;
                if (cov > 0) {
                    copy_cols(n, cov, c.chkA.p + (size_t)(o1 - chk_lo) * ld, ld,
                              c.r64.p + (size_t)off * ld, ld, st);
                    axpby(n, cov, sigma, c.chkB.p + (size_t)(o1 - chk_lo) * ld, ld, 1.0,
                          c.r64.p + (size_t)off * ld, ld, st);
                }
                off += len;
            }
            for (const auto &f : fresh) {
                spmm<double>(A->pat, A->val.p, colp(V, f[1]), ld, c.r64.p + (size_t)f[0] * ld, ld,
                             f[2], st);
                spmm_calls++;
                axpby(n, f[2], sigma, c.bbuf.p + (size_t)f[0] * ld, ld, 1.0,
                      c.r64.p + (size_t)f[0] * ld, ld, st);
            }
        }
        GCGE_CUDA(cudaMemcpyAsync(c.dvec.p, hscale, sizeof(double) * bsz, cudaMemcpyHostToDevice, st));
        scale_columns(n, bsz, c.bbuf.p, ld, c.dvec.p, st);
        // shifted operator S = A + sigma B on the union pattern
        shift_values(c.upat.padded, c.ua.p, c.ub.p, sigma, c.us64.p, mixed ? c.us32.p : nullptr,
                     st);
        timer.mark(PH_LINSOL);
        if (ud == 1 || ud == 2) {
            // the caller's solver (:590-592) on b = (lambda + sigma) B x, which
            // the reference keeps in the Ritz-vector columns [offset[1], +bsz)
            // (:484, :527), solving into V[:, startW:endW]
            GCGE_REQUIRE(ops && ops->MultiLinearSolver, GCGE_ERR_ARG,
                         "ComputeW: user_defined_multi_linear_solver without MultiLinearSolver");
            GCGE_REQUIRE(g.compW_cg_auto_shift == 0, GCGE_ERR_ARG,  // (:503)
                         "ComputeW: a user-defined solver excludes the automatic shift");
            copy_cols(n, bsz, c.bbuf.p, ld, colp(ritz, offset[1]), ritz->ld, st);
            GCGE_CUDA(cudaStreamSynchronize(st));
            int s2[2] = {offset[1], startW}, e2[2] = {offset[1] + bsz, endW};
            ops->MultiLinearSolver(Ah, Rh, Vh, s2, e2, ops);
            const int err = take_error();
            if (err != GCGE_OK) throw CudaError{err, "ComputeW: user-defined MultiLinearSolver"};
            // BlockPCG after it (ud == 2) starts from its x with its b
            copy_cols(n, bsz, colp(ritz, offset[1]), ritz->ld, c.bbuf.p, ld, st);
        }
        if (ud != 1) w_solve(colp(V, startW), bsz, mixed, have_sx);
        timer.mark(PH_W);
        endW = orth(colp(V, 0), ld, n, startW, endW, B != nullptr, g.compW_orth_zero_tol,
                    g.compW_orth_max_reorth, g.compW_orth_method, g.compW_orth_block_size);
        sizeW = endW - startW;
    }

    // BlockPCG on S x = b (b in c.bbuf, S = A + sigma B on the union pattern,
    // its values already formed) for bsz columns, starting from and overwriting
    // x (V columns, leading dimension ld).
    void w_solve(double *x, int bsz, bool mixed, bool have_sx = false) {
        if (bsz <= 0) return;
        const bool rel = std::strcmp(g.compW_cg_tol_type, "rel") == 0;
        if (!mixed) {
            const int kp = rows_width(bsz, 8);
            col_to_rows<double, double>(n, bsz, kp, x, ld, c.xr64.p, st);
            col_to_rows<double, double>(n, bsz, kp, c.bbuf.p, ld, c.br64.p, st);
            block_pcg_rows<double>(c.pcg, c.upat, c.us64.p, c.br64.p, c.xr64.p, c.rr64.p,
                                   c.pr64.p, c.wr64.p, kp, bsz, g.compW_cg_max_iter,
                                   g.compW_cg_rate, g.compW_cg_tol, rel, false, st);
            rows_to_col<double, double>(n, bsz, kp, c.xr64.p, x, ld, false, st);
            spmm_calls++;  // the residual b - S x0 inside the solve
        } else {
            // CG from x0 on S x = b is CG from 0 on S d = b - S x0: the residual
            // is formed in FP64 (it is a difference of nearly equal vectors once
            // the Ritz vectors converge), the correction d is iterated in FP32,
            // and x = x0 + d is accumulated in FP64.
            const int kp = rows_width(bsz, 4);
            if (!have_sx) {  // else r64 already holds S x
                spmm<double>(c.upat, c.us64.p, x, ld, c.r64.p, ld, bsz, st);
                spmm_calls++;
            }
            axpby(n, bsz, 1.0, c.bbuf.p, ld, -1.0, c.r64.p, ld, st);
            col_to_rows<double, float>(n, bsz, kp, c.r64.p, ld, c.br32.p, st);
            block_pcg_rows<float>(c.pcg, c.upat, c.us32.p, c.br32.p, c.xr32.p, c.rr32.p,
                                  c.pr32.p, c.wr32.p, kp, bsz, g.compW_cg_max_iter,
                                  g.compW_cg_rate, g.compW_cg_tol, rel, true, st);
            rows_to_col<float, double>(n, bsz, kp, c.xr32.p, x, ld, true, st);
        }
    }

    // The A x and B x of Ritz-vector columns [o1, o2) are in c.chkA / c.chkB.
    bool have_products(int o1, int o2) const {
        return o1 >= chk_lo && o2 <= chk_lo + chk_n && c.chkB.p != nullptr;
    }

    // ---------------- ComputeW12 (:703-929), compW_cg_order 2: the first half
    // of the unconverged columns gets two W directions, the BlockPCG solution
    // x1 of S x = b from the Ritz vectors and x2, the same solve restarted from
    // x1 (the right-hand side is the same for both; the reference rebuilds it
    // only because its shifted product used it as scratch).
    void compute_w12(const std::vector<int> &offset) {
        GCGE_REQUIRE(g.user_defined_multi_linear_solver == 0, GCGE_ERR_ARG,  // (:709)
                     "ComputeW12 runs BlockPCG only (user_defined_multi_linear_solver must be 0)");
        timer.mark(PH_W);
        double sg = 0.0;
        if (g.compW_cg_auto_shift == 1)
            sg = -ss_eval[sizeC] + (ss_eval[sizeC + 1] - ss_eval[sizeC]) * 0.01;
        g.sigma = g.compW_cg_shift + sg;
        sigma = g.sigma;
        startW = endP;
        int total = 0;
        for (int i = 0; i < offset[0]; ++i) total += offset[2 * i + 2] - offset[2 * i + 1];
        const int half = total / 2;
        int bsz = 0;
        double *hscale = c.hbuf.p;
        for (int i = 0; i < offset[0]; ++i) {
            const int o1 = offset[2 * i + 1];
            int len = offset[2 * i + 2] - o1;
            if (bsz + len >= half) len = half - bsz;
            copy_cols(n, len, colp(ritz, o1), ritz->ld, colp(V, startW + bsz), ld, st);
            if (have_products(o1, o1 + len))
                copy_cols(n, len, c.chkB.p + (size_t)(o1 - chk_lo) * ld, ld,
                          c.bbuf.p + (size_t)bsz * ld, ld, st);
            else
                applyB(colp(V, o1), ld, c.bbuf.p + (size_t)bsz * ld, ld, len);
            for (int j = 0; j < len; ++j) hscale[bsz + j] = ss_eval[o1 + j] + sigma;
            bsz += len;
            if (bsz >= half) break;
        }
        if (bsz > 0) {
            GCGE_CUDA(cudaMemcpyAsync(c.dvec.p, hscale, sizeof(double) * bsz,
                                      cudaMemcpyHostToDevice, st));
            scale_columns(n, bsz, c.bbuf.p, ld, c.dvec.p, st);
        }
        const bool mixed = c.precision == GCGE_PREC_MIXED && !c.escalated;
        shift_values(c.upat.padded, c.ua.p, c.ub.p, sigma, c.us64.p, mixed ? c.us32.p : nullptr,
                     st);
        timer.mark(PH_LINSOL);
        w_solve(colp(V, startW), bsz, mixed);
        endW = startW + bsz;
        copy_cols(n, bsz, colp(V, startW), ld, colp(V, endW), ld, st);
        w_solve(colp(V, endW), bsz, mixed);
        endW += bsz;
        timer.mark(PH_W);
        endW = orth(colp(V, 0), ld, n, startW, endW, B != nullptr, g.compW_orth_zero_tol,
                    g.compW_orth_max_reorth, g.compW_orth_method, g.compW_orth_block_size);
        sizeW = endW - startW;
    }

    // ---------------- ComputeRayleighRitz (:931-1258)
    void compute_rr(int nevConv) {
        timer.mark(PH_RR);
        const int s_prev = sizeV - sizeC;
        if (sizeP > 0) {
            // PtAP = coefP^T Mold coefP in the previous projected space (:942-955)
            dlincomb(c, s_prev, s_prev, sizeP, M, s_prev, c.coefP.p, s_prev, c.dtmp.p, s_prev,
                     nullptr, 0, st);
            dgram(c, s_prev, sizeP, sizeP, c.coefP.p, s_prev, c.dtmp.p, s_prev, c.ptap.p, sizeP,
                  c.gscr.p, c.gscr.n, st);
        }
        sizeV = sizeX + sizeP + sizeW;
        startN += nevConv - sizeC;
        endN += nevConv - sizeC;
        endN = std::min(endN, endX);
        sizeN = endN - startN;
        sizeC = nevConv;
        const int s = sizeV - sizeC;
        std::swap(M, Mold);
        const int xp = sizeX + sizeP - sizeC;
        timer.mark(PH_RRW);
        if (sizeW > 0) {
            // [X P W]^T A W (:976-993)
            spmm<double>(A->pat, A->val.p, colp(V, startW), ld, c.T1.p, ld, sizeW, st);
            spmm_calls++;
            dgram(c, n, endW - startN, sizeW, colp(V, startN), ld, c.T1.p, ld, M + (size_t)xp * s,
                  s, c.gscr.p, c.gscr.n, st);
            transpose_copy(xp, sizeW, M + (size_t)xp * s, s, M + xp, s, st);
        }
        if (sizeX == sizeV) {
            // first pass: the whole X^T A X in column blocks (:998-1017)
            const int bsz = std::max(1, std::min(g.block_size, sizeX - sizeC));
            for (int c0 = sizeC; c0 < sizeX; c0 += bsz) {
                const int kc = std::min(bsz, sizeX - c0);
                spmm<double>(A->pat, A->val.p, colp(V, c0), ld, c.T1.p, ld, kc, st);
                spmm_calls++;
                dgram(c, n, sizeX - sizeC, kc, colp(V, sizeC), ld, c.T1.p, ld,
                      M + (size_t)(c0 - sizeC) * s, s, c.gscr.p, c.gscr.n, st);
            }
        } else {
            // X block = diag(Ritz values), XP block = 0, P block = PtAP (:1018-1039)
            for (int j = 0; j < xp; ++j)
                GCGE_CUDA(cudaMemsetAsync(M + (size_t)j * s, 0, sizeof(double) * xp, st));
            const int nx = sizeX - sizeC;
            // second half of c.hup (ComputeP uses the first): rewritten next
            // iteration, after the stream has passed this copy
            double *hd = c.hup.p + 2 * (size_t)c.cap_s;
            for (int i = 0; i < nx; ++i) hd[i] = ss_eval[sizeC + i];
            GCGE_CUDA(cudaMemcpyAsync(c.dvec.p, hd, sizeof(double) * nx, cudaMemcpyHostToDevice, st));
            GCGE_CUDA(cudaMemcpy2DAsync(M, sizeof(double) * (s + 1), c.dvec.p, sizeof(double),
                                        sizeof(double), nx, cudaMemcpyDeviceToDevice, st));
            if (sizeP > 0)
                copy_cols(sizeP, sizeP, c.ptap.p, sizeP, M + nx + (size_t)nx * s, s, st);
        }
        timer.mark(PH_EIG);
        std::vector<double> w(s);
        sym_eig(c.eig, s, M, s, w.data(), c.evec.p, s, c.refine_steps, st,
                c.precision == GCGE_PREC_MIXED && !c.escalated);
        for (int i = 0; i < s; ++i) ss_eval[sizeC + i] = w[i] - 0.0;
        timer.mark(PH_RR);
    }

    // Mixed solve: the returned eigenvalues are the FP64 Rayleigh quotients
    // x^T A x / x^T B x of the returned vectors.  The Ritz values of the last
    // projection carry the basis' B-orthonormality error, which the digit-plane
    // products and the FP32 inner solve leave larger than the FP64 solve does
    // (up to ~1e-9 with ComputeW12); the quotients of vectors whose relative
    // residual is below the tolerance are accurate to its square.  The vectors
    // are returned as the iteration left them: a last Rayleigh-Ritz or Lowdin
    // step would restore B-orthonormality but mixes vectors of a cluster,
    // which can lift a residual just above the tolerance.
    void rayleigh_quotients(double *eval, int k) {
        if (k <= 0) return;
        spmm<double>(A->pat, A->val.p, ritz->data, ritz->ld, c.T1.p, ld, k, st);
        spmm_calls++;
        applyB(ritz->data, ritz->ld, c.T2.p, ld, k);
        coldot(n, k, ritz->data, ritz->ld, c.T1.p, ld, c.dvec.p, c.gscr.p, c.gscr.n, st);
        coldot(n, k, ritz->data, ritz->ld, c.T2.p, ld, c.dvec.p + k, c.gscr.p, c.gscr.n, st);
        GCGE_CUDA(cudaMemcpyAsync(c.hbuf.p, c.dvec.p, sizeof(double) * 2 * k,
                                  cudaMemcpyDeviceToHost, st));
        GCGE_CUDA(cudaStreamSynchronize(st));
        for (int j = 0; j < k; ++j) {
            const double num = c.hbuf.p[j], den = c.hbuf.p[k + j];
            if (den > 0.0 && std::isfinite(num / den)) eval[j] = num / den;
        }
    }

    // ---------------- GCG outer loop (:1259-1562)
    int run(double *eval, int nevGiven, int *nevConvIO) {
        const int nevInit = g.nevInit, nevMax = g.nevMax, bs = g.block_size;
        GCGE_REQUIRE(nevInit >= nevGiven, GCGE_ERR_ARG, "nevInit < nevGiven");
        GCGE_REQUIRE(nevInit <= nevMax, GCGE_ERR_ARG, "nevInit > nevMax");
        GCGE_REQUIRE(nevInit >= 3 * bs || nevInit == nevMax, GCGE_ERR_ARG,
                     "nevInit must be >= 3*block_size or == nevMax");
        GCGE_REQUIRE(nevMax >= *nevConvIO + bs || nevMax >= bs, GCGE_ERR_ARG, "nevMax too small");
        GCGE_REQUIRE(V->ncols >= nevMax + 2 * bs && ritz->ncols >= nevMax, GCGE_ERR_ARG,
                     "workspace multivectors too small");
        GCGE_REQUIRE(bs <= 40 && bs >= 1, GCGE_ERR_ARG, "block_size out of range (1..40)");
        GCGE_REQUIRE(nevMax + 2 * bs <= n, GCGE_ERR_ARG, "nevMax + 2*block_size exceeds n");
        GCGE_REQUIRE(nevGiven >= 0, GCGE_ERR_ARG, "nevGiven < 0");
        int numIterMax = g.numIterMax;
        sizeC = 0;
        sizeN = bs;
        sizeX = nevInit;
        sizeP = 0;
        sizeW = 0;
        sizeV = sizeX;
        startN = 0;
        endN = startN + sizeN;
        endX = sizeX;
        startP = endX;
        endP = startP;
        startW = endP;
        endW = startW;
        ss_eval.assign(nevMax + 2 * bs, 1.0);
        M = c.M0.p;
        Mold = c.M1.p;
        std::vector<int> offsetP(bs + 3, 0), offsetW(bs + 3, 0);
        initialize_x(nevGiven);
        compute_rr(0);
        for (int i = sizeV; i < nevMax + 2 * bs; ++i) ss_eval[i] = ss_eval[sizeV - 1];
        compute_ritz_vec();
        int nev0 = std::min(*nevConvIO, nevMax);
        int nevc = 0;
        int nev = nevInit < nevMax ? 2 * bs : nev0;
        nev = std::min(nev, nev0);
        int numIter = 0;
        do {
            int numCheck = numIter <= 0 ? 0 : (startN + sizeN < endX ? sizeN : endX - startN);
            numCheck = std::min(numCheck, g.check_conv_max_num);
            if (numCheck == 0) numCheck = 1;
            nevc = check_convergence(numCheck, offsetW);
            if (nevc >= nev) {
                if (nevc >= nev0) break;
                nev = std::min(nev + sizeP + sizeW, nev0);
                const int newX = std::min(sizeX + sizeP + sizeW, nevMax);
                const int s = sizeV - sizeC;
                dlincomb(c, n, s, newX - endX, colp(V, startN), ld,
                         c.evec.p + (size_t)(endX - sizeC) * s, s, colp(ritz, endX), ritz->ld,
                         nullptr, 0, st);
                sizeX = newX;
                sizeP = 0;
                sizeW = 0;
                sizeV = sizeX;
                startP = endX;
                endP = startP;
                startW = endP;
                endW = startW;
                endX = sizeX;
                endN = std::min(startN + bs, endX);
                sizeN = endN - startN;
                numIterMax -= numIter;
                numIter = 0;
            }
            bool restarted = false;
            if (restart_pending) {
                restart_pending = false;
                restarted = restart_active();
            }
            if (numIter == 0 || restarted) {
                sizeP = 0;
                startP = endX;
                endP = startP;
            } else {
                compute_p(offsetP);
            }
            compute_x();
            if (g.compW_cg_order != 1)  // (:1456-1461)
                compute_w12(offsetW);
            else
                compute_w(offsetW);
            std::swap(offsetP, offsetW);
            compute_rr(nevc);
            for (int i = sizeV; i < nevMax + 2 * bs; ++i) ss_eval[i] = ss_eval[sizeV - 1];
            compute_ritz_vec();
            ++numIter;
            ++iter_print;
        } while (numIter < numIterMax);
        g.numIter = numIter + (g.numIterMax - numIterMax);
        for (int i = 0; i < sizeX; ++i) eval[i] = ss_eval[i];
        if (c.precision == GCGE_PREC_MIXED) rayleigh_quotients(eval, sizeX);
        *nevConvIO = nevc;
        g.nevConv = nevc;
        timer.mark(PH_NONE);
        GCGE_CUDA(cudaStreamSynchronize(st));
        return nevc >= nev0 ? GCGE_OK : GCGE_ERR_NOT_CONVERGED;
    }
};

// Union pattern of A, B and the diagonal with the values of A and of B laid
// out on it (B = NULL contributes the identity).
void prepare_union(SolverCtx &c, SparseMat *A, SparseMat *B, cudaStream_t st) {
    const unsigned long long ka = A->serial, kb = B ? B->serial : 0ULL;
    if (c.has_union && c.keyA == ka && c.keyB == kb) return;
    // union pattern of A, B (or the identity) and the diagonal, built on the device
    DevCsr U;
    DevBuf<double> ubv;
    union_csr_device(A->csr, B ? &B->csr : nullptr, U, ubv, st);
    sell_from_csr_device(U, ubv.p, c.upat, c.ua, &c.ub, st);
    const size_t P = std::max<size_t>(c.upat.padded, 1);
    c.us64.alloc(P);
    c.us32.alloc(P);
    GCGE_CUDA(cudaStreamSynchronize(st));  // U and ubv are freed on return
    c.keyA = ka;
    c.keyB = kb;
    c.has_union = true;
}

void gcg_eigensolver(void *Ah, void *Bh, double *eval, void **evec, int nevGiven, int *nevConv,
                     OPS *ops) {
    SolverCtx *c = ctx_for(ops, false);
    if (!c) {
        set_error(GCGE_ERR_ARG, "EigenSolver: EigenSolverSetup_GCG was not called on this ops");
        return;
    }
    const auto t0 = std::chrono::steady_clock::now();
    const unsigned long long l0 = t_kernel_launches;
    try {
        SparseMat *A = as_mat(Ah);
        SparseMat *B = Bh ? as_mat(Bh) : nullptr;
        GCGE_REQUIRE(A != nullptr, GCGE_ERR_HANDLE, "EigenSolver: A is not a CUDA matrix");
        GCGE_REQUIRE(Bh == nullptr || B != nullptr, GCGE_ERR_HANDLE,
                     "EigenSolver: B is not a CUDA matrix");
        MultiVec *V = as_mv(c->pub.mv_ws[0]);
        MultiVec *R = as_mv(evec);
        GCGE_REQUIRE(V && R && as_mv(c->pub.mv_ws[1]), GCGE_ERR_HANDLE,
                     "EigenSolver: workspaces are not CUDA multivectors");
        GCGE_REQUIRE(V->nrows == A->n && R->nrows == A->n, GCGE_ERR_ARG, "EigenSolver: size mismatch");
        GCGE_REQUIRE(!B || B->n == A->n, GCGE_ERR_ARG, "EigenSolver: B size mismatch");
        cudaStream_t st = lib_stream();
        prepare_union(*c, A, B, st);
        c->reserve(A->n, c->pub.nevMax, c->pub.nevInit, c->pub.block_size, spmm_blocks(c->upat));
        if (c->precision == GCGE_PREC_MIXED) {
            const size_t nb = pcg_block_elems(A->n, rows_width(std::min(c->pub.block_size, 40), 4));
            for (auto *b : {&c->xr32, &c->br32, &c->rr32, &c->pr32, &c->wr32}) b->alloc(nb);
        }
        c->pub.A = Ah;
        c->pub.B = Bh;
        c->pub.evec = evec;
        c->pub.eval = eval;
        c->pub.nevGiven = nevGiven;
        GCGE_REQUIRE(V->ld == R->ld, GCGE_ERR_ARG, "EigenSolver: leading dimensions differ");
        c->escalated = false;
        GcgRun run(*c, A, B, V, R);
        run.ops = ops;
        run.Ah = Ah;
        run.Vh = c->pub.mv_ws[0];
        run.Rh = evec;
        c->pcg.timing_reset(st);
        const int status = run.run(eval, nevGiven, nevConv);
        c->pcg.collect(st);
        if (c->precision == GCGE_PREC_MIXED && tc_digits_available()) tc_check_error(st);
        c->info.pcg_spmm_ms = c->pcg.spmm_ms;
        c->info.pcg_spmm_launches = (int)c->pcg.total_iters;
        c->info.pcg_spmm_bytes = c->pcg.spmm_bytes;
        c->info.pcg_kernel_launches = c->pcg.launches;
        c->info.pcg_kernel_ms = c->pcg.kernel_ms;
        c->info.pcg_kernel_bytes = c->pcg.kernel_bytes;
        c->info.precision_escalation_iter = run.escalated_at;
        run.pcg_iters = (int)c->pcg.total_iters;
        run.spmm_calls += (int)c->pcg.total_iters;
        c->info.nconv = *nevConv;
        c->info.niter = c->pub.numIter;
        c->info.status = status;
        c->info.pcg_iters = run.pcg_iters;
        c->info.spmm_calls = run.spmm_calls;
        run.timer.collect(c->info.phase_ms);
        c->last_status = status;
    } catch (const CudaError &e) {
        set_error(e.status, e.where.c_str());
        c->info.status = e.status;
        c->last_status = e.status;
    }
    c->info.kernel_launches = (int)(t_kernel_launches - l0);
    c->info.seconds =
        std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (c->pub.printtime) {
        const double *p = c->info.phase_ms;
        printf("|--GCG----------------------------\n");
        printf("|checkconv   compP   compRR   (rr_matW   eig)   compRV   compW   (linsol)   compX   initX  [ms]\n");
        printf("|%.2f\t%.2f\t%.2f\t(%.2f\t%.2f)\t%.2f\t%.2f\t(%.2f)\t%.2f\t%.2f\n", p[0], p[1],
               p[2] + p[3] + p[4], p[3], p[4], p[5], p[6] + p[7], p[7], p[8], p[9]);
    }
}

}  // namespace gcge
