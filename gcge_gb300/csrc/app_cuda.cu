// app_cuda: the CUDA backend of the OPS plugin surface and the C ABI of the
// library.  Semantics of each slot follow the reference backends it stands in
// for (app/app_ccs.c, app/app_lapack.c, src/ops_multi_vec.c); see gcge_cuda.h
// for the slot-by-slot map.  Host-side coefficient arrays and inner-product
// results cross the boundary exactly as in the reference (host double*,
// column-major, leading dimension), so a call that returns inner products
// synchronises the library stream.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <unordered_map>

#include "gcg.cuh"

namespace gcge {

thread_local unsigned long long t_kernel_launches = 0;
thread_local int t_pcg_share = 0;
static thread_local int t_last_error = GCGE_OK;
static thread_local std::string t_last_where;
static std::mutex g_detail_mu;
static std::string g_last_detail;
static std::atomic<unsigned long long> g_serial{1};

void set_error(int status, const char *where) {
    if (t_last_error == GCGE_OK) {
        t_last_error = status;
        t_last_where = where ? where : "";
    }
    {
        std::lock_guard<std::mutex> lk(g_detail_mu);
        g_last_detail = where ? where : "";
    }
    if (getenv("GCGE_CUDA_VERBOSE")) fprintf(stderr, "[gcge_cuda] error %d: %s\n", status, where);
}
int take_error() {
    const int e = t_last_error;
    t_last_error = GCGE_OK;
    return e;
}
const char *status_string(int s) {
    switch (s) {
        case GCGE_OK: return "ok";
        case GCGE_ERR_CUDA: return "CUDA runtime error";
        case GCGE_ERR_ARG: return "invalid argument";
        case GCGE_ERR_ALLOC: return "allocation failed";
        case GCGE_ERR_HANDLE: return "not a CUDA matrix or multivector";
        case GCGE_ERR_NUMERIC: return "non-finite or breakdown in the solver";
        case GCGE_ERR_NOT_CONVERGED: return "not converged within numIterMax";
        case GCGE_ERR_NO_DEVICE: return "no CUDA device";
        case GCGE_ERR_TOO_LARGE: return "projected problem too large";
        default: return "unknown";
    }
}

namespace {
// Per-device facts, queried once per device: SM count, and the stream-ordered
// pool told to keep freed blocks cached for reuse.
struct DeviceInfo {
    std::once_flag once;
    int sms = 0;
};
DeviceInfo g_dev[kMaxDevices];
std::once_flag g_count_once;
int g_ndev = 0;

// The calling thread's stream and OPS-slot staging buffers on each device it
// has used.  Destroyed at thread exit: buffers freed on their own stream, then
// the stream synchronised and destroyed.
struct ThreadDevice {
    cudaStream_t s = nullptr;
    SlotStage stage;
};
struct ThreadCtx {
    ThreadDevice dev[kMaxDevices];
    ~ThreadCtx() {
        for (int d = 0; d < kMaxDevices; ++d) {
            ThreadDevice &t = dev[d];
            if (!t.s) continue;
            if (cudaSetDevice(d) != cudaSuccess) continue;
            t.stage.release_on(t.s);
            cudaStreamSynchronize(t.s);
            cudaStreamDestroy(t.s);
            t.s = nullptr;
        }
    }
};
thread_local ThreadCtx t_ctx;
}  // namespace

void SlotStage::release_on(cudaStream_t st) {
    dcoef.release_on(st);
    dbeta.release_on(st);
    dres.release_on(st);
    scr.release_on(st);
    tc_exps.release_on(st);
}

int current_device() {
    std::call_once(g_count_once, [] {
        if (cudaGetDeviceCount(&g_ndev) != cudaSuccess) {
            cudaGetLastError();
            g_ndev = 0;
        }
    });
    if (g_ndev <= 0) throw CudaError{GCGE_ERR_NO_DEVICE, "no CUDA device visible"};
    int dev = 0;
    GCGE_CUDA(cudaGetDevice(&dev));
    GCGE_REQUIRE(dev >= 0 && dev < kMaxDevices, GCGE_ERR_NO_DEVICE, "device index out of range");
    DeviceInfo &d = g_dev[dev];
    std::call_once(d.once, [&d, dev] {
        if (cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            d.sms <= 0) {
            cudaGetLastError();
            d.sms = 148;
        }
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
            unsigned long long keep = ~0ULL;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
    });
    return dev;
}

cudaStream_t lib_stream() {
    ThreadDevice &t = t_ctx.dev[current_device()];
    if (t.s == nullptr) GCGE_CUDA(cudaStreamCreateWithFlags(&t.s, cudaStreamNonBlocking));
    return t.s;
}
int device_sms() { return g_dev[current_device()].sms; }
SlotStage &slot_stage() { return t_ctx.dev[current_device()].stage; }

MultiVec *as_mv(void *h) {
    MultiVec *m = reinterpret_cast<MultiVec *>(h);
    return (m && m->magic == kMultiVecMagic) ? m : nullptr;
}
SparseMat *as_mat(void *h) {
    SparseMat *m = reinterpret_cast<SparseMat *>(h);
    return (m && m->magic == kMatMagic) ? m : nullptr;
}
unsigned long long mat_serial(const SparseMat *m) { return m->serial; }

static MultiVec *mv_create(int nrows, int ncols) {
    MultiVec *m = new MultiVec();
    m->nrows = nrows;
    m->ncols = ncols;
    m->ld = std::max(32, (nrows + 31) / 32 * 32);
    const size_t bytes = sizeof(double) * (size_t)m->ld * std::max(ncols, 1);
    cudaError_t e = cudaMallocAsync((void **)&m->data, bytes, lib_stream());
    if (e != cudaSuccess) {
        delete m;
        throw CudaError{GCGE_ERR_ALLOC, std::string("multivector: ") + cudaGetErrorString(e)};
    }
    GCGE_CUDA(cudaMemsetAsync(m->data, 0, bytes, lib_stream()));
    return m;
}
static void mv_destroy(MultiVec *m) {
    if (!m) return;
    if (m->owns && m->data) {
        cudaStream_t st = nullptr;
        try {
            st = lib_stream();
        } catch (...) {
        }
        if (st) cudaFreeAsync(m->data, st);
        else cudaFree(m->data);
    }
    m->magic = 0;
    delete m;
}

#define GCGE_TRY(...)                                   \
    try {                                               \
        __VA_ARGS__;                                    \
    } catch (const ::gcge::CudaError &e_) {             \
        ::gcge::set_error(e_.status, e_.where.c_str()); \
    }
#define GCGE_TRY_RET(...)                               \
    try {                                               \
        __VA_ARGS__;                                    \
        return GCGE_OK;                                 \
    } catch (const ::gcge::CudaError &e_) {             \
        ::gcge::set_error(e_.status, e_.where.c_str()); \
        ::gcge::take_error();                           \
        return e_.status;                               \
    }

static MultiVec *need_mv(void *h, const char *what) {
    MultiVec *m = as_mv(h);
    GCGE_REQUIRE(m != nullptr, GCGE_ERR_HANDLE, std::string(what) + ": not a CUDA multivector");
    return m;
}
static void check_range(const MultiVec *m, int s, int e, const char *what) {
    GCGE_REQUIRE(s >= 0 && e >= s && e <= m->ncols, GCGE_ERR_ARG,
                 std::string(what) + ": column range out of bounds");
}

// ---------------------------------------------------------------- mat ops
static void mat_dot(SparseMat *A, MultiVec *x, MultiVec *y, int *start, int *end) {
    const int k = end[0] - start[0];
    GCGE_REQUIRE(k == end[1] - start[1], GCGE_ERR_ARG, "MatDotMultiVec: ranges differ");
    check_range(x, start[0], end[0], "MatDotMultiVec x");
    check_range(y, start[1], end[1], "MatDotMultiVec y");
    if (k == 0) return;
    cudaStream_t st = lib_stream();
    const double *X = x->data + (size_t)start[0] * x->ld;
    double *Y = y->data + (size_t)start[1] * y->ld;
    if (A == nullptr) {
        copy_cols(y->nrows, k, X, x->ld, Y, y->ld, st);  // mat == NULL -> copy
        return;
    }
    GCGE_REQUIRE(A->n == x->nrows && A->n == y->nrows, GCGE_ERR_ARG, "MatDotMultiVec: size");
    spmm<double>(A->pat, A->val.p, X, x->ld, Y, y->ld, k, st);
}

static void CUDA_MatDotMultiVec(void *mat, void **x, void **y, int *start, int *end, OPS *ops) {
    (void)ops;
    GCGE_TRY({
        SparseMat *A = nullptr;
        if (mat) {
            A = as_mat(mat);
            GCGE_REQUIRE(A != nullptr, GCGE_ERR_HANDLE, "MatDotMultiVec: not a CUDA matrix");
        }
        mat_dot(A, need_mv(x, "MatDotMultiVec"), need_mv(y, "MatDotMultiVec"), start, end);
    });
}
static void CUDA_MatView(void *mat, OPS *ops) {
    GCGE_TRY({
        SparseMat *A = as_mat(mat);
        GCGE_REQUIRE(A != nullptr, GCGE_ERR_HANDLE, "MatView");
        std::vector<int> ptr(A->n + 1), ind(std::max<long long>(A->nnz, 1));
        std::vector<double> val(std::max<long long>(A->nnz, 1));
        GCGE_CUDA(cudaMemcpy(ptr.data(), A->csr.ptr.p, sizeof(int) * (A->n + 1),
                             cudaMemcpyDeviceToHost));
        if (A->nnz > 0) {
            GCGE_CUDA(cudaMemcpy(ind.data(), A->csr.ind.p, sizeof(int) * A->nnz,
                                 cudaMemcpyDeviceToHost));
            GCGE_CUDA(cudaMemcpy(val.data(), A->csr.val.p, sizeof(double) * A->nnz,
                                 cudaMemcpyDeviceToHost));
        }
        for (int i = 0; i < A->n; ++i) {
            for (int j = 0; j < A->n; ++j) {
                double v = 0.0;
                for (int e = ptr[i]; e < ptr[i + 1]; ++e)
                    if (ind[e] == j) v += val[e];
                ops->Printf("%6.4e\t", v);
            }
            ops->Printf("\n");
        }
    });
}

// ---------------------------------------------------------------- multivec
static void CUDA_MultiVecCreateByMat(void ***mv, int num, void *src_mat, OPS *ops) {
    (void)ops;
    GCGE_TRY({
        SparseMat *A = as_mat(src_mat);
        GCGE_REQUIRE(A != nullptr, GCGE_ERR_HANDLE, "MultiVecCreateByMat: not a CUDA matrix");
        *mv = reinterpret_cast<void **>(mv_create(A->n, num));
    });
}
static void CUDA_MultiVecCreateByVec(void ***mv, int num, void *src_vec, OPS *ops) {
    (void)ops;
    GCGE_TRY({ *mv = reinterpret_cast<void **>(mv_create(need_mv(src_vec, "CreateByVec")->nrows, num)); });
}
static void CUDA_MultiVecCreateByMultiVec(void ***mv, int num, void **src, OPS *ops) {
    (void)ops;
    GCGE_TRY({ *mv = reinterpret_cast<void **>(mv_create(need_mv(src, "CreateByMultiVec")->nrows, num)); });
}
static void CUDA_MultiVecDestroy(void ***mv, int num, OPS *ops) {
    (void)num;
    (void)ops;
    if (!mv || !*mv) return;
    GCGE_TRY({
        MultiVec *m = need_mv(*mv, "MultiVecDestroy");
        cudaStreamSynchronize(lib_stream());
        mv_destroy(m);
        *mv = nullptr;
    });
}
static void CUDA_GetVecFromMultiVec(void **mv, int col, void **vec, OPS *ops) {
    (void)ops;
    GCGE_TRY({
        MultiVec *m = need_mv(mv, "GetVecFromMultiVec");
        check_range(m, col, col + 1, "GetVecFromMultiVec");
        MultiVec *v = new MultiVec();
        v->nrows = m->nrows;
        v->ncols = 1;
        v->ld = m->ld;
        v->data = m->data + (size_t)col * m->ld;
        v->owns = false;
        *vec = v;
    });
}
static void CUDA_RestoreVecForMultiVec(void **mv, int col, void **vec, OPS *ops) {
    (void)mv;
    (void)col;
    (void)ops;
    GCGE_TRY({
        MultiVec *v = need_mv(*vec, "RestoreVecForMultiVec");
        v->magic = 0;
        delete v;
        *vec = nullptr;
    });
}
static void CUDA_MultiVecView(void **x, int start, int end, OPS *ops) {
    GCGE_TRY({
        MultiVec *m = need_mv(x, "MultiVecView");
        check_range(m, start, end, "MultiVecView");
        std::vector<double> h((size_t)m->nrows * std::max(end - start, 0));
        if (end > start) {
            GCGE_CUDA(cudaMemcpy2DAsync(h.data(), sizeof(double) * m->nrows,
                                        m->data + (size_t)start * m->ld, sizeof(double) * m->ld,
                                        sizeof(double) * m->nrows, end - start,
                                        cudaMemcpyDeviceToHost, lib_stream()));
            GCGE_CUDA(cudaStreamSynchronize(lib_stream()));
        }
        for (int i = 0; i < m->nrows; ++i) {
            for (int c = 0; c < end - start; ++c) ops->Printf("%6.4e\t", h[i + (size_t)c * m->nrows]);
            ops->Printf("\n");
        }
    });
}

static void CUDA_MultiVecSetRandomValue(void **x, int start, int end, OPS *ops) {
    (void)ops;
    static unsigned long long counter = 1;
    GCGE_TRY({
        MultiVec *m = need_mv(x, "MultiVecSetRandomValue");
        check_range(m, start, end, "MultiVecSetRandomValue");
        fill_uniform(m->nrows, end - start, m->data + (size_t)start * m->ld, m->ld, counter++,
                     lib_stream());
    });
}

// y = alpha x + beta y over the column ranges (app/app_lapack.c:334-395)
static void CUDA_MultiVecAxpby(double alpha, void **x, double beta, void **y, int *start, int *end,
                               OPS *ops) {
    (void)ops;
    GCGE_TRY({
        MultiVec *Y = need_mv(y, "MultiVecAxpby");
        const int k = end[1] - start[1];
        GCGE_REQUIRE(end[0] - start[0] == k, GCGE_ERR_ARG, "MultiVecAxpby: ranges differ");
        check_range(Y, start[1], end[1], "MultiVecAxpby y");
        const double *X = nullptr;
        int ldx = 0;
        if (x) {
            MultiVec *Xm = need_mv(x, "MultiVecAxpby");
            check_range(Xm, start[0], end[0], "MultiVecAxpby x");
            GCGE_REQUIRE(Xm->nrows == Y->nrows, GCGE_ERR_ARG, "MultiVecAxpby: rows differ");
            X = Xm->data + (size_t)start[0] * Xm->ld;
            ldx = Xm->ld;
        }
        axpby(Y->nrows, k, alpha, X, ldx, beta, Y->data + (size_t)start[1] * Y->ld, Y->ld,
              lib_stream());
    });
}

// y = x coef + y diag(beta) (app/app_lapack.c:463-534)
static void CUDA_MultiVecLinearComb(void **x, void **y, int is_vec, int *start, int *end,
                                    double *coef, int ldc, double *beta, int incb, OPS *ops) {
    (void)is_vec;
    (void)ops;
    GCGE_TRY({
        MultiVec *Y = need_mv(y, "MultiVecLinearComb");
        const int k = end[0] - start[0], m = end[1] - start[1];
        if (k == 0 || m == 0 || Y->nrows == 0) return;
        check_range(Y, start[1], end[1], "MultiVecLinearComb y");
        cudaStream_t st = lib_stream();
        SlotStage &sg = slot_stage();
        DevBuf<double> &dcoef = sg.dcoef, &dbeta = sg.dbeta;
        PinnedBuf<double> &hstage = sg.hstage;
        double *Yp = Y->data + (size_t)start[1] * Y->ld;
        const double *dB = nullptr;
        if (beta) {
            const int nb = incb == 0 ? 1 : m;
            hstage.alloc((size_t)nb + (size_t)k * m + 1);
            GCGE_CUDA(cudaStreamSynchronize(st));
            for (int j = 0; j < nb; ++j) hstage.p[j] = beta[(size_t)j * (incb == 0 ? 0 : incb)];
            dbeta.alloc(nb);
            GCGE_CUDA(cudaMemcpyAsync(dbeta.p, hstage.p, sizeof(double) * nb, cudaMemcpyHostToDevice, st));
            dB = dbeta.p;
        }
        if (x && coef) {
            MultiVec *X = need_mv(x, "MultiVecLinearComb");
            check_range(X, start[0], end[0], "MultiVecLinearComb x");
            GCGE_REQUIRE(X->nrows == Y->nrows, GCGE_ERR_ARG, "MultiVecLinearComb: rows differ");
            hstage.alloc((size_t)k * m + 1 + (size_t)m);
            GCGE_CUDA(cudaStreamSynchronize(st));
            for (int j = 0; j < m; ++j)
                for (int i = 0; i < k; ++i) hstage.p[i + (size_t)j * k] = coef[i + (size_t)j * ldc];
            dcoef.alloc((size_t)k * m);
            GCGE_CUDA(cudaMemcpyAsync(dcoef.p, hstage.p, sizeof(double) * k * m, cudaMemcpyHostToDevice, st));
            // with beta: Y = X C + diag(beta) Y; without: Y = X C
            lincomb(Y->nrows, k, m, X->data + (size_t)start[0] * X->ld, X->ld, dcoef.p, k, Yp, Y->ld,
                    dB, incb == 0 ? 0 : 1, st);
        } else if (beta) {
            scale_columns_strided(Y->nrows, m, Yp, Y->ld, dB, incb == 0 ? 0 : 1, st);
        }
        GCGE_CUDA(cudaStreamSynchronize(st));
    });
}

// inner products with the 'N' / 'S' / 'D' conventions of DenseMatQtAP
// (app/app_lapack.c:64-183), results to host
static void inner_prod_impl(char nsd, MultiVec *X, MultiVec *Y, int *start, int *end, double *ip,
                       int ldIP) {
    const int nr = end[0] - start[0], nc = end[1] - start[1];
    if (nr <= 0 || nc <= 0) return;
    check_range(X, start[0], end[0], "MultiVecInnerProd x");
    check_range(Y, start[1], end[1], "MultiVecInnerProd y");
    GCGE_REQUIRE(X->nrows == Y->nrows, GCGE_ERR_ARG, "MultiVecInnerProd: rows differ");
    cudaStream_t st = lib_stream();
    SlotStage &sg = slot_stage();
    DevBuf<double> &dres = sg.dres, &scr = sg.scr;
    PinnedBuf<double> &hres = sg.hres;
    const int n = X->nrows;
    const double *Xp = X->data + (size_t)start[0] * X->ld;
    const double *Yp = Y->data + (size_t)start[1] * Y->ld;
    if (nsd == 'D') {
        GCGE_REQUIRE(nr == nc, GCGE_ERR_ARG, "MultiVecInnerProd 'D': ranges differ");
        dres.alloc(nc);
        scr.alloc((size_t)nc * 4096);
        coldot(n, nc, Xp, X->ld, Yp, Y->ld, dres.p, scr.p, scr.n, st);
        hres.alloc(nc);
        GCGE_CUDA(cudaMemcpyAsync(hres.p, dres.p, sizeof(double) * nc, cudaMemcpyDeviceToHost, st));
        GCGE_CUDA(cudaStreamSynchronize(st));
        for (int i = 0; i < nc; ++i) ip[(size_t)ldIP * i] = hres.p[i];
        return;
    }
    dres.alloc((size_t)nr * nc);
    scr.alloc(gram_scratch_elems(n, nr, nc));
    gram(n, nr, nc, Xp, X->ld, Yp, Y->ld, dres.p, nr, scr.p, scr.n, st);
    hres.alloc((size_t)nr * nc);
    GCGE_CUDA(cudaMemcpyAsync(hres.p, dres.p, sizeof(double) * nr * nc, cudaMemcpyDeviceToHost, st));
    GCGE_CUDA(cudaStreamSynchronize(st));
    if (nsd == 'S') {
        GCGE_REQUIRE(nr == nc, GCGE_ERR_ARG, "MultiVecInnerProd 'S': not square");
        // lower triangle computed, mirrored to the upper (app/app_lapack.c:116-134)
        for (int j = 0; j < nc; ++j)
            for (int i = j; i < nr; ++i) {
                const double v = hres.p[i + (size_t)j * nr];
                ip[i + (size_t)j * ldIP] = v;
                ip[j + (size_t)i * ldIP] = v;
            }
    } else {
        for (int j = 0; j < nc; ++j)
            for (int i = 0; i < nr; ++i) ip[i + (size_t)j * ldIP] = hres.p[i + (size_t)j * nr];
    }
}

static void CUDA_MultiVecInnerProd(char nsdIP, void **x, void **y, int is_vec, int *start, int *end,
                                   double *inner_prod, int ldIP, OPS *ops) {
    (void)is_vec;
    (void)ops;
    GCGE_TRY({
        inner_prod_impl(nsdIP, need_mv(x, "MultiVecInnerProd"), need_mv(y, "MultiVecInnerProd"), start,
                   end, inner_prod, ldIP);
    });
}

// qAp = Q^T op(A) P (src/ops_multi_vec.c:351-411): A P into mv_ws, then the
// inner product, both on the device; 'T' returns the transpose.
static void CUDA_MultiVecQtAP(char ntsA, char ntsdQAP, void **mvQ, void *matA, void **mvP,
                              int is_vec, int *start, int *end, double *qAp, int ldQAP,
                              void **mv_ws, OPS *ops) {
    (void)ntsA;
    (void)is_vec;
    (void)ops;
    GCGE_TRY({
        const int nrows = end[0] - start[0], ncols = end[1] - start[1];
        if (nrows <= 0 || ncols <= 0) return;
        MultiVec *Q = need_mv(mvQ, "MultiVecQtAP"), *P = need_mv(mvP, "MultiVecQtAP");
        MultiVec *PA = P;
        int s2[2] = {start[0], start[1]}, e2[2] = {end[0], end[1]};
        if (matA) {
            SparseMat *A = as_mat(matA);
            GCGE_REQUIRE(A != nullptr, GCGE_ERR_HANDLE, "MultiVecQtAP: not a CUDA matrix");
            MultiVec *W = need_mv(mv_ws, "MultiVecQtAP workspace");
            GCGE_REQUIRE(W->ncols >= ncols, GCGE_ERR_ARG, "MultiVecQtAP: workspace too small");
            int ss[2] = {start[1], 0}, ee[2] = {end[1], ncols};
            mat_dot(A, P, W, ss, ee);
            PA = W;
            s2[1] = 0;
            e2[1] = ncols;
        }
        if (ntsdQAP == 'T') {
            int st2[2] = {s2[1], s2[0]}, en2[2] = {e2[1], e2[0]};
            inner_prod_impl('N', PA, Q, st2, en2, qAp, ldQAP);
        } else {
            inner_prod_impl(ntsdQAP, Q, PA, s2, e2, qAp, ldQAP);
        }
    });
}

// ---------------------------------------------------------------- vec ops
static void CUDA_VecCreateByMat(void **v, void *m, OPS *ops) {
    void **mv = nullptr;
    CUDA_MultiVecCreateByMat(&mv, 1, m, ops);
    *v = mv;
}
static void CUDA_VecCreateByVec(void **v, void *src, OPS *ops) {
    void **mv = nullptr;
    CUDA_MultiVecCreateByVec(&mv, 1, src, ops);
    *v = mv;
}
static void CUDA_VecDestroy(void **v, OPS *ops) {
    void **mv = reinterpret_cast<void **>(*v);
    CUDA_MultiVecDestroy(&mv, 1, ops);
    *v = nullptr;
}
static void CUDA_VecView(void *x, OPS *ops) { CUDA_MultiVecView((void **)x, 0, 1, ops); }
static void CUDA_VecInnerProd(void *x, void *y, double *ip, OPS *ops) {
    int s[2] = {0, 0}, e[2] = {1, 1};
    CUDA_MultiVecInnerProd('S', (void **)x, (void **)y, 0, s, e, ip, 1, ops);
}
static void CUDA_VecSetRandomValue(void *x, OPS *ops) { CUDA_MultiVecSetRandomValue((void **)x, 0, 1, ops); }
static void CUDA_VecAxpby(double a, void *x, double b, void *y, OPS *ops) {
    int s[2] = {0, 0}, e[2] = {1, 1};
    CUDA_MultiVecAxpby(a, (void **)x, b, (void **)y, s, e, ops);
}
static void CUDA_MatDotVec(void *m, void *x, void *y, OPS *ops) {
    int s[2] = {0, 0}, e[2] = {1, 1};
    CUDA_MatDotMultiVec(m, (void **)x, (void **)y, s, e, ops);
}

// ---------------------------------------------------------------- defaults
static void default_printf(const char *fmt, ...) {
    va_list vp;
    va_start(vp, fmt);
    vprintf(fmt, vp);
    va_end(vp);
}
static double default_wtime(void) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}
// "-name value" lookup with the reference's types 'i', 'f', 's'
// (src/ops_multi_vec.c:58-95); returns 1 when the option was found with a value.
static int default_option(const char *name, char type, void *value, int argc, char *argv[], OPS *ops) {
    (void)ops;
    for (int i = 0; i < argc; ++i) {
        if (std::strcmp(argv[i], name) != 0) continue;
        if (i + 1 >= argc) return 0;
        switch (type) {
            case 'i': *(int *)value = atoi(argv[i + 1]); break;
            case 'f': *(double *)value = atof(argv[i + 1]); break;
            case 's': std::strcpy((char *)value, argv[i + 1]); break;
            default: break;
        }
        return 1;
    }
    return 0;
}

// ---------------------------------------------------------------- MultiVecOrth
// State behind ops->orth_workspace after MultiVecOrthSetup_*: the method, its
// parameters and the device work buffers of the orthogonalisation.
struct OrthSetup {
    bool bgs = false;
    int block_size = -1, max_reorth = 1;
    double zero_tol = 1e-14;
    SolverCtx work;
};
static std::mutex g_orth_mu;
static std::unordered_map<OPS *, OrthSetup *> g_orth;

static OrthSetup *orth_for(OPS *ops, bool create) {
    std::lock_guard<std::mutex> lk(g_orth_mu);
    auto it = g_orth.find(ops);
    if (it != g_orth.end()) return it->second;
    if (!create) return nullptr;
    OrthSetup *o = new OrthSetup();
    g_orth[ops] = o;
    return o;
}
static void orth_release(OPS *ops) {
    OrthSetup *o = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_orth_mu);
        auto it = g_orth.find(ops);
        if (it == g_orth.end()) return;
        o = it->second;
        g_orth.erase(it);
    }
    delete o;
}

// ops->MultiVecOrth (src/ops_orth.c:203-394 "mgs", :519-623 "bgs"): columns
// [start_x, *end_x) of x B-orthonormalised against [0, start_x) and among
// themselves; *end_x shrinks by the columns dropped as dependent.
static void cuda_multivec_orth(void **x, int start_x, int *end_x, void *B, OPS *ops) {
    try {
        OrthSetup *o = orth_for(ops, false);
        GCGE_REQUIRE(o && ops->orth_workspace == (void *)o, GCGE_ERR_ARG,
                     "MultiVecOrth: no MultiVecOrthSetup_* on this ops");
        MultiVec *xv = as_mv(x);
        SparseMat *Bm = B ? as_mat(B) : nullptr;
        GCGE_REQUIRE(xv && end_x && (!B || Bm), GCGE_ERR_HANDLE, "MultiVecOrth: handles");
        GCGE_REQUIRE(start_x >= 0 && *end_x >= start_x && *end_x <= xv->ncols, GCGE_ERR_ARG,
                     "MultiVecOrth: range");
        GCGE_REQUIRE(!Bm || Bm->n == xv->nrows, GCGE_ERR_ARG, "MultiVecOrth: B size");
        if (*end_x == start_x) return;
        o->work.reserve(xv->nrows, xv->ncols, xv->ncols, 1, 1);
        if (o->bgs)
            *end_x = bgs_orth(o->work, Bm, xv->data, xv->ld, xv->nrows, start_x, *end_x,
                              Bm != nullptr, o->zero_tol, o->max_reorth, o->block_size, nullptr);
        else
            *end_x = borth(o->work, Bm, xv->data, xv->ld, xv->nrows, start_x, *end_x, Bm != nullptr,
                           o->zero_tol, o->max_reorth, nullptr);
        GCGE_CUDA(cudaStreamSynchronize(lib_stream()));
    } catch (const CudaError &e) {
        set_error(e.status, e.where.c_str());
    }
}

static void orth_setup(bool bgs, int block_size, int max_reorth, double orth_zero_tol, OPS *ops) {
    OrthSetup *o = orth_for(ops, true);
    o->bgs = bgs;
    o->block_size = block_size;
    o->max_reorth = max_reorth;
    o->zero_tol = orth_zero_tol;
    ops->orth_workspace = (void *)o;
    ops->MultiVecOrth = cuda_multivec_orth;
}

static void init_solver_defaults(GCGSolver &g) {
    // static defaults of EigenSolverSetup_GCG (src/ops_eig_sol_gcg.c:1573-1603)
    std::memset(&g, 0, sizeof(g));
    g.nevMax = 3;
    g.gapMin = 0.01;
    g.nevInit = 3;
    g.block_size = 1;
    g.numIterMax = 4;
    std::strcpy(g.initX_orth_method, "mgs");
    g.initX_orth_block_size = -1;
    g.initX_orth_max_reorth = 1;
    g.initX_orth_zero_tol = 1e-14;
    g.check_conv_max_num = 15;
    std::strcpy(g.compP_orth_method, "mgs");
    g.compP_orth_block_size = -1;
    g.compP_orth_max_reorth = 1;
    g.compP_orth_zero_tol = 1e-14;
    std::strcpy(g.compW_orth_method, "mgs");
    g.compW_orth_block_size = -1;
    g.compW_orth_max_reorth = 1;
    g.compW_orth_zero_tol = 1e-14;
    g.compW_cg_max_iter = 40;
    g.compW_cg_rate = 1e-2;
    g.compW_cg_tol = 1e-8;
    std::strcpy(g.compW_cg_tol_type, "abs");
    g.compW_cg_auto_shift = 0;
    g.compW_cg_shift = 0.0;
    g.compW_cg_order = 1;
    g.compRR_min_gap = 0.01;
    g.compRR_min_num = -1;
    g.compRR_tol = 1e-16;
}

}  // namespace gcge

using namespace gcge;

// ==================================================================== C ABI
extern "C" {

int ops_cuda_last_error(void) { return take_error(); }
const char *ops_cuda_error_string(int s) { return status_string(s); }
const char *ops_cuda_last_error_detail(void) {
    std::lock_guard<std::mutex> lk(g_detail_mu);
    static thread_local std::string copy;
    copy = g_last_detail;
    return copy.c_str();
}

void OPS_Create(OPS **ops) {
    *ops = (OPS *)calloc(1, sizeof(OPS));
}
void OPS_Setup(OPS *ops) {
    if (!ops->Printf) ops->Printf = default_printf;
    if (!ops->GetWtime) ops->GetWtime = default_wtime;
    if (!ops->GetOptionFromCommandLine) ops->GetOptionFromCommandLine = default_option;
}
void OPS_Destroy(OPS **ops) {
    if (!ops || !*ops) return;
    orth_release(*ops);
    ctx_release(*ops);
    linsol_release(*ops);
    amg_release(*ops);
    if ((*ops)->lapack_ops) OPS_Destroy(&(*ops)->lapack_ops);
    free(*ops);
    *ops = nullptr;
}

// src/ops_orth.c:395-414 (mgs) and :625-641 (bgs).  mv_ws and dbl_ws are
// accepted for signature compatibility; the device work buffers belong to the
// ops object and are freed by OPS_Destroy.
void MultiVecOrthSetup_ModifiedGramSchmidt(int block_size, int max_reorth, double orth_zero_tol,
                                           void **mv_ws, double *dbl_ws, OPS *ops) {
    (void)mv_ws;
    (void)dbl_ws;
    orth_setup(false, block_size, max_reorth, orth_zero_tol, ops);
}
void MultiVecOrthSetup_BinaryGramSchmidt(int block_size, int max_reorth, double orth_zero_tol,
                                         void **mv_ws, double *dbl_ws, OPS *ops) {
    (void)mv_ws;
    (void)dbl_ws;
    orth_setup(true, block_size, max_reorth, orth_zero_tol, ops);
}

void OPS_CUDA_Set(OPS *ops) {
    ops->Printf = default_printf;
    ops->GetWtime = default_wtime;
    ops->GetOptionFromCommandLine = default_option;
    ops->MatView = CUDA_MatView;
    ops->MatAxpby = nullptr;  // as app_ccs: the shift goes through the union-pattern operator
    ops->VecCreateByMat = CUDA_VecCreateByMat;
    ops->VecCreateByVec = CUDA_VecCreateByVec;
    ops->VecDestroy = CUDA_VecDestroy;
    ops->VecView = CUDA_VecView;
    ops->VecInnerProd = CUDA_VecInnerProd;
    ops->VecLocalInnerProd = CUDA_VecInnerProd;
    ops->VecSetRandomValue = CUDA_VecSetRandomValue;
    ops->VecAxpby = CUDA_VecAxpby;
    ops->MatDotVec = CUDA_MatDotVec;
    ops->MatTransDotVec = CUDA_MatDotVec;  // symmetric matrices (app/app_ccs.c:140-150)
    ops->MultiVecCreateByMat = CUDA_MultiVecCreateByMat;
    ops->MultiVecCreateByVec = CUDA_MultiVecCreateByVec;
    ops->MultiVecCreateByMultiVec = CUDA_MultiVecCreateByMultiVec;
    ops->MultiVecDestroy = CUDA_MultiVecDestroy;
    ops->GetVecFromMultiVec = CUDA_GetVecFromMultiVec;
    ops->RestoreVecForMultiVec = CUDA_RestoreVecForMultiVec;
    ops->MultiVecView = CUDA_MultiVecView;
    ops->MultiVecLocalInnerProd = CUDA_MultiVecInnerProd;
    ops->MultiVecInnerProd = CUDA_MultiVecInnerProd;
    ops->MultiVecSetRandomValue = CUDA_MultiVecSetRandomValue;
    ops->MultiVecAxpby = CUDA_MultiVecAxpby;
    ops->MultiVecLinearComb = CUDA_MultiVecLinearComb;
    ops->MatDotMultiVec = CUDA_MatDotMultiVec;
    ops->MatTransDotMultiVec = CUDA_MatDotMultiVec;
    ops->MultiVecQtAP = CUDA_MultiVecQtAP;
    // level transfers for the block AMG solver (no app_ccs counterpart)
    ops->MultiVecFromItoJ = CUDA_MultiVecFromItoJ;
}

int CUDA_MatCreateFromCCS(void **mat, int nrows, int ncols, const int *j_col, const int *i_row,
                          const double *data) {
    GCGE_TRY_RET({
        GCGE_REQUIRE(mat && j_col && nrows > 0 && nrows == ncols, GCGE_ERR_ARG,
                     "CUDA_MatCreateFromCCS: square matrix with column pointers required");
        const int n = nrows;
        const long long nnz = j_col[n];
        GCGE_REQUIRE(nnz >= 0 && (nnz == 0 || (i_row && data)), GCGE_ERR_ARG,
                     "CUDA_MatCreateFromCCS: arrays");
        for (int j = 0; j < n; ++j)
            GCGE_REQUIRE(j_col[j] <= j_col[j + 1], GCGE_ERR_ARG,
                         "CUDA_MatCreateFromCCS: column pointers must not decrease");
        GCGE_REQUIRE(j_col[0] == 0, GCGE_ERR_ARG, "CUDA_MatCreateFromCCS: j_col[0] must be 0");
        SparseMat *A = new SparseMat();
        A->serial = g_serial.fetch_add(1);
        A->n = n;
        A->nnz = nnz;
        cudaStream_t st = lib_stream();
        try {
            // CCS -> CSR on the device (y = A x for any A), then SELL-32
            csr_from_ccs_device(n, j_col, i_row, data, A->csr, st);
            sell_from_csr_device(A->csr, nullptr, A->pat, A->val, nullptr, st);
            GCGE_CUDA(cudaStreamSynchronize(st));
        } catch (...) {
            delete A;
            throw;
        }
        *mat = A;
    });
}
void CUDA_MatDestroy(void **mat) {
    if (!mat || !*mat) return;
    SparseMat *A = as_mat(*mat);
    if (!A) {
        set_error(GCGE_ERR_HANDLE, "CUDA_MatDestroy");
        return;
    }
    cudaStreamSynchronize(lib_stream());
    A->magic = 0;
    delete A;
    *mat = nullptr;
}
// ops->MatAxpby (src/ops.h:52: Y = alpha X + beta Y).  app_ccs leaves the slot
// NULL, and so does OPS_CUDA_Set, so GCG takes the same branch as with the
// reference's CCS backend (src/ops_eig_sol_gcg.c:600-631); the GPU GCG forms
// A + sigma B on the union pattern of A and B itself.  A caller may install
// CUDA_MatAxpby in the slot.  Y takes the union pattern of X and Y (rebuilt
// on the device) and a new identity, so solver caches keyed on Y rebuild.
void CUDA_MatAxpby(double alpha, void *matX, double beta, void *matY, OPS *ops) {
    (void)ops;
    try {
        SparseMat *X = as_mat(matX), *Y = as_mat(matY);
        GCGE_REQUIRE(X && Y, GCGE_ERR_HANDLE, "MatAxpby: matrices");
        GCGE_REQUIRE(X->n == Y->n, GCGE_ERR_ARG, "MatAxpby: sizes differ");
        cudaStream_t st = lib_stream();
        DevCsr U;
        DevBuf<double> yv;
        if (X == Y) {  // Y = (alpha + beta) Y on its own pattern
            const double f = alpha + beta;
            axpby((int)Y->csr.nnz, 1, 0.0, nullptr, 0, f, Y->csr.val.p, (int)Y->csr.nnz, st);
        } else {
            // values of X on the union in U.val, values of Y in yv
            union_csr_device(X->csr, &Y->csr, U, yv, st);
            axpby((int)U.nnz, 1, alpha, U.val.p, (int)U.nnz, beta, yv.p, (int)U.nnz, st);
            std::swap(Y->csr.ptr.p, U.ptr.p);
            std::swap(Y->csr.ptr.n, U.ptr.n);
            std::swap(Y->csr.ind.p, U.ind.p);
            std::swap(Y->csr.ind.n, U.ind.n);
            std::swap(Y->csr.val.p, yv.p);
            std::swap(Y->csr.val.n, yv.n);
            Y->csr.nnz = U.nnz;
            Y->nnz = U.nnz;
        }
        sell_from_csr_device(Y->csr, nullptr, Y->pat, Y->val, nullptr, st);
        Y->serial = g_serial.fetch_add(1);
        GCGE_CUDA(cudaStreamSynchronize(st));
    } catch (const CudaError &e) {
        set_error(e.status, e.where.c_str());
    }
}

int CUDA_MatNnz(void *mat, long long *nnz) {
    SparseMat *A = as_mat(mat);
    if (!A) return GCGE_ERR_HANDLE;
    *nnz = A->nnz;
    return GCGE_OK;
}

int CUDA_MultiVecSetFromHost(void **mv, int start, int end, const double *host, int ldh) {
    GCGE_TRY_RET({
        MultiVec *m = need_mv(mv, "CUDA_MultiVecSetFromHost");
        check_range(m, start, end, "CUDA_MultiVecSetFromHost");
        GCGE_REQUIRE(ldh >= m->nrows, GCGE_ERR_ARG, "CUDA_MultiVecSetFromHost: ldh");
        if (end > start) {
            GCGE_CUDA(cudaMemcpy2DAsync(m->data + (size_t)start * m->ld, sizeof(double) * m->ld, host,
                                        sizeof(double) * ldh, sizeof(double) * m->nrows, end - start,
                                        cudaMemcpyHostToDevice, lib_stream()));
            GCGE_CUDA(cudaStreamSynchronize(lib_stream()));
        }
    });
}
// Columns of a device block stored by the GPU straight into page-locked host
// memory (column c of src, leading dimension lds, into dst with ldd).  The
// copy engine's first pass over data that kernels have just written runs at
// a tenth of the link's rate on this part (0.3-0.9 s for the 5.4 GB of a
// 128^3 solve's eigenvectors, against 28 ms for a repeated copy); stores from
// a kernel go at the link's rate.
__global__ void __launch_bounds__(256) k_cols_to_host(const double *__restrict__ src, size_t lds,
                                                      double *__restrict__ dst, size_t ldd,
                                                      int rows) {
    const double *s = src + (size_t)blockIdx.y * lds;
    double *d = dst + (size_t)blockIdx.y * ldd;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (((reinterpret_cast<uintptr_t>(s) | reinterpret_cast<uintptr_t>(d)) & 15) == 0) {
        const size_t h = (size_t)rows / 2;
        for (; i < h; i += stride)
            reinterpret_cast<double2 *>(d)[i] = reinterpret_cast<const double2 *>(s)[i];
        if ((rows & 1) && blockIdx.x == 0 && threadIdx.x == 0) d[rows - 1] = s[rows - 1];
    } else {
        for (; i < (size_t)rows; i += stride) d[i] = s[i];
    }
}

int CUDA_MultiVecGetToHost(void **mv, int start, int end, double *host, int ldh) {
    GCGE_TRY_RET({
        MultiVec *m = need_mv(mv, "CUDA_MultiVecGetToHost");
        check_range(m, start, end, "CUDA_MultiVecGetToHost");
        GCGE_REQUIRE(ldh >= m->nrows, GCGE_ERR_ARG, "CUDA_MultiVecGetToHost: ldh");
        if (end > start) {
            cudaStream_t st = lib_stream();
            const double *src = m->data + (size_t)start * m->ld;
            cudaPointerAttributes pa{};
            const bool pinned = cudaPointerGetAttributes(&pa, host) == cudaSuccess &&
                                pa.type == cudaMemoryTypeHost && pa.devicePointer != nullptr;
            cudaGetLastError();
            if (pinned && m->nrows > 0) {
                const int bx = (int)std::min<long long>(64, ((long long)m->nrows + 511) / 512);
                k_cols_to_host<<<dim3(bx, end - start), 256, 0, st>>>(
                    src, m->ld, static_cast<double *>(pa.devicePointer), (size_t)ldh, m->nrows);
                GCGE_CHECK_LAUNCH();
                count_launch();
            } else {
                GCGE_CUDA(cudaMemcpy2DAsync(host, sizeof(double) * ldh, src,
                                            sizeof(double) * m->ld, sizeof(double) * m->nrows,
                                            end - start, cudaMemcpyDeviceToHost, st));
            }
            GCGE_CUDA(cudaStreamSynchronize(st));
        }
    });
}
int CUDA_MultiVecSize(void **mv, int *nrows, int *ncols) {
    MultiVec *m = as_mv(mv);
    if (!m) return GCGE_ERR_HANDLE;
    *nrows = m->nrows;
    *ncols = m->ncols;
    return GCGE_OK;
}

// ---------------------------------------------------------------- GCG setup
void EigenSolverSetup_GCG(double gapMin, int nevInit, int nevMax, int block_size, double tol[2],
                          int numIterMax, int print, int printtime,
                          int user_defined_multi_linear_solver, void **mv_ws[4], double *dbl_ws,
                          int *int_ws, OPS *ops) {
    SolverCtx *c = ctx_for(ops, true);
    GCGSolver &g = c->pub;
    if (!c->pub_init) {
        init_solver_defaults(g);
        c->pub_init = true;
    }
    g.gapMin = gapMin;
    g.nevInit = nevInit;
    g.nevMax = nevMax;
    g.block_size = block_size;
    g.tol[0] = tol[0];
    g.tol[1] = tol[1];
    g.numIterMax = numIterMax;
    g.print = print;
    g.printtime = printtime;
    for (int i = 0; i < 4; ++i) g.mv_ws[i] = mv_ws[i];
    g.dbl_ws = dbl_ws;
    g.int_ws = int_ws;
    g.compRR_min_gap = gapMin;
    g.check_conv_max_num = block_size;
    g.user_defined_multi_linear_solver = user_defined_multi_linear_solver;
    ops->eigen_solver_workspace = (void *)&g;
    ops->EigenSolver = gcg_eigensolver;
}

void EigenSolverSetParameters_GCG(
    int check_conv_max_num, const char *initX_orth_method, int initX_orth_block_size,
    int initX_orth_max_reorth, double initX_orth_zero_tol, const char *compP_orth_method,
    int compP_orth_block_size, int compP_orth_max_reorth, double compP_orth_zero_tol,
    const char *compW_orth_method, int compW_orth_block_size, int compW_orth_max_reorth,
    double compW_orth_zero_tol, int compW_cg_max_iter, double compW_cg_rate, double compW_cg_tol,
    const char *compW_cg_tol_type, int compW_cg_auto_shift, int compRR_min_num,
    double compRR_min_gap, double compRR_tol, OPS *ops) {
    // set-if-given semantics of src/ops_eig_sol_gcg.c:1684-1741
    SolverCtx *c = ctx_for(ops, false);
    if (!c) {
        set_error(GCGE_ERR_ARG, "EigenSolverSetParameters_GCG before EigenSolverSetup_GCG");
        return;
    }
    GCGSolver &g = c->pub;
    auto cpy = [](char *dst, const char *src) {
        std::strncpy(dst, src, 7);
        dst[7] = 0;
    };
    if (check_conv_max_num > 0) g.check_conv_max_num = check_conv_max_num;
    if (initX_orth_method) cpy(g.initX_orth_method, initX_orth_method);
    if (initX_orth_block_size > 0) g.initX_orth_block_size = initX_orth_block_size;
    if (initX_orth_max_reorth >= 0) g.initX_orth_max_reorth = initX_orth_max_reorth;
    if (initX_orth_zero_tol > 0) g.initX_orth_zero_tol = initX_orth_zero_tol;
    if (compP_orth_method) cpy(g.compP_orth_method, compP_orth_method);
    if (compP_orth_block_size > 0) g.compP_orth_block_size = compP_orth_block_size;
    if (compP_orth_max_reorth >= 0) g.compP_orth_max_reorth = compP_orth_max_reorth;
    if (compP_orth_zero_tol > 0) g.compP_orth_zero_tol = compP_orth_zero_tol;
    if (compW_orth_method) cpy(g.compW_orth_method, compW_orth_method);
    if (compW_orth_block_size > 0) g.compW_orth_block_size = compW_orth_block_size;
    if (compW_orth_max_reorth >= 0) g.compW_orth_max_reorth = compW_orth_max_reorth;
    if (compW_orth_zero_tol > 0) g.compW_orth_zero_tol = compW_orth_zero_tol;
    if (compW_cg_max_iter > 0) g.compW_cg_max_iter = compW_cg_max_iter;
    if (compW_cg_rate > 0) g.compW_cg_rate = compW_cg_rate;
    if (compW_cg_tol > 0) g.compW_cg_tol = compW_cg_tol;
    if (compW_cg_tol_type) cpy(g.compW_cg_tol_type, compW_cg_tol_type);
    g.compW_cg_auto_shift = compW_cg_auto_shift;
    if (compRR_min_gap > 0) g.compRR_min_gap = compRR_min_gap;
    if (compRR_min_num > 0) g.compRR_min_num = compRR_min_num;
    if (compRR_tol > 0) g.compRR_tol = compRR_tol;
}

// src/ops_eig_sol_gcg.c:1743-1862: every "-gcge_*" option present in argv
// overrides its parameter, read with ops->GetOptionFromCommandLine.  Option
// names and types are the reference's, with two exceptions: -gcge_compRR_min_gap
// is read as a double (the reference reads an int into the double), and the
// reference's "-gcge_compRR_tol    " carries four trailing spaces, kept here,
// so a plain -gcge_compRR_tol is ignored by both.  String values longer than
// the 7 characters of the solver's fields are cut.  The usage table the
// reference prints is not printed.
void EigenSolverSetParametersFromCommandLine_GCG(int argc, char *argv[], OPS *ops) {
    SolverCtx *c = ctx_for(ops, false);
    if (!c || !ops->GetOptionFromCommandLine) {
        set_error(GCGE_ERR_ARG,
                  "EigenSolverSetParametersFromCommandLine_GCG before EigenSolverSetup_GCG");
        return;
    }
    GCGSolver &g = c->pub;
    auto opt = [&](const char *name, char type, void *v) {
        ops->GetOptionFromCommandLine(name, type, v, argc, argv, ops);
    };
    auto opt_s = [&](const char *name, char *dst) {
        char buf[256] = {0};
        if (ops->GetOptionFromCommandLine(name, 's', buf, argc, argv, ops)) {
            std::strncpy(dst, buf, 7);
            dst[7] = 0;
        }
    };
    opt("-gcge_min_gap", 'f', &g.gapMin);
    opt("-gcge_given_nevec", 'i', &g.nevGiven);
    opt("-gcge_max_niter", 'i', &g.numIterMax);
    opt("-gcge_abs_tol", 'f', &g.tol[0]);
    opt("-gcge_rel_tol", 'f', &g.tol[1]);
    opt("-gcge_user_defined_multi_lin_sol", 'i', &g.user_defined_multi_linear_solver);
    opt_s("-gcge_initX_orth_method", g.initX_orth_method);
    opt("-gcge_initX_orth_block_size", 'i', &g.initX_orth_block_size);
    opt("-gcge_initX_orth_max_reorth", 'i', &g.initX_orth_max_reorth);
    opt("-gcge_initX_orth_zero_tol", 'f', &g.initX_orth_zero_tol);
    opt("-gcge_check_conv_max_num", 'i', &g.check_conv_max_num);
    opt_s("-gcge_compP_orth_method", g.compP_orth_method);
    opt("-gcge_compP_orth_block_size", 'i', &g.compP_orth_block_size);
    opt("-gcge_compP_orth_max_reorth", 'i', &g.compP_orth_max_reorth);
    opt("-gcge_compP_orth_zero_tol", 'f', &g.compP_orth_zero_tol);
    opt_s("-gcge_compW_orth_method", g.compW_orth_method);
    opt("-gcge_compW_orth_block_size", 'i', &g.compW_orth_block_size);
    opt("-gcge_compW_orth_max_reorth", 'i', &g.compW_orth_max_reorth);
    opt("-gcge_compW_orth_zero_tol", 'f', &g.compW_orth_zero_tol);
    opt("-gcge_compW_cg_max_iter", 'i', &g.compW_cg_max_iter);
    opt("-gcge_compW_cg_rate", 'f', &g.compW_cg_rate);
    opt("-gcge_compW_cg_tol", 'f', &g.compW_cg_tol);
    opt_s("-gcge_compW_cg_tol_type", g.compW_cg_tol_type);
    opt("-gcge_compW_cg_auto_shift", 'i', &g.compW_cg_auto_shift);
    opt("-gcge_compW_cg_shift", 'f', &g.compW_cg_shift);
    opt("-gcge_compW_cg_order", 'i', &g.compW_cg_order);
    opt("-gcge_compRR_min_num", 'i', &g.compRR_min_num);
    opt("-gcge_compRR_min_gap", 'f', &g.compRR_min_gap);
    opt("-gcge_compRR_tol    ", 'f', &g.compRR_tol);
}

void GCGE_Setparameters(double gapMin, int shift, OPS *ops) {
    // parameter set of src/ops_eig_sol_gcg.c:1878-1913
    const double eps = 2.220446049250313e-16;
    EigenSolverSetParameters_GCG(50, "mgs", -1, 2, 2 * eps, "mgs", -1, 2, 2 * eps, "mgs", -1, 2,
                                 2 * eps, 30, 1e-2, 1e-14, "abs", shift, -1, gapMin, 2 * eps, ops);
}

void GCGE_Create(void *A, int nevMax, int block_size, int nevInit, void ***gcg_mv_ws,
                 double *dbl_ws, int *int_ws, OPS *ops) {
    (void)nevInit;
    (void)dbl_ws;
    (void)int_ws;
    ops->MultiVecCreateByMat(&gcg_mv_ws[0], nevMax + 2 * block_size, A, ops);
    ops->MultiVecSetRandomValue(gcg_mv_ws[0], 0, nevMax + 2 * block_size, ops);
    for (int i = 1; i < 4; ++i) {
        ops->MultiVecCreateByMat(&gcg_mv_ws[i], block_size, A, ops);
        ops->MultiVecSetRandomValue(gcg_mv_ws[i], 0, block_size, ops);
    }
}
void GCGE_Destroymvws(void ***gcg_mv_ws, double *dbl_ws, int *int_ws, int nevMax, int block_size,
                      OPS *ops) {
    ops->MultiVecDestroy(&gcg_mv_ws[0], nevMax + 2 * block_size, ops);
    for (int i = 1; i < 4; ++i) ops->MultiVecDestroy(&gcg_mv_ws[i], block_size, ops);
    free(dbl_ws);
    free(int_ws);
}
void EigenSolverCreateWorkspace_GCG(int nevInit, int nevMax, int block_size, void *mat,
                                    void ***mv_ws, double **dbl_ws, int **int_ws, OPS *ops) {
    GCGE_Create(mat, nevMax, block_size, nevInit, mv_ws, nullptr, nullptr, ops);
    const int sizeV = nevInit + 2 * block_size;
    const size_t ld = (size_t)2 * sizeV * sizeV + 10 * sizeV + (nevMax + 2 * block_size) +
                      (size_t)nevMax * block_size;
    const size_t li = (size_t)6 * sizeV + 2 * (block_size + 3);
    if (dbl_ws) *dbl_ws = (double *)calloc(ld, sizeof(double));
    if (int_ws) *int_ws = (int *)calloc(li, sizeof(int));
}
void EigenSolverDestroyWorkspace_GCG(int nevInit, int nevMax, int block_size, void *mat,
                                     void ***mv_ws, double **dbl_ws, int **int_ws, OPS *ops) {
    (void)nevInit;
    (void)mat;
    ops->MultiVecDestroy(&mv_ws[0], nevMax + 2 * block_size, ops);
    for (int i = 1; i < 4; ++i) ops->MultiVecDestroy(&mv_ws[i], block_size, ops);
    if (dbl_ws) {
        free(*dbl_ws);
        *dbl_ws = nullptr;
    }
    if (int_ws) {
        free(*int_ws);
        *int_ws = nullptr;
    }
}

int GCGE_SetPrecision(OPS *ops, int precision) {
    if (precision != GCGE_PREC_FP64 && precision != GCGE_PREC_MIXED) return GCGE_ERR_ARG;
    SolverCtx *c = ctx_for(ops, false);
    if (!c) return GCGE_ERR_ARG;
    c->precision = precision;
    return GCGE_OK;
}
int GCGE_GetSolveInfo(OPS *ops, gcge_solve_info *info) {
    SolverCtx *c = ctx_for(ops, false);
    if (!c || !info) return GCGE_ERR_ARG;
    *info = c->info;
    return GCGE_OK;
}

// ---------------------------------------------------------------- one-call solve
struct gcge_prepared {
    OPS *ops = nullptr;
    void *A = nullptr, *B = nullptr;
    void **evec = nullptr, **x0 = nullptr;
    void **mv_ws[4] = {nullptr, nullptr, nullptr, nullptr};
    int n = 0, nev = 0, bs = 0, nev_init = 0, nev_max = 0, nev_given = 0;
};

static void prepared_free(gcge_prepared *p) {
    if (!p) return;
    if (p->ops) {
        if (p->mv_ws[0]) GCGE_Destroymvws(p->mv_ws, nullptr, nullptr, p->nev_max, p->bs, p->ops);
        if (p->evec) p->ops->MultiVecDestroy(&p->evec, p->nev_max, p->ops);
        if (p->x0) p->ops->MultiVecDestroy(&p->x0, std::max(p->nev_given, 1), p->ops);
        OPS_Destroy(&p->ops);
    }
    CUDA_MatDestroy(&p->A);
    CUDA_MatDestroy(&p->B);
    delete p;
}

int GCGE_Prepare(gcge_prepared **prep, int n, const int *a_colptr, const int *a_rowind,
                 const double *a_val, const int *b_colptr, const int *b_rowind,
                 const double *b_val, int nev, int block_size, int nev_init, int nev_max,
                 int max_iter, const double tol[2], double gap_min, int auto_shift, int precision,
                 const double *X0, int nev_given) {
    if (!prep || n <= 0 || nev <= 0 || block_size <= 0 || nev_init <= 0 || nev_max < nev_init ||
        nev_given < 0 || nev_given > nev_init || (nev_given > 0 && !X0))
        return GCGE_ERR_ARG;
    take_error();
    gcge_prepared *p = new gcge_prepared();
    p->n = n;
    p->nev = nev;
    p->bs = block_size;
    p->nev_init = nev_init;
    p->nev_max = nev_max;
    p->nev_given = nev_given;
    int st = CUDA_MatCreateFromCCS(&p->A, n, n, a_colptr, a_rowind, a_val);
    if (st == GCGE_OK && b_colptr) st = CUDA_MatCreateFromCCS(&p->B, n, n, b_colptr, b_rowind, b_val);
    if (st != GCGE_OK) {
        prepared_free(p);
        return st;
    }
    OPS_Create(&p->ops);
    OPS_CUDA_Set(p->ops);
    OPS_Setup(p->ops);
    p->ops->MultiVecCreateByMat(&p->evec, nev_max, p->A, p->ops);
    p->ops->MultiVecCreateByMat(&p->x0, std::max(nev_given, 1), p->A, p->ops);
    if (nev_given > 0) CUDA_MultiVecSetFromHost(p->x0, 0, nev_given, X0, n);
    GCGE_Create(p->A, nev_max, block_size, nev_init, p->mv_ws, nullptr, nullptr, p->ops);
    double t[2] = {tol[0], tol[1]};
    const int dbg = getenv("GCGE_CUDA_PRINT") ? atoi(getenv("GCGE_CUDA_PRINT")) : 0;
    EigenSolverSetup_GCG(gap_min, nev_init, nev_max, block_size, t, max_iter, dbg > 0, dbg > 1, 0,
                         p->mv_ws, nullptr, nullptr, p->ops);
    GCGE_Setparameters(gap_min, auto_shift, p->ops);
    GCGE_SetPrecision(p->ops, precision);
    st = take_error();
    if (st != GCGE_OK) {
        prepared_free(p);
        return st;
    }
    *prep = p;
    return GCGE_OK;
}

int GCGE_PreparedSolve(gcge_prepared *p, double *eval, double *evec, gcge_solve_info *info) {
    if (!p || !eval) return GCGE_ERR_ARG;
    take_error();
    try {
        MultiVec *E = as_mv(p->evec), *X = as_mv(p->x0);
        cudaStream_t st = lib_stream();
        GCGE_CUDA(cudaMemsetAsync(E->data, 0, sizeof(double) * E->ld * E->ncols, st));
        if (p->nev_given > 0) copy_cols(p->n, p->nev_given, X->data, X->ld, E->data, E->ld, st);
    } catch (const CudaError &e) {
        return e.status;
    }
    int nconv = p->nev;
    p->ops->EigenSolver(p->A, p->B, eval, p->evec, p->nev_given, &nconv, p->ops);
    int st = take_error();
    gcge_solve_info inf{};
    GCGE_GetSolveInfo(p->ops, &inf);
    if (info) *info = inf;
    if (st != GCGE_OK) return st;
    if (evec) {
        st = CUDA_MultiVecGetToHost(p->evec, 0, p->nev_max, evec, p->n);
        if (st != GCGE_OK) return st;
    }
    return inf.status;
}

void GCGE_PreparedDestroy(gcge_prepared **prep) {
    if (!prep || !*prep) return;
    prepared_free(*prep);
    *prep = nullptr;
}

int GCGE_Solve(int n, const int *a_colptr, const int *a_rowind, const double *a_val,
               const int *b_colptr, const int *b_rowind, const double *b_val, int nev,
               int block_size, int nev_init, int nev_max, int max_iter, const double tol[2],
               double gap_min, int auto_shift, int precision, const double *X0, int nev_given,
               double *eval, double *evec, gcge_solve_info *info) {
    gcge_prepared *p = nullptr;
    int st = GCGE_Prepare(&p, n, a_colptr, a_rowind, a_val, b_colptr, b_rowind, b_val, nev,
                          block_size, nev_init, nev_max, max_iter, tol, gap_min, auto_shift,
                          precision, X0, nev_given);
    if (st != GCGE_OK) return st;
    st = GCGE_PreparedSolve(p, eval, evec, info);
    GCGE_PreparedDestroy(&p);
    return st;
}

void *GCGE_HostAlloc(size_t bytes) {
    void *p = nullptr;
    const cudaError_t e = cudaMallocHost(&p, std::max<size_t>(bytes, 1));
    if (e != cudaSuccess) {
        set_error(GCGE_ERR_ALLOC, "GCGE_HostAlloc: cudaMallocHost failed");
        return nullptr;
    }
    return p;
}
void GCGE_HostFree(void *p) {
    if (p) cudaFreeHost(p);
}

static thread_local cudaEvent_t g_t0 = nullptr, g_t1 = nullptr;
int GCGE_TimerStart(void) {
    GCGE_TRY_RET({
        if (!g_t0) {
            GCGE_CUDA(cudaEventCreate(&g_t0));
            GCGE_CUDA(cudaEventCreate(&g_t1));
        }
        GCGE_CUDA(cudaEventRecord(g_t0, lib_stream()));
    });
}
double GCGE_TimerStop(void) {
    try {
        GCGE_REQUIRE(g_t0 != nullptr, GCGE_ERR_ARG, "GCGE_TimerStop without GCGE_TimerStart");
        GCGE_CUDA(cudaEventRecord(g_t1, lib_stream()));
        GCGE_CUDA(cudaEventSynchronize(g_t1));
        float ms = 0.f;
        GCGE_CUDA(cudaEventElapsedTime(&ms, g_t0, g_t1));
        return ms;
    } catch (const CudaError &e) {
        set_error(e.status, e.where.c_str());
        return -1.0;
    }
}

// Device operands of the SpMM measurements: k seeded uniform columns (and
// their FP32 copy with the matrix's FP32 values when fp32), Y of the same
// shape, all owned by the call.
struct SpmmOperands {
    int n = 0, ld = 0;
    DevBuf<double> X, Y, tmp;
    DevBuf<float> X32, Y32, V32;
    SpmmOperands(const SparseMat *A, int k, bool fp32, cudaStream_t st) {
        n = A->n;
        ld = (n + 31) / 32 * 32;
        X.alloc((size_t)ld * k);
        fill_uniform(n, k, X.p, ld, 12345, st);
        if (fp32) {
            X32.alloc((size_t)ld * k);
            Y32.alloc((size_t)ld * k);
            V32.alloc(std::max<size_t>(A->pat.padded, 1));
            copy_f64_to_f32(n, k, X.p, ld, X32.p, ld, st);
            tmp.alloc(std::max<size_t>(A->pat.padded, 1));
            GCGE_CUDA(cudaMemsetAsync(tmp.p, 0, sizeof(double) * A->pat.padded, st));
            shift_values(A->pat.padded, A->val.p, tmp.p, 0.0, nullptr, V32.p, st);
        } else {
            Y.alloc((size_t)ld * k);
        }
    }
};

int GCGE_SetSpMMTuning(int on) {
    set_spmm_tuning(on > 0);
    if (on < 0) clear_spmm_tuning();
    return GCGE_OK;
}

int GCGE_SpMMTuneCandidates(int k, int *chunks, int cap, int *count) {
    if (k < 1 || count == nullptr || (cap > 0 && chunks == nullptr)) {
        set_error(GCGE_ERR_ARG, "GCGE_SpMMTuneCandidates: k < 1 or null output");
        return GCGE_ERR_ARG;
    }
    const std::vector<int> p = spmm_split_candidates(k);
    *count = (int)p.size();
    for (int i = 0; i < (int)p.size() && i < cap; ++i) chunks[i] = (k + p[i] - 1) / p[i];
    return GCGE_OK;
}

int GCGE_SpMMTune(void *mat, int k, int fp32, int *chunk, double *ms, int cap, int *count) {
    GCGE_TRY_RET({
        SparseMat *A = as_mat(mat);
        GCGE_REQUIRE(A != nullptr, GCGE_ERR_HANDLE, "GCGE_SpMMTune: not a CUDA matrix");
        GCGE_REQUIRE(k >= 1 && chunk != nullptr && count != nullptr && (cap <= 0 || ms != nullptr),
                     GCGE_ERR_ARG, "GCGE_SpMMTune: k < 1 or null output");
        cudaStream_t st = lib_stream();
        SpmmOperands o(A, k, fp32 != 0, st);
        std::vector<double> t;
        const int p = fp32 ? spmm_tuned_split<float>(A->pat, o.V32.p, o.X32.p, o.ld, o.Y32.p,
                                                      o.ld, k, st, &t)
                           : spmm_tuned_split<double>(A->pat, A->val.p, o.X.p, o.ld, o.Y.p,
                                                       o.ld, k, st, &t);
        *chunk = (k + p - 1) / p;
        *count = (int)t.size();
        for (int i = 0; i < (int)t.size() && i < cap; ++i) ms[i] = t[i];
        GCGE_CUDA(cudaStreamSynchronize(st));
    });
}

int GCGE_BenchSpMM(void *mat, int k, int fp32, int reps, double *ms_per_launch,
                   double *bytes_per_launch) {
    GCGE_TRY_RET({
        SparseMat *A = as_mat(mat);
        GCGE_REQUIRE(A != nullptr, GCGE_ERR_HANDLE, "GCGE_BenchSpMM: not a CUDA matrix");
        GCGE_REQUIRE(k >= 1 && reps >= 1, GCGE_ERR_ARG, "GCGE_BenchSpMM: k, reps");
        cudaStream_t st = lib_stream();
        const int vs = fp32 ? 4 : 8;
        SpmmOperands o(A, k, fp32 != 0, st);
        const int n = o.n, ld = o.ld;
        DevBuf<double> &X = o.X, &Y = o.Y;
        DevBuf<float> &X32 = o.X32, &Y32 = o.Y32, &V32 = o.V32;
        // warm-up (with tuning on, the first call picks the column split)
        for (int r = 0; r < 3; ++r) {
            if (fp32) spmm<float>(A->pat, V32.p, X32.p, ld, Y32.p, ld, k, st);
            else spmm<double>(A->pat, A->val.p, X.p, ld, Y.p, ld, k, st);
        }
        cudaEvent_t e0, e1;
        GCGE_CUDA(cudaEventCreate(&e0));
        GCGE_CUDA(cudaEventCreate(&e1));
        GCGE_CUDA(cudaEventRecord(e0, st));
        for (int r = 0; r < reps; ++r) {
            if (fp32) spmm<float>(A->pat, V32.p, X32.p, ld, Y32.p, ld, k, st);
            else spmm<double>(A->pat, A->val.p, X.p, ld, Y.p, ld, k, st);
        }
        GCGE_CUDA(cudaEventRecord(e1, st));
        GCGE_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        *ms_per_launch = ms / reps;
        *bytes_per_launch = (double)A->nnz * (vs + 4) + 4.0 * (n + 1) + 2.0 * n * k * vs;
    });
}

}  // extern "C"
