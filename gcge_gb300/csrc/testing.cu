// Component entry points: the dense eigensolver, the block-PCG inner solve,
// the B-orthonormalisation and the long-dimension dense products, each
// callable on its own through the C ABI so they can be checked against the
// CPU oracle (or FP64 host arithmetic) in isolation.
#include <cstring>

#include "gcg.cuh"

using namespace gcge;

extern "C" {

int GCGE_DenseEig(int s, const double *M, int ldm, double *eval, double *Z, int ldz) {
    try {
        GCGE_REQUIRE(s >= 1 && M && eval && Z && ldm >= s && ldz >= s, GCGE_ERR_ARG,
                     "GCGE_DenseEig: arguments");
        cudaStream_t st = lib_stream();
        EigWork wk;
        wk.reserve(s);
        DevBuf<double> dM, dZ;
        dM.alloc((size_t)s * s);
        dZ.alloc((size_t)s * s);
        GCGE_CUDA(cudaMemcpy2DAsync(dM.p, sizeof(double) * s, M, sizeof(double) * ldm,
                                    sizeof(double) * s, s, cudaMemcpyHostToDevice, st));
        sym_eig(wk, s, dM.p, s, eval, dZ.p, s, 8, st);
        GCGE_CUDA(cudaMemcpy2DAsync(Z, sizeof(double) * ldz, dZ.p, sizeof(double) * s,
                                    sizeof(double) * s, s, cudaMemcpyDeviceToHost, st));
        GCGE_CUDA(cudaStreamSynchronize(st));
        return GCGE_OK;
    } catch (const CudaError &e) {
        set_error(e.status, e.where.c_str());
        take_error();
        return e.status;
    }
}

int GCGE_BlockPCG(void *A, void *B, double sigma, void **b, void **x, int k, int max_iter,
                  double rate, double tol, int fp32, int *iters) {
    try {
        SparseMat *Am = as_mat(A);
        SparseMat *Bm = B ? as_mat(B) : nullptr;
        MultiVec *bv = as_mv(b), *xv = as_mv(x);
        GCGE_REQUIRE(Am && (!B || Bm) && bv && xv, GCGE_ERR_HANDLE, "GCGE_BlockPCG: handles");
        GCGE_REQUIRE(k >= 1 && k <= 40 && k <= bv->ncols && k <= xv->ncols, GCGE_ERR_ARG,
                     "GCGE_BlockPCG: k");
        cudaStream_t st = lib_stream();
        SolverCtx c;
        prepare_union(c, Am, Bm, st);
        c.reserve(Am->n, k, k, k, spmm_blocks(c.upat));
        shift_values(c.upat.padded, c.ua.p, c.ub.p, sigma, fp32 ? nullptr : c.us64.p,
                     fp32 ? c.us32.p : nullptr, st);
        const int n = Am->n;
        int it = 0;
        if (!fp32) {
            const int kp = rows_width(k, 8);
            col_to_rows<double, double>(n, k, kp, xv->data, xv->ld, c.xr64.p, st);
            col_to_rows<double, double>(n, k, kp, bv->data, bv->ld, c.br64.p, st);
            block_pcg_rows<double>(c.pcg, c.upat, c.us64.p, c.br64.p, c.xr64.p, c.rr64.p,
                                   c.pr64.p, c.wr64.p, kp, k, max_iter, rate, tol, false, false,
                                   st);
            it = pcg_last_iters(c.pcg, st);
            rows_to_col<double, double>(n, k, kp, c.xr64.p, xv->data, xv->ld, false, st);
        } else {
            const int kp = rows_width(k, 4);
            DevBuf<float> x32, b32, r32, p32, w32;
            for (auto *bb : {&x32, &b32, &r32, &p32, &w32}) bb->alloc(pcg_block_elems(n, kp));
            col_to_rows<double, float>(n, k, kp, xv->data, xv->ld, x32.p, st);
            col_to_rows<double, float>(n, k, kp, bv->data, bv->ld, b32.p, st);
            block_pcg_rows<float>(c.pcg, c.upat, c.us32.p, b32.p, x32.p, r32.p, p32.p, w32.p,
                                  kp, k, max_iter, rate, tol, false, false, st);
            it = pcg_last_iters(c.pcg, st);
            rows_to_col<float, double>(n, k, kp, x32.p, xv->data, xv->ld, false, st);
        }
        GCGE_CUDA(cudaStreamSynchronize(st));
        if (iters) *iters = it;
        return GCGE_OK;
    } catch (const CudaError &e) {
        set_error(e.status, e.where.c_str());
        take_error();
        return e.status;
    }
}

int GCGE_TestBlockPCGBarrierTimeout(void *A, void **b, void **x, int k, double timeout_ms) {
    if (!(timeout_ms > 0.0)) return GCGE_ERR_ARG;
    struct Hook {
        explicit Hook(double ms) {
            t_pcg_barrier_test.active = true;
            t_pcg_barrier_test.timeout_ns = (unsigned long long)(ms * 1e6);
            t_pcg_barrier_test.withhold_last = 1;
        }
        ~Hook() { t_pcg_barrier_test = PcgBarrierTest{}; }
    } hook(timeout_ms);
    int it = 0;
    return GCGE_BlockPCG(A, nullptr, 0.0, b, x, k, 30, 1e-2, 1e-14, 0, &it);
}

int GCGE_BOrth(void *B, void **x, int start, int *end, double zero_tol, int max_reorth) {
    try {
        SparseMat *Bm = B ? as_mat(B) : nullptr;
        MultiVec *xv = as_mv(x);
        GCGE_REQUIRE((!B || Bm) && xv && end, GCGE_ERR_HANDLE, "GCGE_BOrth: handles");
        GCGE_REQUIRE(start >= 0 && *end >= start && *end <= xv->ncols, GCGE_ERR_ARG,
                     "GCGE_BOrth: range");
        SolverCtx c;
        c.reserve(xv->nrows, xv->ncols, xv->ncols, 1, 1);
        *end = borth(c, Bm, xv->data, xv->ld, xv->nrows, start, *end, Bm != nullptr, zero_tol,
                     max_reorth, nullptr);
        GCGE_CUDA(cudaStreamSynchronize(lib_stream()));
        return GCGE_OK;
    } catch (const CudaError &e) {
        set_error(e.status, e.where.c_str());
        take_error();
        return e.status;
    }
}


int GCGE_DenseGram(int n, int m, int w, const double *Q, int ldq, const double *P, int ldp,
                   double *C, int emulated) {
    try {
        GCGE_REQUIRE(n >= 0 && m >= 1 && w >= 1 && C && (n == 0 || (Q && P && ldq >= n && ldp >= n)),
                     GCGE_ERR_ARG, "GCGE_DenseGram: arguments");
        cudaStream_t st = lib_stream();
        DevBuf<double> dQ, dP, dC, scr;
        dQ.alloc(std::max<size_t>((size_t)n * m, 1));
        dP.alloc(std::max<size_t>((size_t)n * w, 1));
        dC.alloc((size_t)m * w);
        const size_t elems = std::max<size_t>(gram_scratch_elems(n, m, w), (size_t)1 << 20);
        scr.alloc(elems);
        if (n > 0) {
            GCGE_CUDA(cudaMemcpy2DAsync(dQ.p, sizeof(double) * n, Q, sizeof(double) * ldq,
                                        sizeof(double) * n, m, cudaMemcpyHostToDevice, st));
            GCGE_CUDA(cudaMemcpy2DAsync(dP.p, sizeof(double) * n, P, sizeof(double) * ldp,
                                        sizeof(double) * n, w, cudaMemcpyHostToDevice, st));
        }
        if (emulated)
            oz_gram(n, m, w, dQ.p, std::max(n, 1), dP.p, std::max(n, 1), dC.p, m, scr.p, elems, st);
        else
            gram(n, m, w, dQ.p, std::max(n, 1), dP.p, std::max(n, 1), dC.p, m, scr.p, elems, st);
        if (emulated && tc_digits_available()) tc_check_error(st);
        GCGE_CUDA(cudaMemcpyAsync(C, dC.p, sizeof(double) * m * w, cudaMemcpyDeviceToHost, st));
        GCGE_CUDA(cudaStreamSynchronize(st));
        return GCGE_OK;
    } catch (const CudaError &e) {
        set_error(e.status, e.where.c_str());
        take_error();
        return e.status;
    }
}

int GCGE_BenchDenseProduct(int kind, int n, int m, int w, int emulated, int reps,
                           double *ms_per_call) {
    try {
        GCGE_REQUIRE((kind == 0 || kind == 1) && n >= 1 && m >= 1 && w >= 1 && reps >= 1 &&
                         ms_per_call,
                     GCGE_ERR_ARG, "GCGE_BenchDenseProduct: arguments");
        cudaStream_t st = lib_stream();
        const int ld = (n + 31) / 32 * 32;
        DevBuf<double> dA, dB, dC, scr;
        DevBuf<unsigned char> ozb;
        dA.alloc((size_t)ld * m);
        fill_uniform(n, m, dA.p, ld, 11, st);
        if (kind == 0) {
            dB.alloc((size_t)ld * w);
            fill_uniform(n, w, dB.p, ld, 12, st);
            dC.alloc((size_t)m * w);
        } else {
            dB.alloc((size_t)m * w);
            fill_uniform(m, w, dB.p, m, 12, st);
            dC.alloc((size_t)ld * w);
            fill_uniform(n, w, dC.p, ld, 13, st);
            ozb.alloc(oz_lincomb_scratch_bytes(m, w));
        }
        const size_t elems = std::max<size_t>(gram_scratch_elems(n, m, w), (size_t)1 << 22);
        scr.alloc(elems);
        auto call = [&]() {
            if (kind == 0) {
                if (emulated) oz_gram(n, m, w, dA.p, ld, dB.p, ld, dC.p, m, scr.p, elems, st);
                else gram(n, m, w, dA.p, ld, dB.p, ld, dC.p, m, scr.p, elems, st);
            } else {
                if (emulated)
                    oz_lincomb(n, m, w, dA.p, ld, dB.p, m, dC.p, ld, nullptr, 0, st, 1.0, ozb.p,
                               ozb.n);
                else lincomb(n, m, w, dA.p, ld, dB.p, m, dC.p, ld, nullptr, 0, st, 1.0);
            }
        };
        call();
        cudaEvent_t e0, e1;
        GCGE_CUDA(cudaEventCreate(&e0));
        GCGE_CUDA(cudaEventCreate(&e1));
        GCGE_CUDA(cudaEventRecord(e0, st));
        for (int r = 0; r < reps; ++r) call();
        GCGE_CUDA(cudaEventRecord(e1, st));
        GCGE_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (emulated && tc_digits_available()) tc_check_error(st);
        *ms_per_call = ms / reps;
        return GCGE_OK;
    } catch (const CudaError &e) {
        set_error(e.status, e.where.c_str());
        take_error();
        return e.status;
    }
}

int GCGE_DenseLinComb(int n, int k, int m, const double *X, int ldx, const double *Cf, int ldc,
                      double *Y, int ldy, const double *beta, double alpha, int emulated) {
    try {
        GCGE_REQUIRE(n >= 1 && k >= 0 && m >= 1 && Y && ldy >= n &&
                         (k == 0 || (X && Cf && ldx >= n && ldc >= k)),
                     GCGE_ERR_ARG, "GCGE_DenseLinComb: arguments");
        cudaStream_t st = lib_stream();
        DevBuf<double> dX, dC, dY, dB;
        dX.alloc(std::max<size_t>((size_t)n * k, 1));
        dC.alloc(std::max<size_t>((size_t)k * m, 1));
        dY.alloc((size_t)n * m);
        if (k > 0) {
            GCGE_CUDA(cudaMemcpy2DAsync(dX.p, sizeof(double) * n, X, sizeof(double) * ldx,
                                        sizeof(double) * n, k, cudaMemcpyHostToDevice, st));
            GCGE_CUDA(cudaMemcpy2DAsync(dC.p, sizeof(double) * k, Cf, sizeof(double) * ldc,
                                        sizeof(double) * k, m, cudaMemcpyHostToDevice, st));
        }
        GCGE_CUDA(cudaMemcpy2DAsync(dY.p, sizeof(double) * n, Y, sizeof(double) * ldy,
                                    sizeof(double) * n, m, cudaMemcpyHostToDevice, st));
        const double *bp = nullptr;
        if (beta) {
            dB.alloc(m);
            GCGE_CUDA(cudaMemcpyAsync(dB.p, beta, sizeof(double) * m, cudaMemcpyHostToDevice, st));
            bp = dB.p;
        }
        DevBuf<unsigned char> ozb;
        if (emulated) {
            ozb.alloc(oz_lincomb_scratch_bytes(k, m));
            oz_lincomb(n, k, m, dX.p, n, dC.p, std::max(k, 1), dY.p, n, bp, 1, st, alpha, ozb.p,
                       ozb.n);
            if (tc_digits_available()) tc_check_error(st);
        } else
            lincomb(n, k, m, dX.p, n, dC.p, std::max(k, 1), dY.p, n, bp, 1, st, alpha);
        GCGE_CUDA(cudaMemcpy2DAsync(Y, sizeof(double) * ldy, dY.p, sizeof(double) * n,
                                    sizeof(double) * n, m, cudaMemcpyDeviceToHost, st));
        GCGE_CUDA(cudaStreamSynchronize(st));
        return GCGE_OK;
    } catch (const CudaError &e) {
        set_error(e.status, e.where.c_str());
        take_error();
        return e.status;
    }
}

}  // extern "C"
