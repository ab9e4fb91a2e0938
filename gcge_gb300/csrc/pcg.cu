// Block conjugate gradient on (A + sigma B) x = b for all columns of a block
// at once (reference BlockPCG, src/ops_lin_sol.c:140-437).
//
// The reference keeps a compacted list of unconverged columns and runs one
// SpMM per contiguous run of them; here every kernel covers the whole block
// and a per-column `active` flag plays the role of the list: inactive columns
// skip their loads, FMAs and updates.  The per-column scalars (rho, p^T w,
// alpha, beta, residual norms) stay on the device; reductions are two-stage
// with a fixed summation order, so results are deterministic.  The shifted
// operator is one SELL matrix S = A + sigma B on the union pattern of A and B
// (the reference's in-place MatAxpby branch, src/ops_eig_sol_gcg.c:600-608),
// so each iteration streams one matrix.  T = double (FP64 GCG) or float
// (mixed precision: FP32 values, FP32 SpMM accumulation; dots in double).
#include <algorithm>

#include "common.cuh"
#include "pcg.cuh"

namespace gcge {

template <typename T>
__global__ void k_colsq(int n, int k, const T *__restrict__ R, int ld, double *__restrict__ part,
                        int kmax, int rows_per_chunk) {
    __shared__ double red[8];
    const int c = blockIdx.y;
    const int r0 = blockIdx.x * rows_per_chunk, r1 = min(n, r0 + rows_per_chunk);
    T s = T(0);
    for (int i = r0 + threadIdx.x; i < r1; i += 256) {
        const T v = R[i + (size_t)c * ld];
        s = fma(v, v, s);
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = (double)s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int i = 0; i < 8; ++i) t += red[i];
        part[(size_t)blockIdx.x * kmax + c] = t;
    }
}

// Deterministic column sums of partials: warp c sums column c.
__device__ inline double sum_partials(const double *part, int nblocks, int kmax, int c, int lane) {
    double s = 0.0;
    for (int b = lane; b < nblocks; b += 32) s += part[(size_t)b * kmax + c];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    return s;
}

// initial residual norms -> init_res, rho2, active, count
__global__ void k_pcg_init(int k, const double *__restrict__ part, int nblocks, int kmax,
                           PcgScalars *sc, double tol) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int c = warp; c < k; c += blockDim.x / 32) {
        const double rr = sum_partials(part, nblocks, kmax, c, lane);
        if (lane == 0) {
            sc->rho2[c] = rr;
            sc->init_res[c] = sqrt(rr);
            sc->last_res[c] = sqrt(rr);
            sc->active[c] = sqrt(rr) > tol * sc->norm_b[c] ? 1 : 0;
            sc->beta[c] = 0.0;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int cnt = 0;
        for (int c = 0; c < k; ++c) cnt += sc->active[c];
        sc->nactive = cnt;
        sc->niter = 0;
    }
}

__global__ void k_pcg_normb(int k, const double *__restrict__ part, int nblocks, int kmax,
                            PcgScalars *sc) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int c = warp; c < k; c += blockDim.x / 32) {
        const double bb = sum_partials(part, nblocks, kmax, c, lane);
        if (lane == 0) sc->norm_b[c] = sqrt(bb);
    }
}

template <typename T>
__global__ void k_pcg_p(int n, int k, const T *__restrict__ R, T *__restrict__ P, int ld,
                        const PcgScalars *__restrict__ sc) {
    const size_t total = (size_t)n * k;
    const bool first = sc->niter == 0;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
         t += (size_t)gridDim.x * blockDim.x) {
        const int c = (int)(t / n), i = (int)(t % n);
        if (!sc->active[c]) continue;
        const size_t o = i + (size_t)c * ld;
        P[o] = first ? R[o] : fma((T)sc->beta[c], P[o], R[o]);
    }
}

__global__ void k_pcg_alpha(int k, const double *__restrict__ part, int nblocks, int kmax,
                            PcgScalars *sc) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int c = warp; c < k; c += blockDim.x / 32) {
        const double ptw = sum_partials(part, nblocks, kmax, c, lane);
        if (lane == 0) {
            sc->ptw[c] = ptw;
            sc->rho1[c] = sc->rho2[c];
            sc->alpha[c] = sc->active[c] ? sc->rho2[c] / ptw : 0.0;
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(256)
k_pcg_xr(int n, int k, T *__restrict__ X, int ldx, T *__restrict__ R, const T *__restrict__ P,
         const T *__restrict__ W, int ld, const PcgScalars *__restrict__ sc,
         double *__restrict__ part, int kmax, int rows_per_chunk) {
    __shared__ double red[8];
    const int c = blockIdx.y;
    const int r0 = blockIdx.x * rows_per_chunk, r1 = min(n, r0 + rows_per_chunk);
    T s = T(0);
    if (sc->active[c]) {
        const T a = (T)sc->alpha[c];
        for (int i = r0 + threadIdx.x; i < r1; i += 256) {
            const size_t o = i + (size_t)c * ld;
            X[i + (size_t)c * ldx] = fma(a, P[o], X[i + (size_t)c * ldx]);
            const T rn = fma(-a, W[o], R[o]);
            R[o] = rn;
            s = fma(rn, rn, s);
        }
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = (double)s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int i = 0; i < 8; ++i) t += red[i];
        part[(size_t)blockIdx.x * kmax + c] = t;
    }
}

// convergence test of src/ops_lin_sol.c:383-394 and beta for the next step
__global__ void k_pcg_conv(int k, const double *__restrict__ part, int nblocks, int kmax,
                           PcgScalars *sc, double rate, double tol) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int c = warp; c < k; c += blockDim.x / 32) {
        const double rr = sum_partials(part, nblocks, kmax, c, lane);
        if (lane == 0 && sc->active[c]) {
            sc->rho2[c] = rr;
            const double res = sqrt(rr);
            sc->last_res[c] = res;
            sc->beta[c] = rr / sc->rho1[c];
            if (!(res > rate * sc->init_res[c] && res > tol * sc->norm_b[c])) sc->active[c] = 0;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int cnt = 0;
        for (int c = 0; c < k; ++c) cnt += sc->active[c];
        sc->nactive = cnt;
        sc->niter += 1;
    }
}

static int chunks_for(int n, int k) {
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return std::max(1, std::min((n + 1023) / 1024, (4 * sms + k - 1) / k));
}

void PcgWork::timing_reset() {
    ev_used = 0;
    spmm_bytes = 0.0;
    spmm_launches = 0;
}
double PcgWork::timing_collect_ms() {
    double ms = 0.0;
    for (size_t i = 0; i + 1 < ev_used; i += 2) {
        float t = 0.f;
        if (cudaEventSynchronize(ev[i + 1]) == cudaSuccess &&
            cudaEventElapsedTime(&t, ev[i], ev[i + 1]) == cudaSuccess)
            ms += t;
    }
    return ms;
}
PcgWork::~PcgWork() {
    for (auto e : ev) cudaEventDestroy(e);
}

void PcgWork::reserve(int n, int kmax_, int spmm_nblocks) {
    kmax = kmax_;
    const size_t need = std::max((size_t)spmm_nblocks, (size_t)chunks_for(n, 1)) * kmax;
    part.alloc(std::max<size_t>(need, 1));
    sc.alloc(1);
    h_sc.alloc(1);
}

template <typename T>
int block_pcg(PcgWork &wk, const SellPattern &pat, const T *sval, const T *Bv, int ldb, T *X,
              int ldx, T *R, T *P, T *W, int ld, int k, int max_iter, double rate, double tol,
              bool rel_tol, cudaStream_t st) {
    GCGE_REQUIRE(k >= 1 && k <= wk.kmax, GCGE_ERR_ARG, "block_pcg: block too wide");
    const int n = pat.n;
    // norm_b (abs: 1; rel: ||b||), src/ops_lin_sol.c:171-197
    PcgScalars hs;
    std::fill(hs.norm_b, hs.norm_b + kPcgMaxCols, 1.0);
    GCGE_CUDA(cudaMemcpyAsync(&wk.sc.p->norm_b[0], hs.norm_b, sizeof(double) * kPcgMaxCols,
                              cudaMemcpyHostToDevice, st));
    const int chunks = chunks_for(n, k);
    const int rpc = (n + chunks - 1) / chunks;
    const dim3 cgrid(chunks, k);
    if (rel_tol) {
        k_colsq<T><<<cgrid, 256, 0, st>>>(n, k, Bv, ldb, wk.part.p, wk.kmax, rpc);
        GCGE_CHECK_LAUNCH();
        k_pcg_normb<<<1, 1024, 0, st>>>(k, wk.part.p, chunks, wk.kmax, wk.sc.p);
        GCGE_CHECK_LAUNCH();
        count_launch(2);
    }
    // r = b - S x  (src/ops_lin_sol.c:202-221)
    spmm<T>(pat, sval, X, ldx, R, ld, k, st);
    if constexpr (sizeof(T) == 8)
        axpby(n, k, 1.0, (const double *)Bv, ldb, -1.0, (double *)R, ld, st);
    else
        axpby_f32(n, k, 1.0f, (const float *)Bv, ldb, -1.0f, (float *)R, ld, st);
    k_colsq<T><<<cgrid, 256, 0, st>>>(n, k, R, ld, wk.part.p, wk.kmax, rpc);
    GCGE_CHECK_LAUNCH();
    k_pcg_init<<<1, 1024, 0, st>>>(k, wk.part.p, chunks, wk.kmax, wk.sc.p, tol);
    GCGE_CHECK_LAUNCH();
    count_launch(2);
    int it = 0;
    const int pgrid = std::max(1, std::min((int)(((size_t)n * k + 255) / 256), 2048));
    for (it = 0; it < max_iter; ++it) {
        GCGE_CUDA(cudaMemcpyAsync(&wk.h_sc.p->nactive, &wk.sc.p->nactive, sizeof(int),
                                  cudaMemcpyDeviceToHost, st));
        GCGE_CUDA(cudaStreamSynchronize(st));
        if (wk.h_sc.p->nactive == 0) break;
        k_pcg_p<T><<<pgrid, 256, 0, st>>>(n, k, R, P, ld, wk.sc.p);
        GCGE_CHECK_LAUNCH();
        const bool timed = wk.ev_used + 2 <= 65536;
        if (timed) {
            while (wk.ev.size() < wk.ev_used + 2) {
                cudaEvent_t e;
                GCGE_CUDA(cudaEventCreate(&e));
                wk.ev.push_back(e);
            }
            GCGE_CUDA(cudaEventRecord(wk.ev[wk.ev_used], st));
        }
        const int nb = spmm_dot<T>(pat, sval, P, ld, W, ld, k, &wk.sc.p->active[0], wk.part.p,
                                   wk.kmax, st);
        if (timed) {
            GCGE_CUDA(cudaEventRecord(wk.ev[wk.ev_used + 1], st));
            wk.ev_used += 2;
        }
        // algorithmic bytes: matrix once, active columns of p read once, of w written once
        wk.spmm_bytes += (double)pat.nnz * (sizeof(T) + 4) + 4.0 * (n + 1) +
                         2.0 * n * wk.h_sc.p->nactive * sizeof(T);
        wk.spmm_launches++;
        k_pcg_alpha<<<1, 1024, 0, st>>>(k, wk.part.p, nb, wk.kmax, wk.sc.p);
        GCGE_CHECK_LAUNCH();
        k_pcg_xr<T><<<cgrid, 256, 0, st>>>(n, k, X, ldx, R, P, W, ld, wk.sc.p, wk.part.p, wk.kmax,
                                           rpc);
        GCGE_CHECK_LAUNCH();
        k_pcg_conv<<<1, 1024, 0, st>>>(k, wk.part.p, chunks, wk.kmax, wk.sc.p, rate, tol);
        GCGE_CHECK_LAUNCH();
        count_launch(4);
    }
    return it;
}

template int block_pcg<double>(PcgWork &, const SellPattern &, const double *, const double *, int,
                               double *, int, double *, double *, double *, int, int, int, double,
                               double, bool, cudaStream_t);
template int block_pcg<float>(PcgWork &, const SellPattern &, const float *, const float *, int,
                              float *, int, float *, float *, float *, int, int, int, double, double,
                              bool, cudaStream_t);

}  // namespace gcge
