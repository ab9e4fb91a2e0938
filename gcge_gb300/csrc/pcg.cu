// Block conjugate gradient on (A + sigma B) x = b for all columns of a block
// at once (reference BlockPCG, src/ops_lin_sol.c:140-437).
//
// The reference keeps a compacted list of unconverged columns and runs one
// SpMM per contiguous run of them; here every kernel covers the whole block
// and a per-column `active` flag plays the role of the list: inactive columns
// keep their x and r (alpha = 0) and drop out of the reductions.  The
// per-column scalars (rho, p^T w, alpha, beta, residual norms) stay on the
// device; reductions are two-stage with a fixed summation order, so results
// are deterministic.  The shifted operator is one SELL matrix S = A + sigma B
// on the union pattern of A and B (the reference's in-place MatAxpby branch,
// src/ops_eig_sol_gcg.c:600-608), so each iteration streams one matrix.
//
// Vectors are row-interleaved n x kp blocks (row i's kp values contiguous,
// kp = k padded to 16 bytes), which turns the SpMM's gathers into contiguous
// 16-byte loads.  T = double (FP64 GCG) or float (mixed precision: FP32
// values, FP32 SpMM accumulation; cross-block sums in double).
#include <algorithm>

#include "common.cuh"
#include "pcg.cuh"

namespace gcge {

// Deterministic column sums of partials: warp c sums column c.
__device__ inline double sum_partials(const double *part, int nblocks, int kmax, int c, int lane) {
    double s = 0.0;
    for (int b = lane; b < nblocks; b += 32) s += part[(size_t)b * kmax + c];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    return s;
}

// Per-column sums of squares of a row block (thread per row, grid-stride).
template <typename T, int KP>
__global__ void __launch_bounds__(256)
k_rows_colsq(int n, int k, const T *__restrict__ R, double *__restrict__ part, int kmax) {
    __shared__ double red[8][KP];
    T acc[KP];
#pragma unroll
    for (int c = 0; c < KP; ++c) acc[c] = T(0);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
#pragma unroll
        for (int c = 0; c < KP; ++c) {
            const T v = R[(size_t)i * KP + c];
            acc[c] = fma(v, v, acc[c]);
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int c = 0; c < KP; ++c) {
        T v = acc[c];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[warp][c] = (double)v;
    }
    __syncthreads();
    for (int c = threadIdx.x; c < KP && c < k; c += blockDim.x) {
        double s = 0.0;
        for (int w = 0; w < 8; ++w) s += red[w][c];
        part[(size_t)blockIdx.x * kmax + c] = s;
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
            sc->alpha[c] = 0.0;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int cnt = 0;
        for (int c = 0; c < k; ++c) cnt += sc->active[c];
        for (int c = k; c < kPcgMaxCols; ++c) sc->active[c] = 0;
        sc->nactive = cnt;
        sc->niter = 0;
    }
}

// p = r + beta p on the active columns (p = r on the first iteration)
template <typename T, int KP>
__global__ void k_rows_p(int n, const T *__restrict__ R, T *__restrict__ P,
                         const PcgScalars *__restrict__ sc) {
    __shared__ T sbeta[KP];
    __shared__ int sact[KP];
    const bool first = sc->niter == 0;
    for (int c = threadIdx.x; c < KP; c += blockDim.x) {
        sbeta[c] = (T)sc->beta[c];
        sact[c] = sc->active[c];
    }
    __syncthreads();
    const size_t total = (size_t)n * KP;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
         t += (size_t)gridDim.x * blockDim.x) {
        const int c = (int)(t % KP);
        if (!sact[c]) continue;
        P[t] = first ? R[t] : fma(sbeta[c], P[t], R[t]);
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

// x += alpha p, r -= alpha w on the active columns, per-column sums of r^2
template <typename T, int KP>
__global__ void __launch_bounds__(256)
k_rows_xr(int n, int k, T *__restrict__ X, T *__restrict__ R, const T *__restrict__ P,
          const T *__restrict__ W, const PcgScalars *__restrict__ sc, double *__restrict__ part,
          int kmax) {
    __shared__ double red[8][KP];
    __shared__ T salpha[KP];
    __shared__ int sact[KP];
    for (int c = threadIdx.x; c < KP; c += blockDim.x) {
        salpha[c] = (T)sc->alpha[c];
        sact[c] = sc->active[c];
    }
    __syncthreads();
    T acc[KP];
#pragma unroll
    for (int c = 0; c < KP; ++c) acc[c] = T(0);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
#pragma unroll
        for (int c = 0; c < KP; ++c) {
            if (!sact[c]) continue;
            const size_t o = (size_t)i * KP + c;
            const T a = salpha[c];
            X[o] = fma(a, P[o], X[o]);
            const T rn = fma(-a, W[o], R[o]);
            R[o] = rn;
            acc[c] = fma(rn, rn, acc[c]);
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int c = 0; c < KP; ++c) {
        T v = acc[c];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[warp][c] = (double)v;
    }
    __syncthreads();
    for (int c = threadIdx.x; c < KP && c < k; c += blockDim.x) {
        double s = 0.0;
        for (int w = 0; w < 8; ++w) s += red[w][c];
        part[(size_t)blockIdx.x * kmax + c] = s;
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

// column-major (S, ld) <-> row-interleaved (T, kp); padding columns are zero
template <typename S, typename T>
__global__ void k_col_to_rows(int n, int k, int kp, const S *__restrict__ X, int ldx,
                              T *__restrict__ Y) {
    const size_t total = (size_t)n * kp;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
         t += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(t / kp), c = (int)(t % kp);
        Y[t] = c < k ? (T)X[i + (size_t)c * ldx] : T(0);
    }
}
template <typename T, typename D>
__global__ void k_rows_to_col(int n, int k, int kp, const T *__restrict__ X, D *__restrict__ Y,
                              int ldy, int add) {
    const size_t total = (size_t)n * k;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
         t += (size_t)gridDim.x * blockDim.x) {
        const int c = (int)(t / n), i = (int)(t % n);
        const D v = (D)X[(size_t)i * kp + c];
        D &y = Y[i + (size_t)c * ldy];
        y = add ? y + v : v;
    }
}

static int num_sms_pcg() {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 148;
    }
    return sms;
}
static int row_blocks(int n) { return std::max(1, std::min((n + 255) / 256, 2 * num_sms_pcg())); }

template <typename S, typename T>
void col_to_rows(int n, int k, int kp, const S *X, int ldx, T *Y, cudaStream_t st) {
    const size_t total = (size_t)n * kp;
    const int g = (int)std::max<size_t>(1, std::min<size_t>((total + 255) / 256, 16 * num_sms_pcg()));
    k_col_to_rows<S, T><<<g, 256, 0, st>>>(n, k, kp, X, ldx, Y);
    GCGE_CHECK_LAUNCH();
    count_launch();
}
template <typename T, typename D>
void rows_to_col(int n, int k, int kp, const T *X, D *Y, int ldy, bool add, cudaStream_t st) {
    const size_t total = (size_t)n * k;
    const int g = (int)std::max<size_t>(1, std::min<size_t>((total + 255) / 256, 16 * num_sms_pcg()));
    k_rows_to_col<T, D><<<g, 256, 0, st>>>(n, k, kp, X, Y, ldy, add ? 1 : 0);
    GCGE_CHECK_LAUNCH();
    count_launch();
}
template void col_to_rows<double, double>(int, int, int, const double *, int, double *, cudaStream_t);
template void col_to_rows<double, float>(int, int, int, const double *, int, float *, cudaStream_t);
template void rows_to_col<double, double>(int, int, int, const double *, double *, int, bool,
                                          cudaStream_t);
template void rows_to_col<float, double>(int, int, int, const float *, double *, int, bool,
                                         cudaStream_t);

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
    kmax = std::max(kmax_, 40);
    const size_t need = (size_t)std::max(spmm_nblocks, 2 * num_sms_pcg()) * kmax;
    part.alloc(std::max<size_t>(need, 1));
    sc.alloc(1);
    h_sc.alloc(1);
}

template <typename T>
int block_pcg_rows(PcgWork &wk, const SellPattern &pat, const T *sval, const T *Bv, T *X, T *R,
                   T *P, T *W, int kp, int k, int max_iter, double rate, double tol, bool rel_tol,
                   cudaStream_t st) {
    GCGE_REQUIRE(k >= 1 && k <= kp && kp <= 40 && k <= kPcgMaxCols, GCGE_ERR_ARG,
                 "block_pcg: block width");
    const int n = pat.n;
    const int rb = row_blocks(n);
    // norm_b (abs: 1; rel: ||b||), src/ops_lin_sol.c:171-197
    {
        PcgScalars &hs = *wk.h_sc.p;
        std::fill(hs.norm_b, hs.norm_b + kPcgMaxCols, 1.0);
        GCGE_CUDA(cudaMemcpyAsync(&wk.sc.p->norm_b[0], hs.norm_b, sizeof(double) * kPcgMaxCols,
                                  cudaMemcpyHostToDevice, st));
    }
    if (rel_tol) {
        GCGE_KP_DISPATCH(T, kp, (k_rows_colsq<T, KP><<<rb, 256, 0, st>>>(n, k, Bv, wk.part.p, wk.kmax)));
        GCGE_CHECK_LAUNCH();
        k_pcg_normb<<<1, 1024, 0, st>>>(k, wk.part.p, rb, wk.kmax, wk.sc.p);
        GCGE_CHECK_LAUNCH();
        count_launch(2);
    }
    // r = b - S x  (src/ops_lin_sol.c:202-221)
    spmm_rows<T>(pat, sval, X, R, kp, k, nullptr, nullptr, 0, false, st);
    if constexpr (sizeof(T) == 8)
        axpby(n * kp, 1, 1.0, (const double *)Bv, n * kp, -1.0, (double *)R, n * kp, st);
    else
        axpby_f32(n * kp, 1, 1.0f, (const float *)Bv, n * kp, -1.0f, (float *)R, n * kp, st);
    GCGE_KP_DISPATCH(T, kp, (k_rows_colsq<T, KP><<<rb, 256, 0, st>>>(n, k, R, wk.part.p, wk.kmax)));
    GCGE_CHECK_LAUNCH();
    k_pcg_init<<<1, 1024, 0, st>>>(k, wk.part.p, rb, wk.kmax, wk.sc.p, tol);
    GCGE_CHECK_LAUNCH();
    count_launch(2);
    int it = 0;
    const int pgrid = std::max(1, std::min((int)(((size_t)n * kp + 255) / 256), 16 * num_sms_pcg()));
    for (it = 0; it < max_iter; ++it) {
        GCGE_CUDA(cudaMemcpyAsync(&wk.h_sc.p->nactive, &wk.sc.p->nactive, sizeof(int),
                                  cudaMemcpyDeviceToHost, st));
        GCGE_CUDA(cudaStreamSynchronize(st));
        const int nactive = wk.h_sc.p->nactive;
        if (nactive == 0) break;
        GCGE_KP_DISPATCH(T, kp, (k_rows_p<T, KP><<<pgrid, 256, 0, st>>>(n, R, P, wk.sc.p)));
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
        const int nb = spmm_rows<T>(pat, sval, P, W, kp, k, &wk.sc.p->active[0], wk.part.p,
                                    wk.kmax, true, st);
        if (timed) {
            GCGE_CUDA(cudaEventRecord(wk.ev[wk.ev_used + 1], st));
            wk.ev_used += 2;
        }
        // algorithmic bytes: the matrix once, the kp-wide rows of p read once
        // and of w written once (inactive columns ride along in the rows)
        wk.spmm_bytes += (double)pat.nnz * (sizeof(T) + 4) + 4.0 * (n + 1) +
                         2.0 * n * kp * sizeof(T);
        wk.spmm_launches++;
        k_pcg_alpha<<<1, 1024, 0, st>>>(k, wk.part.p, nb, wk.kmax, wk.sc.p);
        GCGE_CHECK_LAUNCH();
        GCGE_KP_DISPATCH(T, kp, (k_rows_xr<T, KP><<<rb, 256, 0, st>>>(n, k, X, R, P, W, wk.sc.p,
                                                                      wk.part.p, wk.kmax)));
        GCGE_CHECK_LAUNCH();
        k_pcg_conv<<<1, 1024, 0, st>>>(k, wk.part.p, rb, wk.kmax, wk.sc.p, rate, tol);
        GCGE_CHECK_LAUNCH();
        count_launch(4);
    }
    return it;
}

template int block_pcg_rows<double>(PcgWork &, const SellPattern &, const double *, const double *,
                                    double *, double *, double *, double *, int, int, int, double,
                                    double, bool, cudaStream_t);
template int block_pcg_rows<float>(PcgWork &, const SellPattern &, const float *, const float *,
                                   float *, float *, float *, float *, int, int, int, double,
                                   double, bool, cudaStream_t);

}  // namespace gcge
