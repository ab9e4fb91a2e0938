// Dense multivector kernels (FP64 unless noted): axpby, the tall-skinny
// products X*C (MultiVecLinearComb, Ritz vectors, P) and Q^T P (inner products,
// Gram blocks of Rayleigh-Ritz and B-orthogonalisation), column dots and
// small helpers.
//
// FP64 on GB300 issues about two FMAs per clock per SM (measured 1.2 TFLOP/s
// for the whole part against 70 TFLOP/s FP32), so the products are FP64-FMA
// bound, not HBM bound: the kernels keep every SM busy (split-K for Q^T P,
// small tiles for small outputs) rather than chasing data reuse.
#include <algorithm>

#include "common.cuh"

namespace gcge {

static int num_sms() { return device_sms(); }

// ---------------------------------------------------------------- axpby
template <typename T>
__global__ void k_axpby(int n, int ncols, T alpha, const T *__restrict__ X, int ldx, T beta,
                        T *__restrict__ Y, int ldy) {
    const size_t total = (size_t)n * ncols;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
         t += (size_t)gridDim.x * blockDim.x) {
        const int c = (int)(t / n), i = (int)(t % n);
        T y = beta == T(0) ? T(0) : beta * Y[i + (size_t)c * ldy];
        if (X != nullptr && alpha != T(0)) y = fma(alpha, X[i + (size_t)c * ldx], y);
        Y[i + (size_t)c * ldy] = y;
    }
}

static int grid_for(size_t total, int threads) {
    size_t b = (total + threads - 1) / threads;
    size_t cap = (size_t)num_sms() * 16;
    return (int)std::max<size_t>(1, std::min(b, cap));
}

void axpby(int n, int ncols, double alpha, const double *X, int ldx, double beta, double *Y,
           int ldy, cudaStream_t st) {
    if (n <= 0 || ncols <= 0) return;
    k_axpby<double><<<grid_for((size_t)n * ncols, 256), 256, 0, st>>>(n, ncols, alpha, X, ldx,
                                                                       beta, Y, ldy);
    GCGE_CHECK_LAUNCH();
    count_launch();
}
void axpby_f32(int n, int ncols, float alpha, const float *X, int ldx, float beta, float *Y,
               int ldy, cudaStream_t st) {
    if (n <= 0 || ncols <= 0) return;
    k_axpby<float><<<grid_for((size_t)n * ncols, 256), 256, 0, st>>>(n, ncols, alpha, X, ldx, beta,
                                                                      Y, ldy);
    GCGE_CHECK_LAUNCH();
    count_launch();
}

__global__ void k_scale_cols(int n, int m, double *__restrict__ Y, int ldy,
                             const double *__restrict__ s, int inc) {
    const size_t total = (size_t)n * m;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
         t += (size_t)gridDim.x * blockDim.x) {
        const int c = (int)(t / n), i = (int)(t % n);
        const double b = s[inc == 0 ? 0 : (size_t)c * inc];
        Y[i + (size_t)c * ldy] = b == 0.0 ? 0.0 : b * Y[i + (size_t)c * ldy];
    }
}
void scale_columns_strided(int n, int m, double *Y, int ldy, const double *s, int inc,
                           cudaStream_t st) {
    if (n <= 0 || m <= 0) return;
    k_scale_cols<<<grid_for((size_t)n * m, 256), 256, 0, st>>>(n, m, Y, ldy, s, inc);
    GCGE_CHECK_LAUNCH();
    count_launch();
}
void scale_columns(int n, int k, double *X, int ldx, const double *s, cudaStream_t st) {
    scale_columns_strided(n, k, X, ldx, s, 1, st);
}

// ---------------------------------------------------------------- X * C
// Tile TM rows x TN columns of Y per block, NT threads; thread t owns row
// t % TM and TN / (NT / TM) consecutive columns.  X and C tiles are staged
// through shared memory in chunks of TK.
template <int TM, int TN, int TK, int NT>
__global__ void __launch_bounds__(NT)
k_lincomb(int n, int k, int m, const double *__restrict__ X, int ldx, const double *__restrict__ C,
          int ldc, double *__restrict__ Y, int ldy, const double *__restrict__ beta, int incb,
          double alpha) {
    constexpr int G = NT / TM;      // column groups
    constexpr int CPT = TN / G;     // columns per thread
    __shared__ double Xs[TK][TM];
    __shared__ double Cs[TK][TN + 1];
    const int t = threadIdx.x;
    const int r = t % TM, g = t / TM;
    const int row0 = blockIdx.x * TM, col0 = blockIdx.y * TN;
    double acc[CPT];
#pragma unroll
    for (int j = 0; j < CPT; ++j) acc[j] = 0.0;
    for (int k0 = 0; k0 < k; k0 += TK) {
        for (int idx = t; idx < TK * TM; idx += NT) {
            const int l = idx / TM, rr = idx % TM;
            const int gr = row0 + rr, gl = k0 + l;
            Xs[l][rr] = (gr < n && gl < k) ? X[gr + (size_t)gl * ldx] : 0.0;
        }
        for (int idx = t; idx < TK * TN; idx += NT) {
            const int l = idx % TK, jj = idx / TK;
            const int gl = k0 + l, gc = col0 + jj;
            Cs[l][jj] = (gl < k && gc < m) ? C[gl + (size_t)gc * ldc] : 0.0;
        }
        __syncthreads();
#pragma unroll 4
        for (int l = 0; l < TK; ++l) {
            const double x = Xs[l][r];
#pragma unroll
            for (int j = 0; j < CPT; ++j) acc[j] = fma(x, Cs[l][g * CPT + j], acc[j]);
        }
        __syncthreads();
    }
    const int gr = row0 + r;
    if (gr < n) {
#pragma unroll
        for (int j = 0; j < CPT; ++j) {
            const int gc = col0 + g * CPT + j;
            if (gc < m) {
                double y = alpha * acc[j];
                if (beta != nullptr) {
                    const double b = beta[incb == 0 ? 0 : (size_t)gc * incb];
                    if (b != 0.0) y = fma(b, Y[gr + (size_t)gc * ldy], y);
                }
                Y[gr + (size_t)gc * ldy] = y;
            }
        }
    }
}

void lincomb(int n, int k, int m, const double *X, int ldx, const double *C, int ldc, double *Y,
             int ldy, const double *beta_dev, int incb, cudaStream_t st, double alpha) {
    if (n <= 0 || m <= 0) return;
    if (k <= 0) {  // Y = Y diag(beta)
        if (beta_dev == nullptr) {
            for (int c = 0; c < m; ++c)
                GCGE_CUDA(cudaMemsetAsync(Y + (size_t)c * ldy, 0, sizeof(double) * n, st));
        } else {
            scale_columns_strided(n, m, Y, ldy, beta_dev, incb, st);  // incb 0 = scalar
        }
        return;
    }
    // column tile fitted to m (multiple of 4 up to 32) so thin products waste
    // no FMA lanes; 64-row tiles for tall outputs, 16 x 16 tiles for small ones
    const int tn = m >= 32 ? 32 : ((m + 3) / 4) * 4;
    const long long big_blocks = (long long)((n + 63) / 64) * ((m + tn - 1) / tn);
    if (big_blocks >= 2LL * num_sms()) {
        dim3 grid((n + 63) / 64, (m + tn - 1) / tn);
        switch (tn) {
#define GCGE_LC_CASE(W)                                                                         \
    case W:                                                                                    \
        k_lincomb<64, W, 16, 256><<<grid, 256, 0, st>>>(n, k, m, X, ldx, C, ldc, Y, ldy, beta_dev, \
                                                        incb, alpha);                          \
        break;
            GCGE_LC_CASE(4) GCGE_LC_CASE(8) GCGE_LC_CASE(12) GCGE_LC_CASE(16) GCGE_LC_CASE(20)
            GCGE_LC_CASE(24) GCGE_LC_CASE(28) GCGE_LC_CASE(32)
#undef GCGE_LC_CASE
            default: break;
        }
    } else {
        dim3 grid((n + 15) / 16, (m + 15) / 16);
        k_lincomb<16, 16, 16, 64><<<grid, 64, 0, st>>>(n, k, m, X, ldx, C, ldc, Y, ldy, beta_dev,
                                                       incb, alpha);
    }
    GCGE_CHECK_LAUNCH();
    count_launch();
}

// ---------------------------------------------------------------- Q^T P
// Block (chunk, mt, wt) accumulates the 32 x TW tile (mt, wt) of Q^T P over
// its row chunk; thread t owns row a = t % 32 of the tile and TW/8 columns.
constexpr int kGT = 32;
template <int TW>
__device__ __forceinline__ void gram_tile(int n, int m, int w, const double *__restrict__ Q, int ldq,
                                          const double *__restrict__ P, int ldp,
                                          double *__restrict__ part, int rows_per_chunk) {
    constexpr int CPT = TW / 8;
    __shared__ double Qs[kGT][kGT + 1];
    __shared__ double Ps[kGT][TW + 1];
    const int t = threadIdx.x;
    const int a = t % kGT, g = t / kGT;  // 8 groups x CPT columns
    const int chunk = blockIdx.x;
    const int a0 = blockIdx.y * kGT, b0 = blockIdx.z * TW;
    const int r_begin = chunk * rows_per_chunk;
    const int r_end = min(n, r_begin + rows_per_chunk);
    double acc[CPT];
#pragma unroll
    for (int j = 0; j < CPT; ++j) acc[j] = 0.0;
    for (int r0 = r_begin; r0 < r_end; r0 += kGT) {
        for (int idx = t; idx < kGT * kGT; idx += 256) {
            const int i = idx % kGT, cc = idx / kGT;
            const int gi = r0 + i;
            Qs[i][cc] = (gi < r_end && a0 + cc < m) ? Q[gi + (size_t)(a0 + cc) * ldq] : 0.0;
        }
        for (int idx = t; idx < kGT * TW; idx += 256) {
            const int i = idx % kGT, cc = idx / kGT;
            const int gi = r0 + i;
            Ps[i][cc] = (gi < r_end && b0 + cc < w) ? P[gi + (size_t)(b0 + cc) * ldp] : 0.0;
        }
        __syncthreads();
#pragma unroll 8
        for (int i = 0; i < kGT; ++i) {
            const double q = Qs[i][a];
#pragma unroll
            for (int j = 0; j < CPT; ++j) acc[j] = fma(q, Ps[i][g * CPT + j], acc[j]);
        }
        __syncthreads();
    }
    const size_t base = (size_t)chunk * m * w;
#pragma unroll
    for (int j = 0; j < CPT; ++j) {
        const int ga = a0 + a, gb = b0 + g * CPT + j;
        if (ga < m && gb < w) part[base + ga + (size_t)gb * m] = acc[j];
    }
}

template <int TW>
__global__ void __launch_bounds__(256)
k_gram_w(int n, int m, int w, const double *__restrict__ Q, int ldq, const double *__restrict__ P,
         int ldp, double *__restrict__ part, int rows_per_chunk) {
    gram_tile<TW>(n, m, w, Q, ldq, P, ldp, part, rows_per_chunk);
}

// 32 x 32 tile instance with a fixed name (used by GCGE_GramNoAlloc)
__global__ void __launch_bounds__(256)
k_gram(int n, int m, int w, const double *__restrict__ Q, int ldq, const double *__restrict__ P,
       int ldp, double *__restrict__ part, int rows_per_chunk) {
    gram_tile<32>(n, m, w, Q, ldq, P, ldp, part, rows_per_chunk);
}

__global__ void k_reduce_chunks(const double *__restrict__ part, int chunks, int m, int w,
                                double *__restrict__ C, int ldc) {
    const int total = m * w;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int c = 0; c < chunks; ++c) s += part[(size_t)c * total + e];
        const int a = e % m, b = e / m;
        C[a + (size_t)b * ldc] = s;
    }
}

static int gram_chunks(int n, int m, int w) {
    const int tw = w >= 32 ? 32 : std::max(8, ((w + 7) / 8) * 8);
    const int tiles = ((m + kGT - 1) / kGT) * ((w + tw - 1) / tw);
    const int want = std::max(1, (3 * num_sms() + tiles - 1) / tiles);
    const int maxc = std::max(1, (n + 127) / 128);
    return std::min(want, maxc);
}
size_t gram_scratch_elems(int n, int m, int w) {
    return (size_t)gram_chunks(n, m, w) * m * w;
}

void gram(int n, int m, int w, const double *Q, int ldq, const double *P, int ldp, double *C,
          int ldc, double *scratch, size_t scratch_elems, cudaStream_t st) {
    if (m <= 0 || w <= 0) return;
    if (n <= 0) {
        for (int b = 0; b < w; ++b)
            GCGE_CUDA(cudaMemsetAsync(C + (size_t)b * ldc, 0, sizeof(double) * m, st));
        return;
    }
    const int chunks = gram_chunks(n, m, w);
    GCGE_REQUIRE((size_t)chunks * m * w <= scratch_elems, GCGE_ERR_ARG, "gram: scratch too small");
    int rpc = (n + chunks - 1) / chunks;
    rpc = (rpc + kGT - 1) / kGT * kGT;
    const int nchunks = (n + rpc - 1) / rpc;
    const int tw = w >= 32 ? 32 : std::max(8, ((w + 7) / 8) * 8);
    dim3 grid(nchunks, (m + kGT - 1) / kGT, (w + tw - 1) / tw);
    switch (tw) {
        case 8: k_gram_w<8><<<grid, 256, 0, st>>>(n, m, w, Q, ldq, P, ldp, scratch, rpc); break;
        case 16: k_gram_w<16><<<grid, 256, 0, st>>>(n, m, w, Q, ldq, P, ldp, scratch, rpc); break;
        case 24: k_gram_w<24><<<grid, 256, 0, st>>>(n, m, w, Q, ldq, P, ldp, scratch, rpc); break;
        default: k_gram_w<32><<<grid, 256, 0, st>>>(n, m, w, Q, ldq, P, ldp, scratch, rpc); break;
    }
    GCGE_CHECK_LAUNCH();
    const int tot = m * w;
    k_reduce_chunks<<<std::max(1, std::min((tot + 255) / 256, 4 * num_sms())), 256, 0, st>>>(
        scratch, nchunks, m, w, C, ldc);
    GCGE_CHECK_LAUNCH();
    count_launch(2);
}

// ---------------------------------------------------------------- column dots
__global__ void __launch_bounds__(256)
k_coldot(int n, int k, const double *__restrict__ X, int ldx, const double *__restrict__ Y, int ldy,
         double *__restrict__ part, int rows_per_chunk) {
    __shared__ double red[8];
    const int c = blockIdx.y;
    const int r_begin = blockIdx.x * rows_per_chunk;
    const int r_end = min(n, r_begin + rows_per_chunk);
    double s = 0.0;
    for (int i = r_begin + threadIdx.x; i < r_end; i += 256)
        s = fma(X[i + (size_t)c * ldx], Y[i + (size_t)c * ldy], s);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double tsum = 0.0;
        for (int i = 0; i < 8; ++i) tsum += red[i];
        part[(size_t)blockIdx.x * k + c] = tsum;
    }
}

void coldot(int n, int k, const double *X, int ldx, const double *Y, int ldy, double *out,
            double *scratch, size_t scratch_elems, cudaStream_t st) {
    if (k <= 0) return;
    int chunks = std::max(1, std::min((n + 2047) / 2048, (2 * num_sms() + k - 1) / k));
    while ((size_t)chunks * k > scratch_elems && chunks > 1) chunks /= 2;
    GCGE_REQUIRE((size_t)chunks * k <= scratch_elems, GCGE_ERR_ARG, "coldot: scratch too small");
    const int rpc = (n + chunks - 1) / chunks;
    dim3 grid(chunks, k);
    k_coldot<<<grid, 256, 0, st>>>(n, k, X, ldx, Y, ldy, scratch, rpc);
    GCGE_CHECK_LAUNCH();
    count_launch();
    reduce_partials(scratch, chunks, k, k, out, st);
}

__global__ void k_reduce_partials(const double *__restrict__ part, int nblocks, int kmax,
                                  double *__restrict__ out) {
    __shared__ double red[256];
    const int c = blockIdx.x;
    double s = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += 256) s += part[(size_t)b * kmax + c];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[c] = red[0];
}

void reduce_partials(const double *partial, int nblocks, int kmax, int k, double *out,
                     cudaStream_t st) {
    if (k <= 0) return;
    k_reduce_partials<<<k, 256, 0, st>>>(partial, nblocks, kmax, out);
    GCGE_CHECK_LAUNCH();
    count_launch();
}

// ---------------------------------------------------------------- helpers
template <typename S, typename D>
__global__ void k_convert(int n, int k, const S *__restrict__ X, int ldx, D *__restrict__ Y,
                          int ldy) {
    const size_t total = (size_t)n * k;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
         t += (size_t)gridDim.x * blockDim.x) {
        const int c = (int)(t / n), i = (int)(t % n);
        Y[i + (size_t)c * ldy] = (D)X[i + (size_t)c * ldx];
    }
}
void copy_f64_to_f32(int n, int k, const double *X, int ldx, float *Y, int ldy, cudaStream_t st) {
    if (n <= 0 || k <= 0) return;
    k_convert<double, float><<<grid_for((size_t)n * k, 256), 256, 0, st>>>(n, k, X, ldx, Y, ldy);
    GCGE_CHECK_LAUNCH();
    count_launch();
}
__global__ void k_add_f32(int n, int k, const float *__restrict__ X, int ldx, double *__restrict__ Y,
                          int ldy) {
    const size_t total = (size_t)n * k;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
         t += (size_t)gridDim.x * blockDim.x) {
        const int c = (int)(t / n), i = (int)(t % n);
        Y[i + (size_t)c * ldy] += (double)X[i + (size_t)c * ldx];
    }
}
void add_f32_to_f64(int n, int k, const float *X, int ldx, double *Y, int ldy, cudaStream_t st) {
    if (n <= 0 || k <= 0) return;
    k_add_f32<<<grid_for((size_t)n * k, 256), 256, 0, st>>>(n, k, X, ldx, Y, ldy);
    GCGE_CHECK_LAUNCH();
    count_launch();
}
void copy_f32_to_f64(int n, int k, const float *X, int ldx, double *Y, int ldy, cudaStream_t st) {
    if (n <= 0 || k <= 0) return;
    k_convert<float, double><<<grid_for((size_t)n * k, 256), 256, 0, st>>>(n, k, X, ldx, Y, ldy);
    GCGE_CHECK_LAUNCH();
    count_launch();
}

__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
__global__ void k_fill_uniform(int n, int k, double *__restrict__ X, int ldx,
                               unsigned long long seed) {
    const size_t total = (size_t)n * k;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
         t += (size_t)gridDim.x * blockDim.x) {
        const int c = (int)(t / n), i = (int)(t % n);
        const unsigned long long z = mix64(seed * 0x9E3779B97F4A7C15ULL + t + 1);
        X[i + (size_t)c * ldx] = (double)(z >> 11) * (1.0 / 9007199254740992.0);
    }
}
void fill_uniform(int n, int k, double *X, int ldx, unsigned long long seed, cudaStream_t st) {
    if (n <= 0 || k <= 0) return;
    k_fill_uniform<<<grid_for((size_t)n * k, 256), 256, 0, st>>>(n, k, X, ldx, seed);
    GCGE_CHECK_LAUNCH();
    count_launch();
}

__global__ void k_gather_cols(int n, int k, const double *__restrict__ X, int ldx,
                              const int *__restrict__ idx, double *__restrict__ Y, int ldy) {
    const size_t total = (size_t)n * k;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
         t += (size_t)gridDim.x * blockDim.x) {
        const int c = (int)(t / n), i = (int)(t % n);
        Y[i + (size_t)c * ldy] = X[i + (size_t)idx[c] * ldx];
    }
}
void gather_columns(int n, int k, const double *X, int ldx, const int *idx, double *Y, int ldy,
                    cudaStream_t st) {
    if (n <= 0 || k <= 0) return;
    k_gather_cols<<<grid_for((size_t)n * k, 256), 256, 0, st>>>(n, k, X, ldx, idx, Y, ldy);
    GCGE_CHECK_LAUNCH();
    count_launch();
}

__global__ void k_identity(int n, double *__restrict__ X, int ldx) {
    const size_t total = (size_t)n * n;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
         t += (size_t)gridDim.x * blockDim.x) {
        const int c = (int)(t / n), i = (int)(t % n);
        X[i + (size_t)c * ldx] = i == c ? 1.0 : 0.0;
    }
}
void set_identity(int n, double *X, int ldx, cudaStream_t st) {
    if (n <= 0) return;
    k_identity<<<grid_for((size_t)n * n, 256), 256, 0, st>>>(n, X, ldx);
    GCGE_CHECK_LAUNCH();
    count_launch();
}

__global__ void k_fill(size_t count, double *__restrict__ X, double v) {
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < count;
         t += (size_t)gridDim.x * blockDim.x)
        X[t] = v;
}
void fill_value(size_t count, double *X, double v, cudaStream_t st) {
    if (count == 0) return;
    k_fill<<<grid_for(count, 256), 256, 0, st>>>(count, X, v);
    GCGE_CHECK_LAUNCH();
    count_launch();
}

}  // namespace gcge

namespace gcge {

__global__ void k_absmax(int m, int w, const double *__restrict__ C, int ldc, double *out) {
    __shared__ double red[32];
    double v = 0.0;
    for (int e = threadIdx.x; e < m * w; e += blockDim.x) {
        const double a = fabs(C[(e % m) + (size_t)(e / m) * ldc]);
        v = (a > v || a != a) ? a : v;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const double u = __shfl_xor_sync(0xffffffffu, v, o);
        v = (u > v || u != u) ? u : v;
    }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = 0.0;
        for (int i = 0; i < (int)(blockDim.x + 31) / 32; ++i) r = (red[i] > r || red[i] != red[i]) ? red[i] : r;
        *out = r;
    }
}
void absmax(int m, int w, const double *C, int ldc, double *out, cudaStream_t st) {
    k_absmax<<<1, 1024, 0, st>>>(m, w, C, ldc, out);
    GCGE_CHECK_LAUNCH();
    count_launch();
}

__global__ void k_zero_rows(int m, int k, double *__restrict__ X, int ldx,
                            const int *__restrict__ mask) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < m * k; e += gridDim.x * blockDim.x) {
        const int i = e % m, j = e / m;
        if (mask[i]) X[i + (size_t)j * ldx] = 0.0;
    }
}
void zero_rows(int m, int k, double *X, int ldx, const int *mask, cudaStream_t st) {
    if (m <= 0 || k <= 0) return;
    k_zero_rows<<<std::max(1, std::min(1024, (m * k + 255) / 256)), 256, 0, st>>>(m, k, X, ldx,
                                                                                  mask);
    GCGE_CHECK_LAUNCH();
    count_launch();
}

__global__ void k_transpose(int m, int k, const double *__restrict__ X, int ldx,
                            double *__restrict__ Y, int ldy) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < m * k; e += gridDim.x * blockDim.x) {
        const int i = e % m, j = e / m;
        Y[j + (size_t)i * ldy] = X[i + (size_t)j * ldx];
    }
}
void transpose_copy(int m, int k, const double *X, int ldx, double *Y, int ldy, cudaStream_t st) {
    if (m <= 0 || k <= 0) return;
    k_transpose<<<std::max(1, std::min(1024, (m * k + 255) / 256)), 256, 0, st>>>(m, k, X, ldx, Y,
                                                                                  ldy);
    GCGE_CHECK_LAUNCH();
    count_launch();
}

__global__ void k_shift(size_t count, const double *__restrict__ a, const double *__restrict__ b,
                        double sigma, double *__restrict__ y64, float *__restrict__ y32) {
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < count;
         t += (size_t)gridDim.x * blockDim.x) {
        const double v = fma(sigma, b[t], a[t]);
        if (y64) y64[t] = v;
        if (y32) y32[t] = (float)v;
    }
}
void shift_values(size_t count, const double *a, const double *b, double sigma, double *y64,
                  float *y32, cudaStream_t st) {
    if (count == 0) return;
    k_shift<<<grid_for(count, 256), 256, 0, st>>>(count, a, b, sigma, y64, y32);
    GCGE_CHECK_LAUNCH();
    count_launch();
}

void copy_cols(int n, int k, const double *X, int ldx, double *Y, int ldy, cudaStream_t st) {
    if (n <= 0 || k <= 0 || X == Y) return;
    GCGE_CUDA(cudaMemcpy2DAsync(Y, sizeof(double) * ldy, X, sizeof(double) * ldx,
                                sizeof(double) * n, k, cudaMemcpyDeviceToDevice, st));
}

}  // namespace gcge
