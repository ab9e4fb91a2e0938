// Sparse kernels on SELL-32 matrices: SpMM over a block of columns and the
// fused residual norm ||(A - lambda_c B) x_c||^2 of CheckConvergence (the
// block-PCG SpMM lives inside the persistent kernel of pcg.cu).
//
// Layout: one warp owns one 32-row slice; lane l owns row 32*slice + l and
// walks the slice's entries e = 0..width-1 at slice_ptr + e*32 + l, so each
// step of the warp reads 32 consecutive column indices / values (one 128-byte
// line for int32/fp32, two for fp64).  The dense block X is column-major; for
// a fixed stencil offset the 32 lanes read 32 consecutive x[j] of a column.
// Every column's accumulator stays in registers, so the matrix is streamed
// once for all k columns (reference: one column at a time, app/app_ccs.c:120-131).
#include <algorithm>
#include <numeric>

#include "common.cuh"

namespace gcge {

constexpr int kSpmmThreads = 128;  // 4 slices per block

int spmm_blocks(const SellPattern &pat) {
    return (pat.nslices + (kSpmmThreads / 32) - 1) / (kSpmmThreads / 32);
}

// ---------------------------------------------------------------- kernels
template <typename T, int K>
__global__ void __launch_bounds__(kSpmmThreads)
k_spmm(const long long *__restrict__ sp, const int *__restrict__ col, const T *__restrict__ val,
       int n, int nslices, const T *__restrict__ X, int ldx, T *__restrict__ Y, int ldy, int k) {
    const int slice = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (slice >= nslices) return;
    const long long beg = sp[slice], end = sp[slice + 1];
    T acc[K];
#pragma unroll
    for (int c = 0; c < K; ++c) acc[c] = T(0);
    for (long long e = beg + lane; e < end; e += 32) {
        const int j = __ldg(col + e);
        const T a = __ldg(val + e);
        const T *xj = X + j;
#pragma unroll
        for (int c = 0; c < K; ++c)
            if (c < k) acc[c] = fma(a, __ldg(xj + (size_t)c * ldx), acc[c]);
    }
    const int row = slice * 32 + lane;
    if (row < n) {
#pragma unroll
        for (int c = 0; c < K; ++c)
            if (c < k) Y[row + (size_t)c * ldy] = acc[c];
    }
}

template <int K>
__global__ void __launch_bounds__(kSpmmThreads)
k_residual(const long long *__restrict__ sa, const int *__restrict__ ca,
           const double *__restrict__ va, const long long *__restrict__ sb,
           const int *__restrict__ cb, const double *__restrict__ vb, int n, int nslices,
           const double *__restrict__ X, int ldx, const double *__restrict__ lam, int k,
           double *__restrict__ partial, int kmax, double *__restrict__ ax,
           double *__restrict__ bx, int ldo) {
    __shared__ double red[kSpmmThreads / 32][K];
    __shared__ double slam[K];
    const int slice = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int c = threadIdx.x; c < K; c += blockDim.x) slam[c] = c < k ? lam[c] : 0.0;
    __syncthreads();
    // A x and B x, each on its own matrix's SELL pattern (as the reference's
    // two SpMMs and axpby, src/ops_eig_sol_gcg.c:220-238); padding entries
    // carry a zero value and the row's own column.  A x is stored before B x
    // is formed in the same registers (half the registers of keeping both, so
    // twice the resident warps), and read back for the residual.
    double acc[K];
#pragma unroll
    for (int c = 0; c < K; ++c) acc[c] = 0.0;
    const int row = slice * 32 + lane;
    if (slice < nslices) {
        for (long long e = sa[slice] + lane, end = sa[slice + 1]; e < end; e += 32) {
            const double v = __ldg(va + e);
            const double *xj = X + __ldg(ca + e);
#pragma unroll
            for (int c = 0; c < K; ++c)
                if (c < k) acc[c] = fma(v, __ldg(xj + (size_t)c * ldx), acc[c]);
        }
    }
    if (row < n) {
#pragma unroll
        for (int c = 0; c < K; ++c)
            if (c < k) ax[row + (size_t)c * ldo] = acc[c];
    }
#pragma unroll
    for (int c = 0; c < K; ++c) acc[c] = 0.0;
    if (slice < nslices) {
        if (sb != nullptr) {
            for (long long e = sb[slice] + lane, end = sb[slice + 1]; e < end; e += 32) {
                const double v = __ldg(vb + e);
                const double *xj = X + __ldg(cb + e);
#pragma unroll
                for (int c = 0; c < K; ++c)
                    if (c < k) acc[c] = fma(v, __ldg(xj + (size_t)c * ldx), acc[c]);
            }
        } else if (row < n) {  // B = I
#pragma unroll
            for (int c = 0; c < K; ++c)
                if (c < k) acc[c] = X[row + (size_t)c * ldx];
        }
    }
    if (row < n) {
#pragma unroll
        for (int c = 0; c < K; ++c)
            if (c < k) bx[row + (size_t)c * ldo] = acc[c];
    }
#pragma unroll
    for (int c = 0; c < K; ++c) {
        double v = 0.0;
        if (row < n && c < k) {
            const double r = fma(-slam[c], acc[c], ax[row + (size_t)c * ldo]);
            v = r * r;
        }
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[warp][c] = v;
    }
    __syncthreads();
    for (int c = threadIdx.x; c < K; c += blockDim.x) {
        double s = 0.0;
#pragma unroll
        for (int w = 0; w < kSpmmThreads / 32; ++w) s += red[w][c];
        if (c < kmax) partial[(size_t)blockIdx.x * kmax + c] = s;
    }
}

// ---------------------------------------------------------------- dispatch
#define GCGE_K_DISPATCH(kk, BODY)                          \
    do {                                                   \
        if ((kk) <= 4) { constexpr int KT = 4; BODY; }        \
        else if ((kk) <= 8) { constexpr int KT = 8; BODY; }   \
        else if ((kk) <= 16) { constexpr int KT = 16; BODY; } \
        else if ((kk) <= 24) { constexpr int KT = 24; BODY; } \
        else if ((kk) <= 32) { constexpr int KT = 32; BODY; } \
        else { constexpr int KT = 40; BODY; }                 \
    } while (0)

constexpr int kMaxChunk = 40;

template <typename T>
void spmm(const SellPattern &pat, const T *val, const T *X, int ldx, T *Y, int ldy, int k,
          cudaStream_t st) {
    if (k <= 0 || pat.n == 0) return;
    const int blocks = spmm_blocks(pat);
    for (int c0 = 0; c0 < k; c0 += kMaxChunk) {
        const int kc = std::min(kMaxChunk, k - c0);
        GCGE_K_DISPATCH(kc, (k_spmm<T, KT><<<blocks, kSpmmThreads, 0, st>>>(
                                pat.slice_ptr.p, pat.col.p, val, pat.n, pat.nslices,
                                X + (size_t)c0 * ldx, ldx, Y + (size_t)c0 * ldy, ldy, kc)));
        GCGE_CHECK_LAUNCH();
        count_launch();
    }
}

int residual_norms(const SellPattern &pa, const double *va, const SellPattern *pb,
                   const double *vb, const double *X, int ldx, const double *lam, int k,
                   double *partial, int kmax, cudaStream_t st, double *ax, double *bx, int ldo) {
    GCGE_REQUIRE(k <= kMaxChunk && k <= kmax, GCGE_ERR_ARG, "residual_norms: too many columns");
    GCGE_REQUIRE(ax != nullptr && bx != nullptr, GCGE_ERR_ARG, "residual_norms: no product buffers");
    GCGE_REQUIRE(!pb || (pb->n == pa.n && pb->nslices == pa.nslices), GCGE_ERR_ARG,
                 "residual_norms: patterns differ in size");
    const int blocks = spmm_blocks(pa);
    if (k <= 0) return 0;
    GCGE_K_DISPATCH(k, (k_residual<KT><<<blocks, kSpmmThreads, 0, st>>>(
                           pa.slice_ptr.p, pa.col.p, va, pb ? pb->slice_ptr.p : nullptr,
                           pb ? pb->col.p : nullptr, vb, pa.n, pa.nslices, X, ldx, lam, k,
                           partial, kmax, ax, bx, ldo)));
    GCGE_CHECK_LAUNCH();
    count_launch();
    return blocks;
}

template void spmm<double>(const SellPattern &, const double *, const double *, int, double *,
                           int, int, cudaStream_t);
template void spmm<float>(const SellPattern &, const float *, const float *, int, float *, int,
                          int, cudaStream_t);
}  // namespace gcge

// ==================================================================== widths
namespace gcge {

// Smallest block-PCG row width >= k whose 16-byte column groups are whole
// (instantiated widths of the block-PCG kernel).
int rows_width(int k, int elem_bytes) {
    static const int w32[] = {4, 8, 12, 16, 20, 24, 28, 32, 36, 40};
    static const int w64[] = {2, 4, 6, 8, 12, 16, 20, 24, 28, 32, 36, 40};
    if (elem_bytes == 4) {
        for (int w : w32)
            if (w >= k) return w;
    } else {
        for (int w : w64)
            if (w >= k) return w;
    }
    throw CudaError{GCGE_ERR_ARG, "block PCG: block wider than 40 columns"};
}

}  // namespace gcge
