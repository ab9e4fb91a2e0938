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
#include <atomic>
#include <cstdlib>
#include <limits>
#include <map>
#include <numeric>
#include <tuple>

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

// Register width (accumulators per lane) GCGE_K_DISPATCH gives kc columns.
static int spmm_dispatch_width(int kc) {
    return kc <= 4 ? 4 : kc <= 8 ? 8 : kc <= 16 ? 16 : kc <= 24 ? 24 : kc <= 32 ? 32 : 40;
}

// Y = M X in launches of `chunk` columns each (the last one narrower): each
// launch streams the matrix once and keeps its columns' sums in registers.
// Every column's sum runs over the same entries in the same order whatever
// the chunk, so the result does not depend on it.
template <typename T>
static void spmm_split(const SellPattern &pat, const T *val, const T *X, int ldx, T *Y, int ldy,
                       int k, int chunk, cudaStream_t st) {
    const int blocks = spmm_blocks(pat);
    for (int c0 = 0; c0 < k; c0 += chunk) {
        const int kc = std::min(chunk, k - c0);
        GCGE_K_DISPATCH(kc, (k_spmm<T, KT><<<blocks, kSpmmThreads, 0, st>>>(
                                pat.slice_ptr.p, pat.col.p, val, pat.n, pat.nslices,
                                X + (size_t)c0 * ldx, ldx, Y + (size_t)c0 * ldy, ldy, kc)));
        GCGE_CHECK_LAUNCH();
        count_launch();
    }
}

// ---------------------------------------------------------------- tuning
// The column split of an SpMM is a trade: wide launches read the matrix fewer
// times, narrow ones need fewer registers per lane and so keep more warps
// resident to hide the gathers' latency.  Which wins depends on the matrix
// (entries per row, locality of its columns) and the device, so the tuner
// measures it.  Candidates split k columns into p equal launches, p from
// ceil(k / 40) up while a launch keeps at least 8 columns; of the p that give
// the same register width only the smallest is kept (more launches of the
// same width only re-read the matrix).
std::vector<int> spmm_split_candidates(int k) {
    std::vector<int> out;
    if (k <= 0) return out;
    int last = -1;
    for (int p = (k + kMaxChunk - 1) / kMaxChunk;; ++p) {
        const int chunk = (k + p - 1) / p;
        if (!out.empty() && chunk < 8) break;
        const int w = spmm_dispatch_width(chunk);
        if (w != last) {
            out.push_back(p);
            last = w;
        }
        if (chunk <= 8) break;
    }
    return out;
}

namespace {
// A tuned split is kept per device, value type, matrix shape (rows and
// stored entries) and column class (k rounded up to a multiple of 8).
struct SpmmTuneKey {
    int dev, elem, n, kclass;
    long long padded;
    bool operator<(const SpmmTuneKey &o) const {
        return std::tie(dev, elem, n, kclass, padded) <
               std::tie(o.dev, o.elem, o.n, o.kclass, o.padded);
    }
};
std::mutex g_tune_mu;
std::map<SpmmTuneKey, int> g_tune;  // chosen number of launches p
// -1: not yet read from the environment (GCGE_SPMM_TUNE), 0 off, 1 on
std::atomic<int> g_tune_on{-1};

struct EventPair {
    cudaEvent_t a = nullptr, b = nullptr;
    EventPair() {
        GCGE_CUDA(cudaEventCreate(&a));
        cudaError_t e = cudaEventCreate(&b);
        if (e != cudaSuccess) {
            cudaEventDestroy(a);
            GCGE_CUDA(e);
        }
    }
    ~EventPair() {
        cudaEventDestroy(a);
        cudaEventDestroy(b);
    }
};
}  // namespace

bool spmm_tuning_on() {
    int v = g_tune_on.load(std::memory_order_relaxed);
    if (v < 0) {
        const char *e = getenv("GCGE_SPMM_TUNE");
        int want = (e != nullptr && atoi(e) != 0) ? 1 : 0, expect = -1;
        g_tune_on.compare_exchange_strong(expect, want);
        v = g_tune_on.load();
    }
    return v == 1;
}

void set_spmm_tuning(bool on) { g_tune_on.store(on ? 1 : 0); }

void clear_spmm_tuning() {
    std::lock_guard<std::mutex> g(g_tune_mu);
    g_tune.clear();
}

// The number of launches p for an SpMM of k columns: the cached choice for
// this matrix shape and column class, or, on the first call (and always when
// ms_out is given), each candidate timed with CUDA events on `st` (one
// untimed run, then kTuneReps timed runs) on the caller's own X and Y, which
// hold M X after every run.  A later candidate must beat the best by 2% to
// replace it, so noise does not pick more launches.  Not tuned while `st` is
// being captured into a graph (the timing waits on the host).
template <typename T>
int spmm_tuned_split(const SellPattern &pat, const T *val, const T *X, int ldx, T *Y, int ldy,
                     int k, cudaStream_t st, std::vector<double> *ms_out) {
    constexpr int kTuneReps = 3;
    const std::vector<int> cand = spmm_split_candidates(k);
    if (cand.empty()) return 1;
    if (cand.size() == 1 && ms_out == nullptr) return cand[0];
    const SpmmTuneKey key{current_device(), (int)sizeof(T), pat.n, (k + 7) / 8, pat.padded};
    if (ms_out == nullptr) {
        std::lock_guard<std::mutex> g(g_tune_mu);
        auto it = g_tune.find(key);
        if (it != g_tune.end()) return it->second;
    }
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    GCGE_CUDA(cudaStreamIsCapturing(st, &cs));
    if (cs != cudaStreamCaptureStatusNone) return cand[0];
    EventPair ev;
    double best = std::numeric_limits<double>::infinity();
    int bestp = cand[0];
    for (int p : cand) {
        const int chunk = (k + p - 1) / p;
        spmm_split(pat, val, X, ldx, Y, ldy, k, chunk, st);
        GCGE_CUDA(cudaEventRecord(ev.a, st));
        for (int r = 0; r < kTuneReps; ++r) spmm_split(pat, val, X, ldx, Y, ldy, k, chunk, st);
        GCGE_CUDA(cudaEventRecord(ev.b, st));
        GCGE_CUDA(cudaEventSynchronize(ev.b));
        float ms = 0.f;
        GCGE_CUDA(cudaEventElapsedTime(&ms, ev.a, ev.b));
        const double t = (double)ms / kTuneReps;
        if (ms_out) ms_out->push_back(t);
        if (t < best * 0.98) {
            best = t;
            bestp = p;
        }
    }
    std::lock_guard<std::mutex> g(g_tune_mu);
    g_tune[key] = bestp;
    return bestp;
}

template <typename T>
void spmm(const SellPattern &pat, const T *val, const T *X, int ldx, T *Y, int ldy, int k,
          cudaStream_t st) {
    if (k <= 0 || pat.n == 0) return;
    int chunk = kMaxChunk;
    if (k > 8 && spmm_tuning_on()) {
        const int p = spmm_tuned_split<T>(pat, val, X, ldx, Y, ldy, k, st, nullptr);
        chunk = (k + p - 1) / p;
    }
    spmm_split(pat, val, X, ldx, Y, ldy, k, chunk, st);
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
template int spmm_tuned_split<double>(const SellPattern &, const double *, const double *, int,
                                      double *, int, int, cudaStream_t, std::vector<double> *);
template int spmm_tuned_split<float>(const SellPattern &, const float *, const float *, int,
                                     float *, int, int, cudaStream_t, std::vector<double> *);
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
