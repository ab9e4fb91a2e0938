// GCGE_GramNoAlloc: the tall-skinny Gram product C = Q^T P without any memory
// allocation.  The split-K partial sums that the library's Gram kernel needs
// live in a fixed device array declared at file scope below, instead of in
// memory the library or the caller allocates.
//
// Who needs this: callers that are not allowed to call cudaMalloc/cudaFree -
// code whose device memory is owned by another allocator or by a pre-sized
// pool (a host framework that forbids raw device allocations), and
// latency-critical loops in which an allocation, which may synchronise the
// device, is not acceptable.  They pass device pointers for Q, P and C and get
// the product with two kernel launches and nothing else.
//
// Limits and sharing:
//  * the scratch array holds GCGE_NOALLOC_SCRATCH_BYTES (4 MiB); m * w must not
//    exceed that many doubles (m*w <= 524288), larger requests are rejected
//    with GCGE_ERR_TOO_LARGE before anything is launched;
//  * every GPU that loads the library keeps the array until the process exits;
//  * all calls on a device share the one array: calls whose kernels overlap on
//    the GPU (different streams, or different host threads, without ordering
//    between them) race on it and give wrong results.  Calls on one stream are
//    ordered and safe.  Nothing has to start at zero: each call writes every
//    partial sum it later reads;
//  * the device address of the array is looked up (cudaGetSymbolAddress) by the
//    first call on each device, with that device current, and cached; that
//    first call should therefore come before any stream capture.
#include <mutex>

#include "common.cuh"

namespace gcge {
// Gram kernels of dense.cu: row-chunk partial tiles, then a fixed-order sum.
__global__ void __launch_bounds__(256)
k_gram(int n, int m, int w, const double *__restrict__ Q, int ldq, const double *__restrict__ P,
       int ldp, double *__restrict__ part, int rows_per_chunk);
__global__ void k_reduce_chunks(const double *__restrict__ part, int chunks, int m, int w,
                                double *__restrict__ C, int ldc);
}  // namespace gcge

namespace {

constexpr size_t kScratchDoubles = GCGE_NOALLOC_SCRATCH_BYTES / sizeof(double);
constexpr int kMaxDevices = gcge::kMaxDevices;
constexpr int kTile = 32;

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

std::mutex g_mu;
double *g_scratch_ptr[kMaxDevices] = {};
int g_sms[kMaxDevices] = {};

// Device address of the scratch array and the SM count of the current device
// (both set up once per device, on its first call).
int scratch_for_current_device(double **out, int *sms) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        gcge::set_error(GCGE_ERR_CUDA, cudaGetErrorString(e));
        return GCGE_ERR_CUDA;
    }
    if (dev < 0 || dev >= kMaxDevices) {
        gcge::set_error(GCGE_ERR_ARG, "GCGE_GramNoAlloc: device index out of range");
        return GCGE_ERR_ARG;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    if (g_scratch_ptr[dev] == nullptr) {
        double *p = nullptr;
        e = cudaGetSymbolAddress((void **)&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr) {
            gcge::set_error(GCGE_ERR_CUDA, "GCGE_GramNoAlloc: cudaGetSymbolAddress failed");
            return GCGE_ERR_CUDA;
        }
        int count = 0;
        e = cudaDeviceGetAttribute(&count, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess || count <= 0) {
            gcge::set_error(GCGE_ERR_CUDA, "GCGE_GramNoAlloc: SM count query failed");
            return GCGE_ERR_CUDA;
        }
        g_sms[dev] = count;
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    *sms = g_sms[dev];
    return GCGE_OK;
}

}  // namespace

extern "C" int GCGE_GramNoAlloc(int n, int m, int w, const double *Q, int ldq, const double *P,
                                int ldp, double *C, int ldc, void *stream) {
    if (n < 0 || m < 1 || w < 1 || C == nullptr || ldc < m ||
        (n > 0 && (Q == nullptr || P == nullptr || ldq < n || ldp < n))) {
        gcge::set_error(GCGE_ERR_ARG, "GCGE_GramNoAlloc: invalid sizes or pointers");
        return GCGE_ERR_ARG;
    }
    if ((size_t)m * (size_t)w > kScratchDoubles) {
        gcge::set_error(GCGE_ERR_TOO_LARGE,
                        "GCGE_GramNoAlloc: m*w exceeds the 4 MiB scratch (524288 doubles)");
        return GCGE_ERR_TOO_LARGE;
    }
    double *scratch = nullptr;
    int sms = 0;
    int st = scratch_for_current_device(&scratch, &sms);
    if (st != GCGE_OK) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (n == 0) {
        cudaError_t e = cudaMemset2DAsync(C, sizeof(double) * ldc, 0, sizeof(double) * m, w, s);
        if (e != cudaSuccess) {
            gcge::set_error(GCGE_ERR_CUDA, cudaGetErrorString(e));
            return GCGE_ERR_CUDA;
        }
        return GCGE_OK;
    }
    const int tiles = ((m + kTile - 1) / kTile) * ((w + kTile - 1) / kTile);
    long long chunks = std::max(1, (3 * sms + tiles - 1) / tiles);
    chunks = std::min<long long>(chunks, std::max(1, (n + 127) / 128));
    chunks = std::min<long long>(chunks, (long long)(kScratchDoubles / ((size_t)m * w)));
    chunks = std::max<long long>(chunks, 1);
    int rpc = (int)((n + chunks - 1) / chunks);
    rpc = (rpc + kTile - 1) / kTile * kTile;
    const int nchunks = (n + rpc - 1) / rpc;
    const dim3 grid(nchunks, (m + kTile - 1) / kTile, (w + kTile - 1) / kTile);
    gcge::k_gram<<<grid, 256, 0, s>>>(n, m, w, Q, ldq, P, ldp, scratch, rpc);
    const int tot = m * w;
    gcge::k_reduce_chunks<<<std::max(1, std::min((tot + 255) / 256, 4 * sms)), 256, 0, s>>>(
        scratch, nchunks, m, w, C, ldc);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        gcge::set_error(GCGE_ERR_CUDA, cudaGetErrorString(e));
        return GCGE_ERR_CUDA;
    }
    gcge::count_launch(2);
    return GCGE_OK;
}
