// Shared definitions of the GB300 GCGE library: status handling, device
// buffers, multivector / sparse-matrix objects and kernel launcher prototypes.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/gcge_cuda.h"

namespace gcge {

// ---------------------------------------------------------------- status
void set_error(int status, const char *where);
int take_error();
const char *status_string(int s);

struct CudaError {
    int status;
    std::string where;
};

// Throws CudaError on failure; every C-ABI entry point catches it and turns it
// into a status code, so no exception crosses the ABI.
#define GCGE_CUDA(call)                                                              \
    do {                                                                             \
        cudaError_t e_ = (call);                                                     \
        if (e_ != cudaSuccess) {                                                     \
            throw ::gcge::CudaError{GCGE_ERR_CUDA, std::string(#call) + ": " +         \
                                                       cudaGetErrorString(e_)};       \
        }                                                                            \
    } while (0)
#define GCGE_CHECK_LAUNCH() GCGE_CUDA(cudaGetLastError())
#define GCGE_REQUIRE(cond, status, msg)                                              \
    do {                                                                             \
        if (!(cond)) throw ::gcge::CudaError{(status), std::string(msg)};            \
    } while (0)

// Count of kernels launched by the library from the calling thread; the
// solver reports the difference over a solve (a solve runs on one thread).
extern thread_local unsigned long long t_kernel_launches;
inline void count_launch(int k = 1) { t_kernel_launches += (unsigned long long)k; }

// Devices a process may drive (indices of per-device caches).
constexpr int kMaxDevices = 64;
// The current device's index, validated; the first call on a device queries
// its attributes.  Throws GCGE_ERR_NO_DEVICE without a device.
int current_device();
// The calling thread's stream on the current device (created on first use,
// destroyed at thread exit): every kernel and copy of a solve runs on it, so
// solves driven from different host threads overlap on the device.
cudaStream_t lib_stream();
// Streaming multiprocessors of the current device (queried once per device).
int device_sms();
// A value computed once per device, on first use with that device current
// (kernel attributes, occupancy and cluster limits are per device).
template <typename T>
struct PerDevice {
    std::once_flag once[kMaxDevices];
    T value[kMaxDevices]{};
    template <typename F>
    T &get(F &&f) {
        const int d = current_device();
        std::call_once(once[d], [&] { value[d] = f(); });
        return value[d];
    }
};
// Number of solves sharing the device with the calling thread's solves (0 or
// 1: the whole device); the persistent block-PCG kernel then takes that share
// of the co-resident grid, so the cooperative kernels of concurrent solves
// always fit on the device together.  Set by the batch/serving workers.
extern thread_local int t_pcg_share;

// ---------------------------------------------------------------- buffers
// Device buffers come from the stream-ordered pool allocator on the calling
// thread's stream (no device-wide synchronisation, freed blocks reused).
template <typename T>
struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (p) {
            cudaStream_t st = nullptr;
            try {
                st = lib_stream();
            } catch (...) {
            }
            if (st) cudaFreeAsync(p, st);
            else cudaFree(p);
        }
        p = nullptr;
        n = 0;
    }
    // free on a given stream (teardown of a thread's per-device state)
    void release_on(cudaStream_t st) {
        if (p) cudaFreeAsync(p, st);
        p = nullptr;
        n = 0;
    }
    void alloc(size_t count) {
        if (count <= n && p) return;
        release();
        if (count == 0) return;
        cudaError_t e = cudaMallocAsync((void **)&p, count * sizeof(T), lib_stream());
        if (e != cudaSuccess) {
            p = nullptr;
            throw CudaError{GCGE_ERR_ALLOC, std::string("cudaMallocAsync: ") + cudaGetErrorString(e)};
        }
        n = count;
    }
    T *get() const { return p; }
};

template <typename T>
struct PinnedBuf {
    T *p = nullptr;
    size_t n = 0;
    PinnedBuf() = default;
    PinnedBuf(const PinnedBuf &) = delete;
    PinnedBuf &operator=(const PinnedBuf &) = delete;
    ~PinnedBuf() {
        if (p) cudaFreeHost(p);
    }
    void alloc(size_t count) {
        if (count <= n && p) return;
        if (p) cudaFreeHost(p);
        p = nullptr;
        n = 0;
        if (count == 0) return;
        GCGE_CUDA(cudaMallocHost((void **)&p, count * sizeof(T)));
        n = count;
    }
};

// Staging buffers of the OPS slots that move coefficients and inner products
// across the host boundary (MultiVecLinearComb, MultiVecInnerProd).  One set
// per host thread and device (slot_stage()), so slots called concurrently from
// several threads, or on several devices, never share a buffer.
struct SlotStage {
    DevBuf<double> dcoef, dbeta, dres, scr;
    PinnedBuf<double> hstage, hres;
    // exponent fields of the tensor-core digit products' operands (ozaki_tc.cu)
    DevBuf<int> tc_exps;
    void release_on(cudaStream_t st);
};
SlotStage &slot_stage();

// ---------------------------------------------------------------- objects
constexpr uint32_t kMultiVecMagic = 0x4D564755u;  // multivector
constexpr uint32_t kMatMagic = 0x4D544755u;       // sparse matrix

// Column-major multivector in HBM: column c starts at data + c * ld.
// ld is nrows rounded up to 32 elements so every column is 256-byte aligned.
struct MultiVec {
    uint32_t magic = kMultiVecMagic;
    int nrows = 0, ncols = 0, ld = 0;
    double *data = nullptr;
    bool owns = true;
};

// SELL-32 (sliced ELLPACK, slice height 32 = one warp) sparsity pattern with
// one or more value arrays in the same padded order.  Entry e of row r lives
// at slice_ptr[r / 32] + e * 32 + r % 32; padding entries repeat the row's own
// column index with a zero value, so every index is in range.
struct SellPattern {
    int n = 0;
    int nslices = 0;
    long long nnz = 0;      // true nonzeros
    long long padded = 0;   // stored entries
    DevBuf<long long> slice_ptr;
    DevBuf<int> col;
};

// CSR on the device, rows sorted by column (format.cu).
struct DevCsr {
    int n = 0;
    long long nnz = 0;
    DevBuf<int> ptr, ind;
    DevBuf<double> val;
};

struct SparseMat {
    uint32_t magic = kMatMagic;
    unsigned long long serial = 0;  // unique per created matrix
    int n = 0;
    long long nnz = 0;
    DevCsr csr;              // y = A x orientation, rows sorted
    SellPattern pat;
    DevBuf<double> val;      // FP64 values in SELL order
};

MultiVec *as_mv(void *h);
SparseMat *as_mat(void *h);

// Device-side formats (format.cu).  csr_from_ccs_device uploads a CCS matrix
// (column pointers, row indices, values on the host) and transposes it to CSR;
// union_csr_device merges A's and B's patterns and the diagonal (B null: the
// identity) with A's values in U.val and B's in ub; sell_from_csr_device lays
// a CSR (and optionally a second value array in the same order) out as SELL-32.
void csr_from_ccs_device(int n, const int *h_colptr, const int *h_rowind, const double *h_val,
                         DevCsr &out, cudaStream_t st);
void union_csr_device(const DevCsr &A, const DevCsr *B, DevCsr &U, DevBuf<double> &ub,
                      cudaStream_t st);
void sell_from_csr_device(const DevCsr &M, const double *second, SellPattern &pat,
                          DevBuf<double> &v0, DevBuf<double> *v1, cudaStream_t st);


// ---------------------------------------------------------------- launchers
// Sparse (spmm.cu).  X, Y column-major with leading dimensions; k columns.
template <typename T>
void spmm(const SellPattern &pat, const T *val, const T *X, int ldx, T *Y, int ldy, int k,
          cudaStream_t st);
// partial[block*kmax+c] = sum over the block's rows of r^2 with r = (A - lam_c B) x_c
int residual_norms(const SellPattern &pa, const double *va, const SellPattern *pb,
                   const double *vb, const double *X, int ldx, const double *lam, int k,
                   double *partial, int kmax, cudaStream_t st, double *ax = nullptr,
                   double *bx = nullptr, int ldo = 0);
int spmm_blocks(const SellPattern &pat);
// Column-split tuner of spmm (spmm.cu): candidate launch counts p for k
// columns (each launch ceil(k / p) columns), the switch (initially from the
// environment variable GCGE_SPMM_TUNE), the cache reset, and the tuned p for
// a call (timing every candidate when ms_out is given).
std::vector<int> spmm_split_candidates(int k);
bool spmm_tuning_on();
void set_spmm_tuning(bool on);
void clear_spmm_tuning();
template <typename T>
int spmm_tuned_split(const SellPattern &pat, const T *val, const T *X, int ldx, T *Y, int ldy,
                     int k, cudaStream_t st, std::vector<double> *ms_out);
// Smallest block-PCG row width >= k (whole 16-byte column groups).
int rows_width(int k, int elem_bytes);


// Dense (dense.cu).
void axpby(int n, int ncols, double alpha, const double *X, int ldx, double beta, double *Y,
           int ldy, cudaStream_t st);
void axpby_f32(int n, int ncols, float alpha, const float *X, int ldx, float beta, float *Y,
               int ldy, cudaStream_t st);
// Y(:, j) = alpha sum_l X(:, l) C(l, j) + beta_j Y(:, j); beta == nullptr -> 0,
// incb == 0 -> scalar *beta.  C on the device.
void lincomb(int n, int k, int m, const double *X, int ldx, const double *C, int ldc, double *Y,
             int ldy, const double *beta_dev, int incb, cudaStream_t st, double alpha = 1.0);
// C(m x w) = Q^T P over n rows; result written to C (device, ldc).
void gram(int n, int m, int w, const double *Q, int ldq, const double *P, int ldp, double *C,
          int ldc, double *scratch, size_t scratch_elems, cudaStream_t st);
size_t gram_scratch_elems(int n, int m, int w);
// Exponent fields of one digit-product operand (the Gram's left operand over
// its row windows, or a linear combination's rows over its columns), kept
// across calls that pass the same unchanged operand with the same shape.  The
// caller owns the scope: it must drop the cache (or let it go out of scope)
// before the operand's values change.
struct TcExpCache {
    const double *ptr = nullptr;
    size_t ld = 0;
    int rows = 0, cols = 0, window = 0, kind = -1;
    DevBuf<int> e;
    bool matches(const double *p, size_t l, int r, int c, int w, int k) const {
        return kind == k && ptr == p && ld == l && rows == r && cols == c && window == w;
    }
    void set(const double *p, size_t l, int r, int c, int w, int k) {
        ptr = p, ld = l, rows = r, cols = c, window = w, kind = k;
    }
};
// FP64-accurate products on the bf16 tensor cores (ozaki.cu): same arguments
// and results as gram / lincomb, to FP64 accuracy.  `cache` (optional) keeps
// the exponent fields of Q (Gram) or X (linear combination) between calls.
void oz_gram(int n, int m, int w, const double *Q, int ldq, const double *P, int ldp, double *C,
             int ldc, double *scratch, size_t scratch_elems, cudaStream_t st,
             TcExpCache *cache = nullptr);
void oz_lincomb(int n, int k, int m, const double *X, int ldx, const double *C, int ldc,
                double *Y, int ldy, const double *beta_dev, int incb, cudaStream_t st,
                double alpha,
                void *scratch, size_t scratch_bytes, TcExpCache *cache = nullptr);
// Scratch bytes oz_lincomb needs for k terms and m columns.
size_t oz_lincomb_scratch_bytes(int k, int m);
// The same products on the 5th-generation tensor cores (ozaki_tc.cu:
// tcgen05.mma with accumulators in tensor memory), same arguments and
// results; oz_gram / oz_lincomb use them where tc_digits_available().
bool tc_digits_available();
void tc_gram(int n, int m, int w, const double *Q, int ldq, const double *P, int ldp, double *C,
             int ldc, double *scratch, size_t scratch_elems, cudaStream_t st,
             TcExpCache *cache = nullptr);
void tc_lincomb(int n, int k, int m, const double *X, int ldx, const double *C, int ldc,
                double *Y, int ldy, const double *beta_dev, int incb, cudaStream_t st,
                double alpha, void *scratch, size_t scratch_bytes, TcExpCache *cache = nullptr);
size_t tc_lincomb_scratch_bytes(int k, int m);
// Throws GCGE_ERR_CUDA (and clears the flag) if a tensor-core product's
// bounded wait ran out since the last check (synchronises the stream).
void tc_check_error(cudaStream_t st);
// per-column dots out[c] = X(:,c) . Y(:,c)
void coldot(int n, int k, const double *X, int ldx, const double *Y, int ldy, double *out,
            double *scratch, size_t scratch_elems, cudaStream_t st);
// out[c] = sum_b partial[b * kmax + c]  (fixed order, deterministic)
void reduce_partials(const double *partial, int nblocks, int kmax, int k, double *out,
                     cudaStream_t st);
void scale_columns(int n, int k, double *X, int ldx, const double *s, cudaStream_t st);
void copy_f64_to_f32(int n, int k, const double *X, int ldx, float *Y, int ldy, cudaStream_t st);
void copy_f32_to_f64(int n, int k, const float *X, int ldx, double *Y, int ldy, cudaStream_t st);
// Y += X (FP32 correction accumulated into an FP64 block)
void add_f32_to_f64(int n, int k, const float *X, int ldx, double *Y, int ldy, cudaStream_t st);
void fill_uniform(int n, int k, double *X, int ldx, unsigned long long seed, cudaStream_t st);
void gather_columns(int n, int k, const double *X, int ldx, const int *idx, double *Y, int ldy,
                    cudaStream_t st);
void set_identity(int n, double *X, int ldx, cudaStream_t st);
void fill_value(size_t count, double *X, double v, cudaStream_t st);
void scale_columns_strided(int n, int m, double *Y, int ldy, const double *s, int inc,
                           cudaStream_t st);
// max |C(i,j)| over an m x w block (device) -> *out (device)
void absmax(int m, int w, const double *C, int ldc, double *out, cudaStream_t st);
// rows with mask[i] != 0 of an m x k block set to zero
void zero_rows(int m, int k, double *X, int ldx, const int *mask, cudaStream_t st);
// Y(i, j) = X(j, i) for an m x k block (X m x k -> Y k x m)
void transpose_copy(int m, int k, const double *X, int ldx, double *Y, int ldy, cudaStream_t st);
// y = a + sigma b over count entries, in double or float
void shift_values(size_t count, const double *a, const double *b, double sigma, double *y64,
                  float *y32, cudaStream_t st);
void copy_cols(int n, int k, const double *X, int ldx, double *Y, int ldy, cudaStream_t st);

}  // namespace gcge
