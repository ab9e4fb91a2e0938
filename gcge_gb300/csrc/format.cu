// Sparse formats built on the device: the CCS input of a square matrix
// (app/app_ccs.h:20-24, as CUDA_MatCreateFromCCS and GCGE_Solve receive it) is
// uploaded as is, transposed to CSR with rows sorted by column, merged with a
// second matrix into the union pattern of the shifted PCG operator
// (A + sigma B, the reference's in-place MatAxpby branch,
// src/ops_eig_sol_gcg.c:600-608), and laid out as SELL-32.  Only the raw
// arrays cross PCIe/C2C; every per-row pass runs as a kernel, so the set-up of
// a solve costs a few milliseconds instead of host loops over every entry.
//
// Determinism: the transpose places entries with atomic row cursors and then
// sorts every row by (column, value bits), so the CSR (and everything built
// from it) is the same on every run.
#include <algorithm>

#include "common.cuh"

namespace gcge {
namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;  // per thread: a block scans 2048 entries
constexpr int kScanTile = kScanThreads * kScanItems;

// Exclusive scan of in[0..n) into out[0..n] (out[n] = total), in three
// passes: tile sums, a single-block scan of the tile sums, tile scans with
// their offsets.
template <typename T>
__global__ void k_tile_sums(const T *__restrict__ in, long long n, long long *__restrict__ sums) {
    __shared__ long long red[kScanThreads];
    const long long base = (long long)blockIdx.x * kScanTile;
    long long s = 0;
    for (int i = 0; i < kScanItems; ++i) {
        const long long k = base + (long long)i * kScanThreads + threadIdx.x;
        if (k < n) s += (long long)in[k];
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = kScanThreads / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) sums[blockIdx.x] = red[0];
}

__global__ void k_scan_sums(long long *sums, long long m) {
    __shared__ long long buf[1024];
    __shared__ long long carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (long long c0 = 0; c0 < m; c0 += 1024) {
        const long long k = c0 + threadIdx.x;
        const long long v = k < m ? sums[k] : 0;
        buf[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < 1024; o <<= 1) {
            const long long t = threadIdx.x >= o ? buf[threadIdx.x - o] : 0;
            __syncthreads();
            buf[threadIdx.x] += t;
            __syncthreads();
        }
        if (k < m) sums[k] = carry + buf[threadIdx.x] - v;  // exclusive
        __syncthreads();
        if (threadIdx.x == 1023) carry += buf[1023];
        __syncthreads();
    }
}

template <typename T, typename O>
__global__ void k_tile_scan(const T *__restrict__ in, long long n, const long long *__restrict__ offs,
                            O *__restrict__ out) {
    __shared__ long long part[kScanThreads];
    const long long base = (long long)blockIdx.x * kScanTile + (long long)threadIdx.x * kScanItems;
    long long v[kScanItems];
    long long mine = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        const long long k = base + i;
        v[i] = k < n ? (long long)in[k] : 0;
        mine += v[i];
    }
    part[threadIdx.x] = mine;
    __syncthreads();
    for (int o = 1; o < kScanThreads; o <<= 1) {  // inclusive Hillis-Steele scan of thread sums
        const long long t = threadIdx.x >= o ? part[threadIdx.x - o] : 0;
        __syncthreads();
        part[threadIdx.x] += t;
        __syncthreads();
    }
    long long run = offs[blockIdx.x] + part[threadIdx.x] - mine;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        const long long k = base + i;
        if (k < n) out[k] = (O)run;
        run += v[i];
        if (k == n - 1) out[n] = (O)run;
    }
}

// Exclusive scan with total: out has n + 1 entries.  Returns the total
// (synchronises once to read it).
template <typename T, typename O>
long long exclusive_scan(const T *in, long long n, O *out, cudaStream_t st) {
    if (n <= 0) {
        GCGE_CUDA(cudaMemsetAsync(out, 0, sizeof(O), st));
        return 0;
    }
    const long long tiles = (n + kScanTile - 1) / kScanTile;
    DevBuf<long long> sums;
    sums.alloc(tiles);
    k_tile_sums<T><<<(unsigned)tiles, kScanThreads, 0, st>>>(in, n, sums.p);
    GCGE_CHECK_LAUNCH();
    k_scan_sums<<<1, 1024, 0, st>>>(sums.p, tiles);
    GCGE_CHECK_LAUNCH();
    k_tile_scan<T, O><<<(unsigned)tiles, kScanThreads, 0, st>>>(in, n, sums.p, out);
    GCGE_CHECK_LAUNCH();
    count_launch(3);
    O total = 0;
    GCGE_CUDA(cudaMemcpyAsync(&total, out + n, sizeof(O), cudaMemcpyDeviceToHost, st));
    GCGE_CUDA(cudaStreamSynchronize(st));
    return (long long)total;
}

// ---------------------------------------------------------------- CCS -> CSR
__global__ void k_ccs_count(int n, long long nnz, const int *__restrict__ rowind,
                            int *__restrict__ cnt, int *__restrict__ bad) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nnz;
         e += (long long)gridDim.x * blockDim.x) {
        const int r = rowind[e];
        if (r < 0 || r >= n) {
            atomicExch(bad, 1);
            continue;
        }
        atomicAdd(&cnt[r], 1);
    }
}

__global__ void k_ccs_place(int n, const int *__restrict__ colptr, const int *__restrict__ rowind,
                            const double *__restrict__ val, const int *__restrict__ ptr,
                            int *__restrict__ cursor, int *__restrict__ ind,
                            double *__restrict__ oval) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        for (int e = colptr[j]; e < colptr[j + 1]; ++e) {
            const int r = rowind[e];
            const int pos = ptr[r] + atomicAdd(&cursor[r], 1);
            ind[pos] = j;
            oval[pos] = val[e];
        }
    }
}

// sort every row by (column, value bits): insertion sort, thread per row
__global__ void k_row_sort(int n, const int *__restrict__ ptr, int *__restrict__ ind,
                           double *__restrict__ val) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        const int b = ptr[r], e = ptr[r + 1];
        for (int i = b + 1; i < e; ++i) {
            const int c = ind[i];
            const double v = val[i];
            const long long vb = __double_as_longlong(v);
            int k = i - 1;
            while (k >= b && (ind[k] > c || (ind[k] == c && __double_as_longlong(val[k]) > vb))) {
                ind[k + 1] = ind[k];
                val[k + 1] = val[k];
                --k;
            }
            ind[k + 1] = c;
            val[k + 1] = v;
        }
    }
}

// ---------------------------------------------------------------- union
// Row r of the union of A's and B's patterns and the diagonal, with A's and
// B's values on it (B == null: the identity).  Pass 1 counts, pass 2 writes.
template <bool WRITE>
__global__ void k_union(int n, const int *__restrict__ ap, const int *__restrict__ ai,
                        const double *__restrict__ av, const int *__restrict__ bp,
                        const int *__restrict__ bi, const double *__restrict__ bvv,
                        int *__restrict__ cnt, const int *__restrict__ up, int *__restrict__ ui,
                        double *__restrict__ ua, double *__restrict__ ub) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        int ka = ap[r];
        const int ea = ap[r + 1];
        int kb = bp ? bp[r] : 0;
        const int eb = bp ? bp[r + 1] : 0;
        bool diag = false;  // diagonal emitted
        int out = WRITE ? up[r] : 0;
        int count = 0;
        while (true) {
            const int ca = ka < ea ? ai[ka] : 0x7FFFFFFF;
            const int cb = bp ? (kb < eb ? bi[kb] : 0x7FFFFFFF) : (diag ? 0x7FFFFFFF : r);
            const int cd = diag ? 0x7FFFFFFF : r;
            const int c = min(ca, min(cb, cd));
            if (c == 0x7FFFFFFF) break;
            double va = 0.0, vb = 0.0;
            while (ka < ea && ai[ka] == c) va += av[ka++];
            if (bp) {
                while (kb < eb && bi[kb] == c) vb += bvv[kb++];
            } else if (c == r) {
                vb = 1.0;
            }
            if (c == r) diag = true;
            if (WRITE) {
                ui[out] = c;
                ua[out] = va;
                ub[out] = vb;
                ++out;
            }
            ++count;
        }
        if (!WRITE) cnt[r] = count;
    }
}

// ---------------------------------------------------------------- SELL
__global__ void k_slice_width(int n, int nslices, const int *__restrict__ ptr,
                              long long *__restrict__ w32) {
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nslices; s += gridDim.x * blockDim.x) {
        int w = 0;
        for (int l = 0; l < 32; ++l) {
            const int r = s * 32 + l;
            if (r < n) w = max(w, ptr[r + 1] - ptr[r]);
        }
        w32[s] = (long long)w * 32;
    }
}

// entry e of row r -> slice_ptr[r / 32] + e * 32 + r % 32; padding: own row
// (clamped to n - 1), value 0
__global__ void k_sell_fill(int n, int nslices, const int *__restrict__ ptr,
                            const int *__restrict__ ind, const double *__restrict__ v0,
                            const double *__restrict__ v1, const long long *__restrict__ sp,
                            int *__restrict__ col, double *__restrict__ o0, double *__restrict__ o1) {
    const long long rows = (long long)nslices * 32;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < rows;
         t += (long long)gridDim.x * blockDim.x) {
        const int r = (int)t, s = r >> 5, l = r & 31;
        const int width = (int)((sp[s + 1] - sp[s]) >> 5);
        const int b = r < n ? ptr[r] : 0;
        const int len = r < n ? ptr[r + 1] - b : 0;
        const int own = r < n ? r : n - 1;
        for (int e = 0; e < width; ++e) {
            const long long pos = sp[s] + (long long)e * 32 + l;
            if (e < len) {
                col[pos] = ind[b + e];
                o0[pos] = v0[b + e];
                if (o1) o1[pos] = v1[b + e];
            } else {
                col[pos] = own;
                o0[pos] = 0.0;
                if (o1) o1[pos] = 0.0;
            }
        }
    }
}

int grid_for(long long work, int threads) {
    return (int)std::max<long long>(1, std::min<long long>((work + threads - 1) / threads, 1 << 16));
}

}  // namespace

void csr_from_ccs_device(int n, const int *h_colptr, const int *h_rowind, const double *h_val,
                         DevCsr &out, cudaStream_t st) {
    const long long nnz = h_colptr[n];
    out.n = n;
    out.nnz = nnz;
    out.ptr.alloc((size_t)n + 1);
    out.ind.alloc(std::max<long long>(nnz, 1));
    out.val.alloc(std::max<long long>(nnz, 1));
    DevBuf<int> cp, ri, cnt, bad;
    DevBuf<double> rv;
    cp.alloc((size_t)n + 1);
    ri.alloc(std::max<long long>(nnz, 1));
    rv.alloc(std::max<long long>(nnz, 1));
    cnt.alloc((size_t)n);
    bad.alloc(1);
    GCGE_CUDA(cudaMemcpyAsync(cp.p, h_colptr, sizeof(int) * ((size_t)n + 1), cudaMemcpyHostToDevice, st));
    if (nnz > 0) {
        GCGE_CUDA(cudaMemcpyAsync(ri.p, h_rowind, sizeof(int) * nnz, cudaMemcpyHostToDevice, st));
        GCGE_CUDA(cudaMemcpyAsync(rv.p, h_val, sizeof(double) * nnz, cudaMemcpyHostToDevice, st));
    }
    GCGE_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(int) * n, st));
    GCGE_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(int), st));
    k_ccs_count<<<grid_for(nnz, 256), 256, 0, st>>>(n, nnz, ri.p, cnt.p, bad.p);
    GCGE_CHECK_LAUNCH();
    count_launch();
    int h_bad = 0;
    GCGE_CUDA(cudaMemcpyAsync(&h_bad, bad.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    exclusive_scan<int, int>(cnt.p, n, out.ptr.p, st);  // synchronises
    GCGE_REQUIRE(h_bad == 0, GCGE_ERR_ARG, "CUDA_MatCreateFromCCS: row index out of range");
    GCGE_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(int) * n, st));
    k_ccs_place<<<grid_for(n, 256), 256, 0, st>>>(n, cp.p, ri.p, rv.p, out.ptr.p, cnt.p, out.ind.p,
                                                   out.val.p);
    GCGE_CHECK_LAUNCH();
    k_row_sort<<<grid_for(n, 256), 256, 0, st>>>(n, out.ptr.p, out.ind.p, out.val.p);
    GCGE_CHECK_LAUNCH();
    count_launch(2);
    GCGE_CUDA(cudaStreamSynchronize(st));  // the staging buffers are freed on return
}

void union_csr_device(const DevCsr &A, const DevCsr *B, DevCsr &U, DevBuf<double> &ub,
                      cudaStream_t st) {
    const int n = A.n;
    DevBuf<int> cnt;
    cnt.alloc((size_t)n);
    U.n = n;
    U.ptr.alloc((size_t)n + 1);
    const int *bp = B ? B->ptr.p : nullptr;
    const int *bi = B ? B->ind.p : nullptr;
    const double *bvv = B ? B->val.p : nullptr;
    k_union<false><<<grid_for(n, 256), 256, 0, st>>>(n, A.ptr.p, A.ind.p, A.val.p, bp, bi, bvv,
                                                       cnt.p, nullptr, nullptr, nullptr, nullptr);
    GCGE_CHECK_LAUNCH();
    count_launch();
    U.nnz = exclusive_scan<int, int>(cnt.p, n, U.ptr.p, st);
    U.ind.alloc(std::max<long long>(U.nnz, 1));
    U.val.alloc(std::max<long long>(U.nnz, 1));
    ub.alloc(std::max<long long>(U.nnz, 1));
    k_union<true><<<grid_for(n, 256), 256, 0, st>>>(n, A.ptr.p, A.ind.p, A.val.p, bp, bi, bvv,
                                                      nullptr, U.ptr.p, U.ind.p, U.val.p, ub.p);
    GCGE_CHECK_LAUNCH();
    count_launch();
}

void sell_from_csr_device(const DevCsr &M, const double *second, SellPattern &pat,
                          DevBuf<double> &v0, DevBuf<double> *v1, cudaStream_t st) {
    const int n = M.n, ns = (n + 31) / 32;
    pat.n = n;
    pat.nslices = ns;
    pat.nnz = M.nnz;
    pat.slice_ptr.alloc((size_t)ns + 1);
    DevBuf<long long> w32;
    w32.alloc(std::max(ns, 1));
    k_slice_width<<<grid_for(ns, 256), 256, 0, st>>>(n, ns, M.ptr.p, w32.p);
    GCGE_CHECK_LAUNCH();
    count_launch();
    pat.padded = exclusive_scan<long long, long long>(w32.p, ns, pat.slice_ptr.p, st);
    const size_t P = std::max<long long>(pat.padded, 1);
    pat.col.alloc(P);
    v0.alloc(P);
    if (v1) v1->alloc(P);
    k_sell_fill<<<grid_for((long long)ns * 32, 256), 256, 0, st>>>(
        n, ns, M.ptr.p, M.ind.p, M.val.p, second, pat.slice_ptr.p, pat.col.p, v0.p,
        v1 ? v1->p : nullptr);
    GCGE_CHECK_LAUNCH();
    count_launch();
}

}  // namespace gcge
