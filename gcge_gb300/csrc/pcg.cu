// Block conjugate gradient on (A + sigma B) x = b for all columns of a block
// at once (reference BlockPCG, src/ops_lin_sol.c:140-437).
//
// The whole solve is ONE persistent kernel launch (cooperative grid, or one
// thread-block cluster for small operators, below).  Each block
// owns a contiguous range of SELL slices (balanced by stored entries) and the
// rows they cover; the iteration runs in three phases separated by grid-wide
// barriers:
//   1. p = r + beta p                      (own rows; p = r on the first step)
//   2. w = S p, partial sums of p^T w      (warp per slice, gathers p rows)
//      -> the last block to arrive sums the partials: alpha = rho / p^T w
//   3. x += alpha p, r -= alpha w, partial sums of r^T r
//      -> the last block: residual norms, convergence test, beta, count
// so nothing returns to the host between iterations.  The reference keeps a
// compacted list of unconverged columns and runs one SpMM per contiguous run
// of them; here a per-column `active` flag plays that role: inactive columns
// keep x and r (alpha = 0), drop out of the sums, and a 16-byte group of
// columns that is wholly inactive is neither gathered nor updated.
//
// Cross-block sums are taken by one block in a fixed order, so results are
// deterministic for a given grid.  The shifted operator is one SELL matrix
// S = A + sigma B on the union pattern of A and B (the reference's in-place
// MatAxpby branch, src/ops_eig_sol_gcg.c:600-608), so each iteration streams
// one matrix.  Vectors are slice-blocked n x kp blocks (kp = k padded to 16
// bytes, G = kp / (16 / sizeof T) 16-byte column groups; for every 32-row
// slice, group u of its 32 rows is one contiguous 512-byte run): a lane owns
// a row and gathers a neighbour row as G 16-byte loads, and for a stencil the
// 32 lanes of a warp read one or two contiguous runs per load instead of 32
// scattered rows.  T = double (FP64 GCG) or float (mixed precision: FP32
// values and FP32 accumulation within a block; cross-block sums in double).
//
// Every barrier wait is bounded (time and poll count); a wait that runs out
// sets an error flag that makes all blocks return, and the host reports it.
//
// Operators of at most two slices per warp of one thread-block cluster (16
// CTAs, or 8) run the same kernel in its cluster form instead: the cluster's
// hardware barrier replaces the grid barrier, and every CTA sums the partials
// and updates its own copy of the scalars, so the per-step barrier cost drops
// from a few microseconds to well under one (small problems of batches and
// serving are bound by it).
#include <cooperative_groups.h>

#include <algorithm>
#include <mutex>
#include <type_traits>

#include "common.cuh"
#include "pcg.cuh"

namespace gcge {

namespace {

constexpr unsigned long long kBarrierTimeoutNs = 4000000000ull;  // 4 s
constexpr long long kBarrierMaxPolls = 1LL << 27;

// 16-byte packs of a slice-blocked block
template <typename T>
struct Pk;
template <>
struct Pk<float> {
    static constexpr int L = 4;
    float v[4];
    __device__ __forceinline__ static Pk ld(const float *p) {
        const float4 t = *reinterpret_cast<const float4 *>(p);
        return Pk{{t.x, t.y, t.z, t.w}};
    }
    __device__ __forceinline__ void st(float *p) const {
        *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
    }
};
template <>
struct Pk<double> {
    static constexpr int L = 2;
    double v[2];
    __device__ __forceinline__ static Pk ld(const double *p) {
        const double2 t = *reinterpret_cast<const double2 *>(p);
        return Pk{{t.x, t.y}};
    }
    __device__ __forceinline__ void st(double *p) const {
        *reinterpret_cast<double2 *>(p) = make_double2(v[0], v[1]);
    }
};

// Element offset of row i, 16-byte group u in a slice-blocked block of width KP.
template <typename T, int KP>
__device__ __forceinline__ size_t boff(int i, int u) {
    constexpr int L = Pk<T>::L, G = KP / L;
    return ((size_t)(i >> 5) * G + u) * (32 * L) + (size_t)(i & 31) * L;
}

// acc += sum over the lane's row of a slice of val[e] * X(col[e], :), e =
// e0 + 32 i, i < width: the column indices and values of the next kPrefetch
// entries are in flight while the current entry's 16-byte groups are gathered,
// so the gathers do not wait on the matrix stream.  Groups with ga[u] false
// are skipped.
constexpr int kPrefetch = 2;
template <typename T, int KP>
__device__ __forceinline__ void gather_row(const int *__restrict__ col, const T *__restrict__ val,
                                           long long e0, int width, const T *X,
                                           const bool (&ga)[KP / Pk<T>::L], T (&acc)[KP]) {
    constexpr int L = Pk<T>::L, G = KP / L;
    int jq[kPrefetch];
    T vq[kPrefetch];
#pragma unroll
    for (int d = 0; d < kPrefetch; ++d) {
        const bool in = d < width;
        jq[d] = in ? __ldg(col + e0 + 32LL * d) : 0;
        vq[d] = in ? __ldg(val + e0 + 32LL * d) : T(0);
    }
#pragma unroll 1
    for (int e = 0; e < width; ++e) {
        const int j = jq[0];
        const T v = vq[0];
#pragma unroll
        for (int d = 0; d + 1 < kPrefetch; ++d) {
            jq[d] = jq[d + 1];
            vq[d] = vq[d + 1];
        }
        const int en = e + kPrefetch;
        jq[kPrefetch - 1] = en < width ? __ldg(col + e0 + 32LL * en) : 0;
        vq[kPrefetch - 1] = en < width ? __ldg(val + e0 + 32LL * en) : T(0);
#pragma unroll
        for (int u = 0; u < G; ++u) {
            if (!ga[u]) continue;
            const Pk<T> x = Pk<T>::ld(X + boff<T, KP>(j, u));
#pragma unroll
            for (int q = 0; q < L; ++q) acc[u * L + q] = fma(v, x.v[q], acc[u * L + q]);
        }
    }
}

// The same sum for the NU column groups [U0, U0 + NU) only (all of them,
// active or not), two matrix entries at a time (both entries' loads in
// flight before their FMAs): the SpMM phase of wide blocks gathers a row in
// two such halves, so that the accumulators of one half leave registers for
// the second entry's loads (4.87 -> 4.75 s of inner solve per 128^3 solve;
// four entries at a time: 4.81 s).
template <typename T, int KP, int U0, int NU, int NE>
__device__ __forceinline__ void gather_entries(const int *__restrict__ col,
                                               const T *__restrict__ val, long long e0, int e,
                                               const T *X, T (&acc)[NU * Pk<T>::L]) {
    constexpr int L = Pk<T>::L;
    int j[NE];
    T v[NE];
#pragma unroll
    for (int d = 0; d < NE; ++d) {
        j[d] = __ldg(col + e0 + 32LL * (e + d));
        v[d] = __ldg(val + e0 + 32LL * (e + d));
    }
    Pk<T> x[NE][NU];
#pragma unroll
    for (int d = 0; d < NE; ++d)
#pragma unroll
        for (int u = 0; u < NU; ++u) x[d][u] = Pk<T>::ld(X + boff<T, KP>(j[d], U0 + u));
#pragma unroll
    for (int d = 0; d < NE; ++d)
#pragma unroll
        for (int u = 0; u < NU; ++u)
#pragma unroll
            for (int q = 0; q < L; ++q) acc[u * L + q] = fma(v[d], x[d][u].v[q], acc[u * L + q]);
}
template <typename T, int KP, int U0, int NU>
__device__ __forceinline__ void gather_row_part(const int *__restrict__ col,
                                                const T *__restrict__ val, long long e0,
                                                int width, const T *X, T (&acc)[NU * Pk<T>::L]) {
    int e = 0;
#pragma unroll 1
    for (; e + 1 < width; e += 2) gather_entries<T, KP, U0, NU, 2>(col, val, e0, e, X, acc);
    if (e < width) gather_entries<T, KP, U0, NU, 1>(col, val, e0, e, X, acc);
}

__device__ __forceinline__ unsigned long long ld_acquire(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(unsigned long long *p, unsigned long long v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Grid-wide barrier number `epoch` (1, 2, ...).  The last block to arrive runs
// `last` with all its threads before it releases the others, so the
// cross-block reductions are done once.  Returns false when the wait ran out
// (or another block's did); the caller then returns.
template <typename F>
__device__ __forceinline__ bool grid_sync(PcgSync *gs, int *error, unsigned long long timeout_ns,
                                          long long max_polls, unsigned long long epoch,
                                          F &&last) {
    __shared__ int s_last, s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned long long old = atomicAdd(&gs->arrive, 1ull);
        const int lst = old + 1ull == epoch * gridDim.x;
        if (lst) __threadfence();
        s_last = lst;
        s_ok = 1;
    }
    __syncthreads();
    if (s_last) {
        last();
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            st_release(&gs->release, epoch);
        }
    } else if (threadIdx.x == 0) {
        const unsigned long long t0 = global_ns();
        for (long long poll = 0; ld_acquire(&gs->release) < epoch; ++poll) {
            if ((poll & 31) == 31 &&
                (*(volatile int *)error != 0 || poll > max_polls ||
                 global_ns() - t0 > timeout_ns)) {
                atomicExch(error, 1);
                s_ok = 0;
                break;
            }
            __nanosleep(32);
        }
    }
    __syncthreads();
    return s_ok != 0;
}

// The barrier of the cluster form (CL): one thread-block cluster runs the
// solve, each CTA keeps its own copy of the scalars in shared memory and runs
// `last` itself after a cluster barrier (the CTAs read the same partials in
// the same order, so the copies agree).  No wait can run out: the barrier is
// the hardware's.
template <bool CL, typename F>
__device__ __forceinline__ bool pcg_sync(PcgSync *gs, int *error, unsigned long long timeout_ns,
                                         long long max_polls, unsigned long long epoch,
                                         F &&last) {
    if constexpr (CL) {
        cooperative_groups::this_cluster().sync();
        last();
        __syncthreads();
        return true;
    } else {
        return grid_sync(gs, error, timeout_ns, max_polls, epoch, last);
    }
}

template <typename T>
struct PcgArgs {
    const long long *sp;
    const int *col;
    const T *val;
    int n, nslices;
    const T *B;
    T *X, *R, *P, *W;
    int k, max_iter, rel_tol, x_zero;
    double rate, tol;
    double matrix_bytes;  // nnz (v + 4) + 4 (n + 1) of S
    PcgScalars *sc;
    PcgSync *sync;
    PcgStats *stats;
    double *part;  // 2 x gridDim.x x KP
    // bound of every grid-barrier wait (device clock and poll count)
    unsigned long long timeout_ns;
    long long max_polls;
    // failure-detection test only: the grid's last block returns before its
    // first barrier, so the others' waits run out (never set otherwise)
    int withhold_last;
};

// Compiler-only ordering point between the 16-byte groups of a row in the
// streaming phases: keeps one group's loads in flight per thread instead of
// all of them, which bounds the registers (warps supply the parallelism).
__device__ __forceinline__ void group_fence() { asm volatile("" ::: "memory"); }

__host__ __device__ constexpr int pow2ceil(int x) {
    int p = 1;
    while (p < x) p <<= 1;
    return p;
}

// Warp sums of N per-lane column values (N a power of two <= 32): returns, in
// lane l, the sum over the 32 lanes of column l % N.  The first steps add
// whole vectors across lanes that differ in high bits; the last log2(N) steps
// exchange halves (a transposing butterfly), so N = 32 columns take 31
// shuffles instead of 160.
template <typename T, int N>
__device__ __forceinline__ T warp_cols_reduce(T (&v)[N], int lane) {
#pragma unroll
    for (int o = 16; o >= N; o >>= 1) {
#pragma unroll
        for (int i = 0; i < N; ++i) v[i] += __shfl_xor_sync(0xffffffffu, v[i], o);
    }
#pragma unroll
    for (int h = N / 2; h >= 1; h >>= 1) {
        const bool up = (lane & h) != 0;
#pragma unroll
        for (int i = 0; i < h; ++i) {
            const T send = up ? v[i] : v[i + h];
            const T keep = up ? v[i + h] : v[i];
            v[i] = keep + __shfl_xor_sync(0xffffffffu, send, h);
        }
    }
    return v[0];
}

// Adds the warp's column sums of acc[0..KP) to wrow[0..KP) (this warp's row of
// shared accumulators; lane c owns column c).
template <typename T, int KP>
__device__ __forceinline__ void warp_cols_add(const T (&acc)[KP], double *wrow, int lane) {
    constexpr int K1 = KP < 32 ? KP : 32;
    constexpr int N1 = pow2ceil(K1);
    T v[N1];
#pragma unroll
    for (int i = 0; i < N1; ++i) v[i] = i < K1 ? acc[i] : T(0);
    const T s = warp_cols_reduce<T, N1>(v, lane);
    if (lane < K1) wrow[lane] += (double)s;
    if constexpr (KP > 32) {
        constexpr int K2 = KP - 32;
        constexpr int N2 = pow2ceil(K2);
        T u[N2];
#pragma unroll
        for (int i = 0; i < N2; ++i) u[i] = i < K2 ? acc[32 + i] : T(0);
        const T s2 = warp_cols_reduce<T, N2>(u, lane);
        if (lane < K2) wrow[32 + lane] += (double)s2;
    }
}

// Column sums of the gridDim.x block partials part[b * KP + c] into
// out[0..KP) (shared memory), fixed order: thread t adds blocks t / KP,
// t / KP + S, ... of column t % KP (S = threads / KP stripes), then the
// stripes are added pairwise in a fixed tree.
template <int KP, int NT>
__device__ __forceinline__ void grid_cols_sum(const double *part, double *out, double *stripe) {
    constexpr int S = NT / KP;
    const int t = threadIdx.x;
    if (gridDim.x <= 32) {
        // few blocks (the cluster form): one thread per column, four chains
        // in a fixed order, no tree and its barriers
        if (t < KP) {
            const int nb = gridDim.x;
            double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
            int b = 0;
            for (; b + 3 < nb; b += 4) {
                s0 += __ldcg(part + (size_t)b * KP + t);
                s1 += __ldcg(part + (size_t)(b + 1) * KP + t);
                s2 += __ldcg(part + (size_t)(b + 2) * KP + t);
                s3 += __ldcg(part + (size_t)(b + 3) * KP + t);
            }
            for (; b < nb; ++b) s0 += __ldcg(part + (size_t)b * KP + t);
            out[t] = (s0 + s1) + (s2 + s3);
        }
        __syncthreads();
        return;
    }
    double s = 0.0;
    if (t < S * KP) {
        const int c = t % KP;
        const int nb = gridDim.x;
        int b = t / KP;
        double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
        // L2 loads: the partials were written by other blocks on other SMs
        for (; b + 3 * S < nb; b += 4 * S) {
            s0 += __ldcg(part + (size_t)b * KP + c);
            s1 += __ldcg(part + (size_t)(b + S) * KP + c);
            s2 += __ldcg(part + (size_t)(b + 2 * S) * KP + c);
            s3 += __ldcg(part + (size_t)(b + 3 * S) * KP + c);
        }
        for (; b < nb; b += S) s0 += __ldcg(part + (size_t)b * KP + c);
        s = (s0 + s1) + (s2 + s3);
    }
    stripe[t] = s;
    __syncthreads();
    for (int width = S; width > 1;) {
        const int half = (width + 1) / 2;
        if (t < (width - half) * KP) stripe[t] += stripe[t + half * KP];
        __syncthreads();
        width = half;
    }
    if (t < KP) out[t] = stripe[t];
    __syncthreads();
}

// Wide blocks (at least 8 column groups, an even number) gather the SpMM
// phase in two halves of the column groups.
template <typename T, int KP>
constexpr bool kSplitGather = (KP / Pk<T>::L) >= 8 && (KP / Pk<T>::L) % 2 == 0;

// Block shape by row width: 512 threads (two resident blocks, <= 64
// registers) for rows up to 80 bytes and for FP32 rows of 40 columns (whose
// phases run in two column parts: 4.76 -> 4.34 s of inner solve per 128^3
// solve against one block per SM), 512 threads (<= 128 registers) up to 160
// bytes, and 256 threads (<= 255 registers) for wider FP64 rows.
template <typename T, int KP>
__host__ __device__ constexpr int pcg_threads() {
    return sizeof(T) * KP <= 160 ? 512 : 256;
}
template <typename T, int KP>
__host__ __device__ constexpr int pcg_min_blocks() {
    // FP32 rows of 40 columns fit 64 registers with their phases split into
    // column parts: two blocks per SM, twice the warps hiding gather latency
    return (sizeof(T) * KP <= 80 || (sizeof(T) == 4 && KP == 40)) ? 2 : 1;
}

template <typename T, int KP, bool CL>
__global__ void __launch_bounds__(pcg_threads<T, KP>(), pcg_min_blocks<T, KP>())
k_block_pcg(PcgArgs<T> a) {
    constexpr int kPcgThreads = pcg_threads<T, KP>();
    constexpr int L = Pk<T>::L;
    constexpr int G = KP / L;  // 16-byte groups per row
    constexpr int nwarps = kPcgThreads / 32;
    // column-group parts of the setup, SpMM and update phases
    constexpr int NP = kSplitGather<T, KP> ? 2 : 1;
    constexpr int GP = G / NP, KPP = KP / NP;
    auto for_parts = [](auto &&f) {
        f(std::integral_constant<int, 0>{});
        if constexpr (NP == 2) f(std::integral_constant<int, 1>{});
    };
    __shared__ double wred[nwarps][KP];  // per-warp column sums of one phase
    __shared__ double stripe[kPcgThreads];
    __shared__ double sum1[KP], sum2[KP];
    __shared__ T s_coef[KP];
    __shared__ int s_act[KP];
    __shared__ int s_gact[G];
    __shared__ int s_nactive;
    __shared__ long long s_range[2];

    // the cluster form's copy of the scalars (one byte in the grid form)
    __shared__ std::conditional_t<CL, PcgScalars, char> s_sc;
    PcgScalars *sc = CL ? reinterpret_cast<PcgScalars *>(&s_sc) : a.sc;
    // the statistics counters are written by one block: the last to arrive
    // (grid form) or the cluster's first
    const bool stats_block = !CL || blockIdx.x == 0;
    PcgSync *gs = a.sync;
    int *error = &a.sync->error;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int k = a.k, n = a.n;
    const double vb = (double)sizeof(T);
    if (!CL && a.withhold_last && gridDim.x > 1 && blockIdx.x == gridDim.x - 1) return;

    // per-warp accumulators: clear, and flush (fixed-order sum over warps)
    auto wred_zero = [&]() {
        for (int i = tid; i < nwarps * KP; i += kPcgThreads) (&wred[0][0])[i] = 0.0;
        __syncthreads();
    };
    auto wred_flush = [&](double *out) {
        __syncthreads();
        if (tid < KP) {
            double s = 0.0;
#pragma unroll
            for (int w = 0; w < nwarps; ++w) s += wred[w][tid];
            out[tid] = s;
        }
        __syncthreads();
    };

    // slice range of this block, balanced by stored entries
    if (tid < 2) {
        const long long total = a.sp[a.nslices];
        const long long target = total * (long long)(blockIdx.x + tid) / gridDim.x;
        int lo = 0, hi = a.nslices;  // first slice s with sp[s] >= target
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (a.sp[mid] < target) lo = mid + 1;
            else hi = mid;
        }
        s_range[tid] = (blockIdx.x + tid == gridDim.x) ? a.nslices : lo;
    }
    __syncthreads();
    const int s0 = (int)s_range[0], s1 = (int)s_range[1];
    const int r0 = min(n, 32 * s0), r1 = min(n, 32 * s1);
    unsigned long long epoch = 0;
    // Per-block partial sums for the barrier `e` (two arrays of gridDim.x rows).
    // The cluster form alternates two sets by the parity of e: its CTAs read
    // the partials after the barrier while faster ones already write the
    // next phase's, and a set is rewritten only after the following barrier.
    auto part_base = [&](unsigned long long e) {
        return a.part + (CL ? (size_t)(e & 1) * 2 * gridDim.x * KP : 0);
    };
    double *part1 = part_base(1) + (size_t)blockIdx.x * KP;
    double *part2 = part_base(1) + (size_t)(gridDim.x + blockIdx.x) * KP;

    auto finish = [&](bool ok) {
        if constexpr (CL) {  // the host reads the scalars of the cluster's first CTA
            if (blockIdx.x == 0) {
                const int *src = reinterpret_cast<const int *>(sc);
                int *dst = reinterpret_cast<int *>(a.sc);
                for (int i = tid; i < (int)(sizeof(PcgScalars) / sizeof(int)); i += kPcgThreads)
                    dst[i] = src[i];
            }
        }
        if (blockIdx.x == 0 && tid == 0) {
            if (!ok || *(volatile int *)error) a.stats->error = 1;
            a.stats->launches += 1;
            a.stats->iters += (unsigned long long)sc->niter;
        }
    };

    // ---------------- r = b - S x (or r = b for x = 0), p = 0, norms
    // (wide blocks work on their column groups in parts, which bounds the
    // accumulator registers of every phase)
    wred_zero();
    if (a.x_zero) {
        for_parts([&](auto part) {
            constexpr int U0 = decltype(part)::value * GP;
            T racc[KPP];
#pragma unroll
            for (int c = 0; c < KPP; ++c) racc[c] = T(0);
            for (int row = r0 + tid; row < r1; row += kPcgThreads) {
#pragma unroll
                for (int uu = 0; uu < GP; ++uu) {
                    const int u = U0 + uu;
                    const Pk<T> b = Pk<T>::ld(a.B + boff<T, KP>(row, u));
                    Pk<T> z;
#pragma unroll
                    for (int q = 0; q < L; ++q) {
                        z.v[q] = T(0);
                        racc[uu * L + q] = fma(b.v[q], b.v[q], racc[uu * L + q]);
                    }
                    b.st(a.R + boff<T, KP>(row, u));
                    z.st(a.X + boff<T, KP>(row, u));
                    z.st(a.P + boff<T, KP>(row, u));
                    group_fence();
                }
            }
            warp_cols_add<T, KPP>(racc, wred[warp] + U0 * L, lane);
        });
    } else {
        for (int s = s0 + warp; s < s1; s += nwarps) {
            const long long beg = a.sp[s], end = a.sp[s + 1];
            const int row = s * 32 + lane;
            for_parts([&](auto part) {
                constexpr int U0 = decltype(part)::value * GP;
                T acc[KPP];
#pragma unroll
                for (int c = 0; c < KPP; ++c) acc[c] = T(0);
                gather_row_part<T, KP, U0, GP>(a.col, a.val, beg + lane, (int)((end - beg) >> 5),
                                               a.X, acc);
                if (row < n) {
#pragma unroll
                    for (int uu = 0; uu < GP; ++uu) {
                        const int u = U0 + uu;
                        const Pk<T> b = Pk<T>::ld(a.B + boff<T, KP>(row, u));
                        Pk<T> r, z;
#pragma unroll
                        for (int q = 0; q < L; ++q) {
                            r.v[q] = b.v[q] - acc[uu * L + q];
                            z.v[q] = T(0);
                            acc[uu * L + q] = r.v[q] * r.v[q];
                        }
                        r.st(a.R + boff<T, KP>(row, u));
                        z.st(a.P + boff<T, KP>(row, u));
                    }
                } else {
#pragma unroll
                    for (int c = 0; c < KPP; ++c) acc[c] = T(0);
                }
                warp_cols_add<T, KPP>(acc, wred[warp] + U0 * L, lane);
            });
        }
    }
    wred_flush(part1);
    if (a.rel_tol) {
        wred_zero();
        for_parts([&](auto part) {
            constexpr int U0 = decltype(part)::value * GP;
            T bacc[KPP];
#pragma unroll
            for (int c = 0; c < KPP; ++c) bacc[c] = T(0);
            for (int row = r0 + tid; row < r1; row += kPcgThreads) {
#pragma unroll
                for (int uu = 0; uu < GP; ++uu) {
                    const Pk<T> b = Pk<T>::ld(a.B + boff<T, KP>(row, U0 + uu));
#pragma unroll
                    for (int q = 0; q < L; ++q)
                        bacc[uu * L + q] = fma(b.v[q], b.v[q], bacc[uu * L + q]);
                    group_fence();
                }
            }
            warp_cols_add<T, KPP>(bacc, wred[warp] + U0 * L, lane);
        });
        wred_flush(part2);
    }
    // initial residual norms (src/ops_lin_sol.c:171-233)
    if (!pcg_sync<CL>(gs, error, a.timeout_ns, a.max_polls, ++epoch, [&]() {
            grid_cols_sum<KP, kPcgThreads>(part_base(epoch), sum1, stripe);
            if (a.rel_tol)
                grid_cols_sum<KP, kPcgThreads>(part_base(epoch) + (size_t)gridDim.x * KP, sum2,
                                               stripe);
            if (tid < kPcgMaxCols) {
                const int c = tid;
                if (c < k) {
                    const double nb = a.rel_tol ? sqrt(sum2[c]) : 1.0;
                    const double rr = sum1[c];
                    sc->norm_b[c] = nb;
                    sc->rho2[c] = rr;
                    sc->init_res[c] = sqrt(rr);
                    sc->last_res[c] = sqrt(rr);
                    sc->active[c] = sqrt(rr) > a.tol * nb ? 1 : 0;
                    sc->left_at[c] = 0;
                    sc->beta[c] = 0.0;
                    sc->alpha[c] = 0.0;
                } else {
                    sc->active[c] = 0;
                    sc->left_at[c] = 0;
                }
            }
            __syncthreads();
            if (tid == 0) {
                int cnt = 0;
                for (int c = 0; c < k; ++c) cnt += sc->active[c];
                sc->nactive = cnt;
                sc->niter = 0;
                if (stats_block)
                    a.stats->kernel_bytes +=
                    a.x_zero ? 4.0 * n * KP * vb : a.matrix_bytes + 4.0 * n * KP * vb;
            }
        })) {
        finish(false);
        return;
    }

    for (int it = 0; it < a.max_iter; ++it) {
        // ---------------- phase 1: p = r + beta p
        if (tid < KP) {
            s_act[tid] = sc->active[tid];
            s_coef[tid] = (T)sc->beta[tid];
        }
        if (tid == 0) s_nactive = sc->nactive;
        __syncthreads();
        if (s_nactive == 0) break;
        if (tid < G) {
            int any = 0;
            for (int q = 0; q < L; ++q) any |= s_act[tid * L + q];
            s_gact[tid] = any;
        }
        __syncthreads();
        const bool first = it == 0;
        for (int row = r0 + tid; row < r1; row += kPcgThreads) {
#pragma unroll
            for (int u = 0; u < G; ++u) {
                if (!s_gact[u]) continue;
                const Pk<T> r = Pk<T>::ld(a.R + boff<T, KP>(row, u));
                Pk<T> p = Pk<T>::ld(a.P + boff<T, KP>(row, u));
#pragma unroll
                for (int q = 0; q < L; ++q)
                    if (s_act[u * L + q])
                        p.v[q] = first ? r.v[q] : fma(s_coef[u * L + q], p.v[q], r.v[q]);
                p.st(a.P + boff<T, KP>(row, u));
                group_fence();
            }
        }
        wred_zero();
        if (!pcg_sync<CL>(gs, error, a.timeout_ns, a.max_polls, ++epoch, [&]() {
                if (tid == 0 && stats_block) a.sync->t_spmm = global_ns();
            })) {
            finish(false);
            return;
        }

        // ---------------- phase 2: w = S p, p^T w
        {
            bool ga[G];
#pragma unroll
            for (int u = 0; u < G; ++u) ga[u] = s_gact[u] != 0;
            for (int s = s0 + warp; s < s1; s += nwarps) {
                const long long beg = a.sp[s], end = a.sp[s + 1];
                const int width = (int)((end - beg) >> 5);
                if constexpr (kSplitGather<T, KP>) {
                    // one half of the column groups of a slice's rows: w, then the
                    // partial sums of p^T w over those columns
                    auto spmm_half = [&](auto half_tag, int s, int width, long long e0) {
                        constexpr int H = decltype(half_tag)::value;
                        constexpr int NU = G / 2, U0 = H * NU;
                        T acc[NU * L];
#pragma unroll
                        for (int c = 0; c < NU * L; ++c) acc[c] = T(0);
                        gather_row_part<T, KP, U0, NU>(a.col, a.val, e0, width, a.P, acc);
                        const int row = s * 32 + lane;
#pragma unroll
                        for (int u = 0; u < NU; ++u) {
                            if (!ga[U0 + u] || row >= n) {
#pragma unroll
                                for (int q = 0; q < L; ++q) acc[u * L + q] = T(0);
                                continue;
                            }
                            Pk<T> w;
#pragma unroll
                            for (int q = 0; q < L; ++q) w.v[q] = acc[u * L + q];
                            w.st(a.W + boff<T, KP>(row, U0 + u));
                            const Pk<T> p = Pk<T>::ld(a.P + boff<T, KP>(row, U0 + u));
#pragma unroll
                            for (int q = 0; q < L; ++q)
                                acc[u * L + q] = s_act[(U0 + u) * L + q] ? p.v[q] * w.v[q] : T(0);
                        }
                        warp_cols_add<T, NU * L>(acc, wred[warp] + U0 * L, lane);
                    };
                    spmm_half(std::integral_constant<int, 0>{}, s, width, beg + lane);
                    spmm_half(std::integral_constant<int, 1>{}, s, width, beg + lane);
                } else {
                    T acc[KP];
#pragma unroll
                    for (int c = 0; c < KP; ++c) acc[c] = T(0);
                    gather_row<T, KP>(a.col, a.val, beg + lane, width, a.P, ga, acc);
                    const int row = s * 32 + lane;
                    if (row < n) {
#pragma unroll
                        for (int u = 0; u < G; ++u) {
                            if (!ga[u]) continue;
                            Pk<T> w;
#pragma unroll
                            for (int q = 0; q < L; ++q) w.v[q] = acc[u * L + q];
                            w.st(a.W + boff<T, KP>(row, u));
                            const Pk<T> p = Pk<T>::ld(a.P + boff<T, KP>(row, u));
#pragma unroll
                            for (int q = 0; q < L; ++q)
                                acc[u * L + q] = s_act[u * L + q] ? p.v[q] * w.v[q] : T(0);
                        }
                    } else {
#pragma unroll
                        for (int c = 0; c < KP; ++c) acc[c] = T(0);
                    }
#pragma unroll
                    for (int u = 0; u < G; ++u)
                        if (!ga[u]) {
#pragma unroll
                            for (int q = 0; q < L; ++q) acc[u * L + q] = T(0);
                        }
                    warp_cols_add<T, KP>(acc, wred[warp], lane);
                }
            }
            wred_flush(part_base(epoch + 1) + (size_t)blockIdx.x * KP);
        }
        // alpha = rho / p^T w (src/ops_lin_sol.c:300-330)
        if (!pcg_sync<CL>(gs, error, a.timeout_ns, a.max_polls, ++epoch, [&]() {
                grid_cols_sum<KP, kPcgThreads>(part_base(epoch), sum1, stripe);
                if (tid < k) {
                    const int c = tid;
                    const double ptw = sum1[c];
                    sc->ptw[c] = ptw;
                    sc->rho1[c] = sc->rho2[c];
                    sc->alpha[c] = sc->active[c] ? sc->rho2[c] / ptw : 0.0;
                }
                if (tid == 0 && stats_block) {
                    int gact = 0;
                    for (int u = 0; u < G; ++u) gact += s_gact[u];
                    const double vec = (double)n * gact * L * vb;
                    a.stats->spmm_ns += global_ns() - a.sync->t_spmm;
                    // SpMM: the matrix once, p read once, w written once
                    a.stats->spmm_bytes += a.matrix_bytes + 2.0 * vec;
                    // iteration: phase 1 (r, p read; p written), phase 2 (p
                    // gathered and re-read, w written), phase 3 (x, p, r, w
                    // read; x, r written)
                    a.stats->kernel_bytes += a.matrix_bytes + 12.0 * vec;
                }
            })) {
            finish(false);
            return;
        }

        // ---------------- phase 3: x += alpha p, r -= alpha w, r^T r
        if (tid < KP) s_coef[tid] = (T)sc->alpha[tid];
        wred_zero();
        for_parts([&](auto part) {
            constexpr int U0 = decltype(part)::value * GP;
            T racc[KPP];
#pragma unroll
            for (int c = 0; c < KPP; ++c) racc[c] = T(0);
            for (int row = r0 + tid; row < r1; row += kPcgThreads) {
#pragma unroll
                for (int uu = 0; uu < GP; ++uu) {
                    const int u = U0 + uu;
                    if (!s_gact[u]) continue;
                    Pk<T> x = Pk<T>::ld(a.X + boff<T, KP>(row, u));
                    Pk<T> r = Pk<T>::ld(a.R + boff<T, KP>(row, u));
                    const Pk<T> p = Pk<T>::ld(a.P + boff<T, KP>(row, u));
                    const Pk<T> w = Pk<T>::ld(a.W + boff<T, KP>(row, u));
#pragma unroll
                    for (int q = 0; q < L; ++q) {
                        const int c = u * L + q;
                        if (s_act[c]) {
                            const T al = s_coef[c];
                            x.v[q] = fma(al, p.v[q], x.v[q]);
                            r.v[q] = fma(-al, w.v[q], r.v[q]);
                            racc[uu * L + q] = fma(r.v[q], r.v[q], racc[uu * L + q]);
                        }
                    }
                    x.st(a.X + boff<T, KP>(row, u));
                    r.st(a.R + boff<T, KP>(row, u));
                    group_fence();
                }
            }
            warp_cols_add<T, KPP>(racc, wred[warp] + U0 * L, lane);
        });
        wred_flush(part_base(epoch + 1) + (size_t)blockIdx.x * KP);
        // convergence test of src/ops_lin_sol.c:383-394 and beta for the next step
        if (!pcg_sync<CL>(gs, error, a.timeout_ns, a.max_polls, ++epoch, [&]() {
                grid_cols_sum<KP, kPcgThreads>(part_base(epoch), sum1, stripe);
                if (tid < k && sc->active[tid]) {
                    const int c = tid;
                    const double rr = sum1[c];
                    sc->rho2[c] = rr;
                    const double res = sqrt(rr);
                    sc->last_res[c] = res;
                    sc->beta[c] = rr / sc->rho1[c];
                    if (!(res > a.rate * sc->init_res[c] && res > a.tol * sc->norm_b[c])) {
                        sc->active[c] = 0;
                        sc->left_at[c] = sc->niter + 1;  // niter moves on after the barrier
                    }
                }
                __syncthreads();
                if (tid == 0) {
                    int cnt = 0;
                    for (int c = 0; c < k; ++c) cnt += sc->active[c];
                    sc->nactive = cnt;
                    sc->niter += 1;
                }
            })) {
            finish(false);
            return;
        }
    }
    finish(true);
}

int num_sms_pcg() { return device_sms(); }

constexpr int kMaxBlocksPerSm = 4;

// Cluster size of the cluster form (16 CTAs where the device schedules such
// a cluster of this kernel, else 8), or 0 when neither can run.
template <typename T, int KP>
int pcg_cluster_size() {
    static PerDevice<int> cache;
    return cache.get([] {
        int csize = 0;
        for (int c : {16, 8}) {
            if (c > 8 && cudaFuncSetAttribute(k_block_pcg<T, KP, true>,
                                              cudaFuncAttributeNonPortableClusterSizeAllowed,
                                              1) != cudaSuccess) {
                cudaGetLastError();
                continue;
            }
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(c);
            cfg.blockDim = dim3(pcg_threads<T, KP>());
            cudaLaunchAttribute at[1];
            at[0].id = cudaLaunchAttributeClusterDimension;
            at[0].val.clusterDim.x = c;
            at[0].val.clusterDim.y = 1;
            at[0].val.clusterDim.z = 1;
            cfg.attrs = at;
            cfg.numAttrs = 1;
            int n = 0;
            if (cudaOccupancyMaxActiveClusters(&n, k_block_pcg<T, KP, true>, &cfg) !=
                cudaSuccess) {
                cudaGetLastError();
                continue;
            }
            if (n > 0) {
                csize = c;
                break;
            }
        }
        return csize;
    });
}

template <typename T, int KP>
void launch_block_pcg(PcgArgs<T> a, cudaStream_t st) {
    // Small operators run in one thread-block cluster: its barrier is the
    // hardware's, where a grid barrier costs a few microseconds through global
    // memory three times per CG step.  FP32 up to two slices per warp of the
    // cluster; FP64 up to one, since its SpMM is bound by the FP64 units of
    // the cluster's 16 SMs (measured on the 2D batch problems: at 390-430
    // slices the cluster form was 1.6x slower in FP64 and 1.4x faster in FP32).
    const int csize = pcg_cluster_size<T, KP>();
    const int per_warp = sizeof(T) == 4 ? 2 : 1;
    if (csize > 0 && a.nslices <= csize * (pcg_threads<T, KP>() / 32) * per_warp) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(csize);
        cfg.blockDim = dim3(pcg_threads<T, KP>());
        cfg.stream = st;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = csize;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        GCGE_CUDA(cudaLaunchKernelEx(&cfg, k_block_pcg<T, KP, true>, a));
        count_launch();
        return;
    }
    static PerDevice<int> occupancy;
    const int bpsm = occupancy.get([] {
        int b = 0;
        GCGE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_block_pcg<T, KP, false>,
                                                                pcg_threads<T, KP>(), 0));
        return std::min(b, kMaxBlocksPerSm);
    });
    GCGE_REQUIRE(bpsm >= 1, GCGE_ERR_CUDA, "block PCG: kernel does not fit on an SM");
    int nb = std::max(1, std::min(bpsm * num_sms_pcg(), a.nslices));
    if (t_pcg_share > 1) nb = std::min(nb, std::max(1, bpsm * num_sms_pcg() / t_pcg_share));
    void *args[] = {&a};
    GCGE_CUDA(cudaLaunchCooperativeKernel((const void *)k_block_pcg<T, KP, false>, dim3(nb),
                                          dim3(pcg_threads<T, KP>()), args, 0, st));
    count_launch();
}

}  // namespace

// column-major (S, ld) <-> slice-blocked (T, kp): element (i, c) of the
// blocked block sits at ((i / 32) G + c / L) 32 L + (i % 32) L + c % L with
// L = 16 / sizeof(T), G = kp / L; rows up to the next multiple of 32 and
// columns k..kp-1 are zero.
template <typename T>
__host__ __device__ __forceinline__ size_t blk_index(int i, int c, int kp) {
    constexpr int L = 16 / (int)sizeof(T);
    const int G = kp / L;
    return ((size_t)(i >> 5) * G + c / L) * (32 * L) + (size_t)(i & 31) * L + c % L;
}
template <typename S, typename T>
__global__ void k_col_to_rows(int n, int k, int kp, const S *__restrict__ X, int ldx,
                              T *__restrict__ Y) {
    constexpr int L = 16 / (int)sizeof(T);
    const int G = kp / L;
    const size_t total = (size_t)((n + 31) / 32) * 32 * kp;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
         t += (size_t)gridDim.x * blockDim.x) {
        // t = ((s G + u) 32 + l) L + e
        const int e = (int)(t % L);
        const size_t q = t / L;
        const int l = (int)(q % 32);
        const size_t su = q / 32;
        const int u = (int)(su % G);
        const int i = (int)(su / G) * 32 + l, c = u * L + e;
        Y[t] = (i < n && c < k) ? (T)X[i + (size_t)c * ldx] : T(0);
    }
}
template <typename T, typename D>
__global__ void k_rows_to_col(int n, int k, int kp, const T *__restrict__ X, D *__restrict__ Y,
                              int ldy, int add) {
    const size_t total = (size_t)n * k;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
         t += (size_t)gridDim.x * blockDim.x) {
        const int c = (int)(t / n), i = (int)(t % n);
        const D v = (D)X[blk_index<T>(i, c, kp)];
        D &y = Y[i + (size_t)c * ldy];
        y = add ? y + v : v;
    }
}

template <typename S, typename T>
void col_to_rows(int n, int k, int kp, const S *X, int ldx, T *Y, cudaStream_t st) {
    const size_t total = (size_t)((n + 31) / 32) * 32 * kp;
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

void PcgWork::timing_reset(cudaStream_t st) {
    ev_used = 0;
    launches = 0;
    kernel_ms = spmm_ms = kernel_bytes = spmm_bytes = 0.0;
    total_iters = 0;
    GCGE_CUDA(cudaMemsetAsync(stats.p, 0, sizeof(PcgStats), st));
}
void PcgWork::collect(cudaStream_t st) {
    GCGE_CUDA(cudaMemcpyAsync(h_stats.p, stats.p, sizeof(PcgStats), cudaMemcpyDeviceToHost, st));
    GCGE_CUDA(cudaStreamSynchronize(st));
    double ms = 0.0;
    for (size_t i = 0; i + 1 < ev_used; i += 2) {
        float t = 0.f;
        if (cudaEventElapsedTime(&t, ev[i], ev[i + 1]) == cudaSuccess) ms += t;
    }
    kernel_ms = ms;
    spmm_ms = (double)h_stats.p->spmm_ns * 1e-6;
    kernel_bytes = h_stats.p->kernel_bytes;
    spmm_bytes = h_stats.p->spmm_bytes;
    total_iters = (long long)h_stats.p->iters;
    if (h_stats.p->error != 0) {
        // the launch that timed out has ended; clear the flag so the next
        // solve on this work area starts clean, then report
        GCGE_CUDA(cudaMemsetAsync(&stats.p->error, 0, sizeof(int), st));
        GCGE_CUDA(cudaStreamSynchronize(st));
        throw CudaError{GCGE_ERR_CUDA, "block PCG: a grid barrier wait timed out"};
    }
}
PcgWork::~PcgWork() {
    for (auto e : ev) cudaEventDestroy(e);
}

void PcgWork::reserve(int n, int kmax_) {
    (void)n;
    kmax = std::max(kmax_, 40);
    part.alloc((size_t)2 * kMaxBlocksPerSm * num_sms_pcg() * kPcgMaxCols);
    if (!sc.p) {
        sc.alloc(1);
        sync.alloc(1);
        stats.alloc(1);
        h_sc.alloc(1);
        h_stats.alloc(1);
        GCGE_CUDA(cudaMemsetAsync(stats.p, 0, sizeof(PcgStats), lib_stream()));
    }
}

int pcg_last_iters(PcgWork &wk, cudaStream_t st) {
    GCGE_CUDA(cudaMemcpyAsync(wk.h_sc.p, wk.sc.p, sizeof(PcgScalars), cudaMemcpyDeviceToHost, st));
    GCGE_CUDA(cudaMemcpyAsync(wk.h_stats.p, wk.stats.p, sizeof(PcgStats), cudaMemcpyDeviceToHost,
                              st));
    GCGE_CUDA(cudaStreamSynchronize(st));
    if (wk.h_stats.p->error != 0) {
        GCGE_CUDA(cudaMemsetAsync(&wk.stats.p->error, 0, sizeof(int), st));
        GCGE_CUDA(cudaStreamSynchronize(st));
        throw CudaError{GCGE_ERR_CUDA, "block PCG: a grid barrier wait timed out"};
    }
    return wk.h_sc.p->niter;
}

thread_local PcgBarrierTest t_pcg_barrier_test;

template <typename T>
void block_pcg_rows(PcgWork &wk, const SellPattern &pat, const T *sval, const T *Bv, T *X, T *R,
                    T *P, T *W, int kp, int k, int max_iter, double rate, double tol, bool rel_tol,
                    bool x_zero, cudaStream_t st) {
    constexpr int L = 16 / (int)sizeof(T);
    GCGE_REQUIRE(k >= 1 && k <= kp && kp <= 40 && kp % L == 0 && k <= kPcgMaxCols, GCGE_ERR_ARG,
                 "block_pcg: block width");
    if (pat.n == 0) return;
    PcgArgs<T> a;
    a.sp = pat.slice_ptr.p;
    a.col = pat.col.p;
    a.val = sval;
    a.n = pat.n;
    a.nslices = pat.nslices;
    a.B = Bv;
    a.X = X;
    a.R = R;
    a.P = P;
    a.W = W;
    a.k = k;
    a.max_iter = std::max(0, max_iter);
    a.rel_tol = rel_tol ? 1 : 0;
    a.x_zero = x_zero ? 1 : 0;
    a.rate = rate;
    a.tol = tol;
    a.matrix_bytes = (double)pat.nnz * (sizeof(T) + 4) + 4.0 * (pat.n + 1);
    a.sc = wk.sc.p;
    a.sync = wk.sync.p;
    a.stats = wk.stats.p;
    a.part = wk.part.p;
    a.timeout_ns = kBarrierTimeoutNs;
    a.max_polls = kBarrierMaxPolls;
    a.withhold_last = 0;
    if (t_pcg_barrier_test.active) {
        a.timeout_ns = t_pcg_barrier_test.timeout_ns;
        a.withhold_last = t_pcg_barrier_test.withhold_last;
    }
    GCGE_CUDA(cudaMemsetAsync(wk.sync.p, 0, sizeof(PcgSync), st));
    const bool timed = wk.ev_used + 2 <= 65536;
    if (timed) {
        while (wk.ev.size() < wk.ev_used + 2) {
            cudaEvent_t e;
            GCGE_CUDA(cudaEventCreate(&e));
            wk.ev.push_back(e);
        }
        GCGE_CUDA(cudaEventRecord(wk.ev[wk.ev_used], st));
    }
    if constexpr (sizeof(T) == 4) {
        switch (kp) {
#define GCGE_PCG_CASE(W_)                                     \
    case W_:                                                  \
        launch_block_pcg<T, W_>(a, st);                       \
        break;
            GCGE_PCG_CASE(4) GCGE_PCG_CASE(8) GCGE_PCG_CASE(12) GCGE_PCG_CASE(16)
            GCGE_PCG_CASE(20) GCGE_PCG_CASE(24) GCGE_PCG_CASE(28) GCGE_PCG_CASE(32)
            GCGE_PCG_CASE(36) GCGE_PCG_CASE(40)
            default: throw CudaError{GCGE_ERR_ARG, "block_pcg: unsupported width"};
        }
    } else {
        switch (kp) {
            GCGE_PCG_CASE(2) GCGE_PCG_CASE(4) GCGE_PCG_CASE(6) GCGE_PCG_CASE(8)
            GCGE_PCG_CASE(12) GCGE_PCG_CASE(16) GCGE_PCG_CASE(20) GCGE_PCG_CASE(24)
            GCGE_PCG_CASE(28) GCGE_PCG_CASE(32) GCGE_PCG_CASE(36) GCGE_PCG_CASE(40)
#undef GCGE_PCG_CASE
            default: throw CudaError{GCGE_ERR_ARG, "block_pcg: unsupported width"};
        }
    }
    if (timed) {
        GCGE_CUDA(cudaEventRecord(wk.ev[wk.ev_used + 1], st));
        wk.ev_used += 2;
    }
    wk.launches++;
}

template void block_pcg_rows<double>(PcgWork &, const SellPattern &, const double *, const double *,
                                     double *, double *, double *, double *, int, int, int, double,
                                     double, bool, bool, cudaStream_t);
template void block_pcg_rows<float>(PcgWork &, const SellPattern &, const float *, const float *,
                                    float *, float *, float *, float *, int, int, int, double,
                                    double, bool, bool, cudaStream_t);

}  // namespace gcge
