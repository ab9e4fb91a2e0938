// Dense symmetric eigensolver for the Rayleigh-Ritz projected matrix
// (replaces the reference's dsyevx call, src/ops_eig_sol_gcg.c:1145-1150 /
// :1207-1209: all eigenpairs, ascending).
//
// GB300 issues FP64 at ~1/58 of its FP32 rate, so an FP64 Jacobi on one SM
// would take tens of milliseconds for s = 200.  The solver therefore
//   1. runs a parallel-order (round-robin) two-sided cyclic Jacobi in FP32,
//      logging each round's rotations: for s >= 88 in a cluster of 8 CTAs
//      whose shared memories hold the matrix rows of the pairs each CTA owns
//      (distributed shared memory; rows move between neighbouring CTAs as the
//      round-robin order advances), else in one 1024-thread CTA with the
//      packed upper triangle in shared memory;
//   2. rebuilds the eigenvector matrix from the rotation log with one warp
//      per row (rows of V = J_1 J_2 ... J_T are independent);
//   3. refines eigenvectors and eigenvalues to FP64 accuracy with the
//      iterative refinement of Ogita & Aishima ("Iterative refinement for
//      symmetric eigenvalue decomposition", Japan J. Indust. Appl. Math. 35,
//      2018), whose cost is four s x s FP64 products per step spread over
//      all SMs;
//   4. diagonalises each remaining cluster of nearly equal eigenvalues
//      exactly on the host (tiny FP64 Jacobi) and sorts ascending.
// The 2x2 rotation is the symmetric Schur decomposition of Golub & Van Loan
// (Matrix Computations, Alg. 8.4.1).
#include <cooperative_groups.h>
#include <mutex>
#include <algorithm>
#include <cmath>
#include <numeric>

#include "common.cuh"
#include "eig.cuh"

namespace gcge {

namespace cg = cooperative_groups;

constexpr int kJacobiThreads = 1024;
constexpr int kMaxSweeps = 12;
constexpr float kRotTol = 1e-7f;   // skip rotations below FP32 resolution
constexpr float kOffTol = 2e-6f;   // ||offdiag||_F <= kOffTol ||A||_F ends the sweeps
constexpr double kClusterGap = 1e-5;      // relative gap below which pairs are clustered
constexpr double kStrongCoupling = 1e-2;  // |E_ij| above which pairs are clustered

__host__ __device__ inline int jac_m(int s) { return (s + 1) & ~1; }

// Round-robin pair i of round r for m (even) indices: element m-1 is fixed.
__host__ __device__ inline void jac_pair(int m, int r, int i, int &p, int &q) {
    int a, b;
    if (i == 0) {
        a = m - 1;
        b = r;
    } else {
        a = (r + i) % (m - 1);
        b = (r - i + (m - 1)) % (m - 1);
    }
    p = a < b ? a : b;
    q = a < b ? b : a;
}

__device__ inline int pk(int x, int y) {  // packed upper index, x <= y
    return (y * (y + 1)) / 2 + x;
}
__device__ inline int pks(int x, int y) { return x <= y ? pk(x, y) : pk(y, x); }

size_t jacobi_smem_bytes(int s) {
    const int m = jac_m(s);
    return (size_t)s * (s + 1) / 2 * sizeof(float) + (size_t)(m / 2) * 2 * sizeof(float) +
           (size_t)(m / 2) * 2 * sizeof(short) + 64;
}
static size_t jacobi_dyn_limit();
static bool jacobi_cluster_usable();
static int jacobi_cluster_max_dim();
// one-CTA kernel capacity, and the cluster kernel's where it can run
int jacobi_max_dim() {
    const size_t lim = jacobi_dyn_limit();
    int s = 8;
    while (jacobi_smem_bytes(s + 1) <= lim) ++s;
    if (jacobi_cluster_usable()) s = std::max(s, jacobi_cluster_max_dim());
    return s;
}

__global__ void __launch_bounds__(kJacobiThreads)
k_jacobi32(int s, const double *__restrict__ M, int ldm, float4 *__restrict__ log, int max_rounds,
           int *__restrict__ info /* [0]=rounds, [1]=sweeps, [2]=converged */) {
    extern __shared__ float sm[];
    const int m = jac_m(s);
    const int np = m / 2;
    float *A = sm;
    float *cs = A + (size_t)s * (s + 1) / 2;
    float *sn = cs + np;
    short *pp = reinterpret_cast<short *>(sn + np);  // pair table of the round: p, q
    __shared__ float red_off[32], red_tot[32];
    __shared__ int stop;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5, nwarps = blockDim.x >> 5;
    const int nq = np + (np & 1), width = nq + 1, nblk = (nq / 2) * width;
    for (int idx = t; idx < s * (s + 1) / 2; idx += blockDim.x) {
        // decode packed index -> (x, y), x <= y
        int y = (int)((sqrtf(8.0f * idx + 1.0f) - 1.0f) * 0.5f);
        while ((y + 1) * (y + 2) / 2 <= idx) ++y;
        while (y * (y + 1) / 2 > idx) --y;
        const int x = idx - y * (y + 1) / 2;
        A[idx] = (float)(0.5 * (M[x + (size_t)y * ldm] + M[y + (size_t)x * ldm]));
    }
    __syncthreads();
    int round = 0, sweep = 0, converged = 0;
    for (sweep = 0; sweep < kMaxSweeps && round + (m - 1) <= max_rounds; ++sweep) {
        // stop when the off-diagonal mass is at the FP32 noise level
        float off = 0.0f, tot = 0.0f;
        for (int idx = t; idx < s * (s + 1) / 2; idx += blockDim.x) {
            int y = (int)((sqrtf(8.0f * idx + 1.0f) - 1.0f) * 0.5f);
            while ((y + 1) * (y + 2) / 2 <= idx) ++y;
            while (y * (y + 1) / 2 > idx) --y;
            const int x = idx - y * (y + 1) / 2;
            const float v = A[idx] * A[idx];
            tot += x == y ? v : 2.0f * v;
            if (x != y) off += 2.0f * v;
        }
        for (int o = 16; o > 0; o >>= 1) {
            off += __shfl_xor_sync(0xffffffffu, off, o);
            tot += __shfl_xor_sync(0xffffffffu, tot, o);
        }
        if (lane == 0) {
            red_off[warp] = off;
            red_tot[warp] = tot;
        }
        __syncthreads();
        if (t == 0) {
            float a = 0.f, b = 0.f;
            for (int w = 0; w < nwarps; ++w) {
                a += red_off[w];
                b += red_tot[w];
            }
            stop = (a <= kOffTol * kOffTol * b) ? 1 : 0;
        }
        __syncthreads();
        if (stop) {
            converged = 1;
            break;
        }
        for (int r = 0; r < m - 1; ++r) {
            // (a) pair table and rotation of each pair
            for (int i = t; i < np; i += blockDim.x) {
                int p, q;
                jac_pair(m, r, i, p, q);
                pp[2 * i] = (short)p;
                pp[2 * i + 1] = (short)q;
                float c = 1.0f, sv = 0.0f;
                if (q < s) {
                    const float app = A[pk(p, p)], aqq = A[pk(q, q)], apq = A[pk(p, q)];
                    const float thr = kRotTol * sqrtf(fabsf(app) * fabsf(aqq));
                    if (fabsf(apq) > thr && fabsf(apq) > 1e-30f) {
                        const float tau = (aqq - app) / (2.0f * apq);
                        const float tt = (tau >= 0.0f ? 1.0f : -1.0f) / (fabsf(tau) + hypotf(1.0f, tau));
                        c = rsqrtf(1.0f + tt * tt);
                        sv = tt * c;
                    }
                }
                cs[i] = c;
                sn[i] = sv;
            }
            __syncthreads();
            // (b) A <- J^T A J on every 2x2 block (i <= j) of the pair grid.  The
            // triangle of blocks is folded into nq / 2 rows of nq + 1 blocks (row r
            // holds pair rows r and nq - 1 - r), which the threads share evenly.
            for (int b = t; b < nblk; b += blockDim.x) {
                const int fr = b / width, fc = b - fr * width;
                int i, j;
                if (fc < nq - fr) {
                    i = fr;
                    j = fr + fc;
                } else {
                    i = nq - 1 - fr;
                    j = i + (fc - (nq - fr));
                }
                if (j >= np) continue;
                {
                    const float ci = cs[i], si = sn[i];
                    const float cj = cs[j], sj = sn[j];
                    if (si == 0.0f && sj == 0.0f) continue;
                    const int pi = pp[2 * i], qi = pp[2 * i + 1];
                    const bool qiv = qi < s;
                    const int pj = pp[2 * j], qj = pp[2 * j + 1];
                    const bool qjv = qj < s;
                    if (i == j) {
                        if (!qiv) continue;
                        const float app = A[pk(pi, pi)], aqq = A[pk(qi, qi)], apq = A[pk(pi, qi)];
                        const float t11 = ci * app - si * apq, t12 = ci * apq - si * aqq;
                        const float t21 = si * app + ci * apq, t22 = si * apq + ci * aqq;
                        A[pk(pi, pi)] = t11 * ci - t12 * si;
                        A[pk(qi, qi)] = t21 * si + t22 * ci;
                        A[pk(pi, qi)] = 0.0f;
                        continue;
                    }
                    const float a11 = A[pks(pi, pj)];
                    const float a12 = qjv ? A[pks(pi, qj)] : 0.0f;
                    const float a21 = qiv ? A[pks(qi, pj)] : 0.0f;
                    const float a22 = (qiv && qjv) ? A[pks(qi, qj)] : 0.0f;
                    const float t11 = ci * a11 - si * a21, t12 = ci * a12 - si * a22;
                    const float t21 = si * a11 + ci * a21, t22 = si * a12 + ci * a22;
                    A[pks(pi, pj)] = t11 * cj - t12 * sj;
                    if (qjv) A[pks(pi, qj)] = t11 * sj + t12 * cj;
                    if (qiv) A[pks(qi, pj)] = t21 * cj - t22 * sj;
                    if (qiv && qjv) A[pks(qi, qj)] = t21 * sj + t22 * cj;
                }
            }
            // (c) log the round
            for (int i = t; i < np; i += blockDim.x)
                log[(size_t)round * np + i] = make_float4(cs[i], sn[i], __int_as_float(pp[2 * i]),
                                                          __int_as_float(pp[2 * i + 1]));
            ++round;
            __syncthreads();
        }
    }
    if (t == 0) {
        info[0] = round;
        info[1] = sweep;
        info[2] = converged;
    }
}

// ---------------------------------------------------------------- cluster Jacobi
// The same rotations in a cluster of kJC CTAs.  Indices are arranged by the
// circle method: with P_r[0] = 0 and P_r[i] = 1 + ((i - 1 - r) mod (m - 1)),
// pair slot k of round r is (P_r[k], P_r[m - 1 - k]); after m - 1 rounds P is
// the identity again.  CTA c owns the slots [c np / kJC, (c + 1) np / kJC) and
// holds the two full rows (m floats each) of each of its slots.  A round:
//   (a) every CTA computes the rotations of its slots and writes them into the
//       round table of every CTA of the cluster;
//   (b) after a cluster barrier, each CTA updates every 2x2 block (own slot i,
//       any slot j) of its rows, A <- J^T A J, and writes the new rows into
//       the other row buffer at the slots they hold in the next round, which
//       for at most two rows per CTA is in the neighbouring CTA's shared
//       memory;
//   (c) a second cluster barrier makes the next buffers complete.
// Rotations and the stopping test are those of k_jacobi32; every CTA sums the
// per-CTA off-diagonal masses in the same order, so all take the same decision.
constexpr int kJC = 8;
// Smaller matrices use the one-CTA kernel.  Measured on GB300 (RR-shaped
// matrices, kernel time): s = 64, 80: one CTA 480, 609 us, cluster 510, 652 us;
// s = 96, 128, 200: one CTA 1152, 2321, 8161 us, cluster 956, 1290, 2403 us.
constexpr int kJacClusterMin = 88;
constexpr int kJacMaxLocal = 32;    // slots per CTA (np <= 256: s <= 512)

__host__ __device__ inline int jc_slots(int np) { return (np + kJC - 1) / kJC; }

size_t jacobi_cluster_smem_bytes(int s) {
    const int m = jac_m(s), np = m / 2, ks = jc_slots(np);
    return (size_t)2 * np * sizeof(float4) + (size_t)2 * 2 * ks * m * sizeof(float) +
           (size_t)2 * kJC * 2 * sizeof(float) + 64;
}

// index at position i of the circle arrangement after r rounds
__device__ __forceinline__ int circle_index(int i, int r, int m1) {
    if (i == 0) return 0;
    int v = i - 1 - r;
    v %= m1;
    if (v < 0) v += m1;
    return 1 + v;
}

// CTA owning slot k (slots [c np / kJC, (c + 1) np / kJC) belong to CTA c)
__device__ __forceinline__ int slot_owner(int k, int np) { return ((k + 1) * kJC - 1) / np; }

__global__ void __launch_bounds__(kJacobiThreads, 1)
k_jacobi32_cluster(int s, const double *__restrict__ M, int ldm, float4 *__restrict__ log,
                   int max_rounds, int *__restrict__ info) {
    cg::cluster_group cl = cg::this_cluster();
    const int rank = (int)cl.block_rank();
    extern __shared__ __align__(16) unsigned char jsm[];
    const int m = jac_m(s), np = m / 2, ks = jc_slots(np), m1 = m - 1;
    float4 *table = reinterpret_cast<float4 *>(jsm);  // [2][np]
    float *rows = reinterpret_cast<float *>(table + 2 * np);  // [2][2 ks][m]
    float *red = rows + (size_t)2 * 2 * ks * m;                 // [2][kJC][2]
    __shared__ float wsum[kJacobiThreads / 32][2];
    __shared__ int stop;
    __shared__ float *s_dst[2 * kJacMaxLocal];  // next-round rows of each local slot
    const size_t bufsz = (size_t)2 * ks * m;
    const int k0 = (rank * np) / kJC, k1 = ((rank + 1) * np) / kJC, nloc = k1 - k0;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5, nwarps = blockDim.x >> 5;
    // rows of round 0 (P = identity): slot k holds rows k and m - 1 - k
    for (int idx = t; idx < 2 * nloc * m; idx += blockDim.x) {
        const int lr = idx / m, y = idx - lr * m;
        const int k = k0 + (lr >> 1);
        const int x = (lr & 1) ? m - 1 - k : k;
        float v = 0.0f;
        if (x < s && y < s) v = (float)(0.5 * (M[x + (size_t)y * ldm] + M[y + (size_t)x * ldm]));
        rows[(size_t)lr * m + y] = v;
    }
    cl.sync();  // every CTA of the cluster runs before any remote access
    int cur = 0, round = 0, sweep = 0, converged = 0;
    for (sweep = 0; sweep < kMaxSweeps && round + m1 <= max_rounds; ++sweep) {
        // off-diagonal mass at the start of the sweep (P = identity again)
        {
            const float *R = rows + cur * bufsz;
            float off = 0.0f, tot = 0.0f;
            for (int idx = t; idx < 2 * nloc * m; idx += blockDim.x) {
                const int lr = idx / m, y = idx - lr * m;
                const int k = k0 + (lr >> 1);
                const int x = (lr & 1) ? m - 1 - k : k;
                const float v = R[(size_t)lr * m + y];
                tot += v * v;
                if (x != y) off += v * v;
            }
            for (int o = 16; o > 0; o >>= 1) {
                off += __shfl_xor_sync(0xffffffffu, off, o);
                tot += __shfl_xor_sync(0xffffffffu, tot, o);
            }
            if (lane == 0) {
                wsum[warp][0] = off;
                wsum[warp][1] = tot;
            }
            __syncthreads();
            if (t == 0) {
                float a = 0.0f, b = 0.0f;
                for (int w = 0; w < nwarps; ++w) {
                    a += wsum[w][0];
                    b += wsum[w][1];
                }
                float *slot = red + ((sweep & 1) * kJC + rank) * 2;
                for (int c = 0; c < kJC; ++c) {
                    float *dst = cl.map_shared_rank(slot, c);
                    dst[0] = a;
                    dst[1] = b;
                }
            }
            cl.sync();
            if (t == 0) {
                float a = 0.0f, b = 0.0f;
                for (int c = 0; c < kJC; ++c) {
                    a += red[((sweep & 1) * kJC + c) * 2];
                    b += red[((sweep & 1) * kJC + c) * 2 + 1];
                }
                stop = (a <= kOffTol * kOffTol * b) ? 1 : 0;
            }
            __syncthreads();
            if (stop) {
                converged = 1;
                break;
            }
        }
        for (int r = 0; r < m1; ++r) {
            const float *R = rows + cur * bufsz;
            float4 *tab = table + (round & 1) * np;
            // (a) rotations of the local slots, into every CTA's round table
            for (int ls = t; ls < nloc; ls += blockDim.x) {
                const int k = k0 + ls;
                const int p = circle_index(k, r, m1), q = circle_index(m - 1 - k, r, m1);
                float c = 1.0f, sv = 0.0f;
                if (p < s && q < s) {
                    const float app = R[(size_t)(2 * ls) * m + p];
                    const float aqq = R[(size_t)(2 * ls + 1) * m + q];
                    const float apq = R[(size_t)(2 * ls) * m + q];
                    const float thr = kRotTol * sqrtf(fabsf(app) * fabsf(aqq));
                    if (fabsf(apq) > thr && fabsf(apq) > 1e-30f) {
                        const float tau = (aqq - app) / (2.0f * apq);
                        const float tt =
                            (tau >= 0.0f ? 1.0f : -1.0f) / (fabsf(tau) + hypotf(1.0f, tau));
                        c = rsqrtf(1.0f + tt * tt);
                        sv = tt * c;
                    }
                }
                const float4 e = make_float4(c, sv, __int_as_float(p), __int_as_float(q));
                for (int cc = 0; cc < kJC; ++cc) *cl.map_shared_rank(tab + k, cc) = e;
                log[(size_t)round * np + k] = e;
                // next-round positions of the slot's two rows (circle method)
                int kt, st_, kb, sb;
                if (np == 1) {
                    kt = 0, st_ = 0, kb = 0, sb = 1;
                } else {
                    if (k == 0) kt = 0, st_ = 0;
                    else if (k <= np - 2) kt = k + 1, st_ = 0;
                    else kt = np - 1, st_ = 1;
                    if (k == 0) kb = 1, sb = 0;
                    else kb = k - 1, sb = 1;
                }
                const int ot = slot_owner(kt, np), ob = slot_owner(kb, np);
                const size_t nb = (size_t)(cur ^ 1) * bufsz;
                float *dt = rows + nb + (size_t)(2 * (kt - (ot * np) / kJC) + st_) * m;
                float *db = rows + nb + (size_t)(2 * (kb - (ob * np) / kJC) + sb) * m;
                s_dst[2 * ls] = ot == rank ? dt : cl.map_shared_rank(dt, ot);
                s_dst[2 * ls + 1] = ob == rank ? db : cl.map_shared_rank(db, ob);
            }
            cl.sync();
            // (b) the 2x2 blocks of the local rows, written to the next buffers
            const float inv_np = 1.0f / (float)np;  // b / np exactly: the quotient's
            for (int b = t; b < nloc * np; b += blockDim.x) {  // fraction is >= 0.5 / np away
                const int li = (int)(((float)b + 0.5f) * inv_np);
                const int j = b - li * np;
                const int ki = k0 + li;
                const float4 ei = tab[ki], ej = tab[j];
                const float ci = ei.x, si = ei.y, cj = ej.x, sj = ej.y;
                const int pj = __float_as_int(ej.z), qj = __float_as_int(ej.w);
                const float *Tp = R + (size_t)(2 * li) * m, *Tq = Tp + m;
                float o11, o12, o21, o22;
                if (ki == j) {
                    const float app = Tp[pj], aqq = Tq[qj], apq = Tp[qj], aqp = Tq[pj];
                    if (si != 0.0f) {
                        const float t11 = ci * app - si * apq, t12 = ci * apq - si * aqq;
                        const float t21 = si * app + ci * apq, t22 = si * apq + ci * aqq;
                        o11 = t11 * ci - t12 * si;
                        o22 = t21 * si + t22 * ci;
                        o12 = o21 = 0.0f;
                    } else {
                        o11 = app;
                        o12 = apq;
                        o21 = aqp;
                        o22 = aqq;
                    }
                } else {
                    const float a11 = Tp[pj], a12 = Tp[qj], a21 = Tq[pj], a22 = Tq[qj];
                    const float t11 = ci * a11 - si * a21, t12 = ci * a12 - si * a22;
                    const float t21 = si * a11 + ci * a21, t22 = si * a12 + ci * a22;
                    o11 = t11 * cj - t12 * sj;
                    o12 = t11 * sj + t12 * cj;
                    o21 = t21 * cj - t22 * sj;
                    o22 = t21 * sj + t22 * cj;
                }
                float *dt = s_dst[2 * li], *db = s_dst[2 * li + 1];
                dt[pj] = o11;
                dt[qj] = o12;
                db[pj] = o21;
                db[qj] = o22;
            }
            cl.sync();
            cur ^= 1;
            ++round;
        }
    }
    if (rank == 0 && t == 0) {
        info[0] = round;
        info[1] = sweep;
        info[2] = converged;
    }
    cl.sync();  // no CTA leaves while another may still address its memory
}

// Largest dynamic shared memory the Jacobi kernel may request: the device's
// opt-in per-block limit minus the kernel's static shared memory.
static size_t jacobi_dyn_limit() {
    static PerDevice<size_t> cache;
    return cache.get([] {
        int optin = 0;
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, current_device());
        cudaFuncAttributes fa{};
        cudaFuncGetAttributes(&fa, k_jacobi32);
        return optin > 0 ? (size_t)optin - fa.sharedSizeBytes : (size_t)48 * 1024;
    });
}
// the same for the cluster kernel (its static shared memory differs)
static size_t jacobi_cluster_dyn_limit() {
    static PerDevice<size_t> cache;
    return cache.get([] {
        int optin = 0;
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, current_device());
        cudaFuncAttributes fa{};
        cudaFuncGetAttributes(&fa, k_jacobi32_cluster);
        return optin > 0 ? (size_t)optin - fa.sharedSizeBytes : (size_t)48 * 1024;
    });
}

// V = J_1 J_2 ... J_T, one warp per row of V: row r starts as e_r and every
// logged rotation (c, s, p, q) maps (v_p, v_q) -> (c v_p - s v_q, s v_p + c v_q).
// Lane l applies the rotations of pairs l, l + 32, ... (NS slots); the log of
// the next kRotGroup rounds is loaded while the current ones are applied, so
// the row's updates do not wait on the log's L2 latency.
constexpr int kRotGroup = 2;
template <int NS>
__global__ void __launch_bounds__(256)
k_apply_rotations(int s, const float4 *__restrict__ log, const int *__restrict__ info,
                  double *__restrict__ V, int ldv) {
    extern __shared__ float rows[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r = blockIdx.x * 8 + warp;
    if (r >= s) return;  // warp-uniform; the kernel has no block-wide barrier
    float *v = rows + (size_t)warp * s;
    const int np = jac_m(s) / 2;
    const int rounds = info[0];
    for (int j = lane; j < s; j += 32) v[j] = (j == r) ? 1.0f : 0.0f;
    __syncwarp();
    auto load = [&](float4 (&dst)[kRotGroup][NS], int t0) {
#pragma unroll
        for (int g = 0; g < kRotGroup; ++g)
#pragma unroll
            for (int k = 0; k < NS; ++k) {
                const int i = lane + 32 * k;
                dst[g][k] = (t0 + g < rounds && i < np) ? log[(size_t)(t0 + g) * np + i]
                                                        : make_float4(1.0f, 0.0f, 0.0f, 0.0f);
            }
    };
    float4 cur[kRotGroup][NS], nxt[kRotGroup][NS];
    load(cur, 0);
    for (int t0 = 0; t0 < rounds; t0 += kRotGroup) {
        load(nxt, t0 + kRotGroup);
#pragma unroll
        for (int g = 0; g < kRotGroup; ++g) {
#pragma unroll
            for (int k = 0; k < NS; ++k) {
                const float4 e = cur[g][k];
                if (e.y == 0.0f) continue;  // also every slot past np or past the last round
                const int p = __float_as_int(e.z), q = __float_as_int(e.w);
                if (p >= s || q >= s) continue;
                const float vp = v[p], vq = v[q];
                v[p] = e.x * vp - e.y * vq;
                v[q] = e.y * vp + e.x * vq;
            }
            __syncwarp();
        }
#pragma unroll
        for (int g = 0; g < kRotGroup; ++g)
#pragma unroll
            for (int k = 0; k < NS; ++k) cur[g][k] = nxt[g][k];
    }
    for (int j = lane; j < s; j += 32) V[r + (size_t)j * ldv] = (double)v[j];
}

template <int NS>
static void launch_rotations(int s, const float4 *log, const int *info, double *V, int ldv,
                             cudaStream_t st) {
    k_apply_rotations<NS><<<(s + 7) / 8, 256, (size_t)8 * s * sizeof(float), st>>>(s, log, info,
                                                                                  V, ldv);
}

// Whether a cluster of kJC CTAs with the largest shared memory the cluster
// kernel may use can be resident on this device (checked once).
static bool jacobi_cluster_usable() {
    static PerDevice<bool> cache;
    return cache.get([] {
        const size_t lim = jacobi_cluster_dyn_limit();
        if (cudaFuncSetAttribute(k_jacobi32_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)lim) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(kJC);
        cfg.blockDim = dim3(kJacobiThreads);
        cfg.dynamicSmemBytes = lim;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = kJC;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int n = 0;
        if (cudaOccupancyMaxActiveClusters(&n, k_jacobi32_cluster, &cfg) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        return n > 0;
    });
}

static int jacobi_cluster_max_dim() {
    const size_t lim = jacobi_cluster_dyn_limit();
    int s = kJacClusterMin;
    while (jacobi_cluster_smem_bytes(s + 1) <= lim && jc_slots(jac_m(s + 1) / 2) <= kJacMaxLocal)
        ++s;
    return s;
}

void EigWork::reserve(int smax) {
    const size_t s2 = (size_t)smax * smax;
    G.alloc(s2);
    W.alloc(s2);
    S.alloc(s2);
    C.alloc(s2);
    X.alloc(s2);
    X2.alloc(s2);
    lam.alloc(smax);
    delta.alloc(4);
    info.alloc(4);
    const int m = jac_m(smax);
    max_rounds = kMaxSweeps * (m - 1);
    log.alloc((size_t)max_rounds * (m / 2) + 1);  // (c, s, p, q) per pair and round
    gscr.alloc(gram_scratch_elems(smax, smax, smax));
    ozb.alloc(oz_lincomb_scratch_bytes(smax, smax));
    h_S.alloc(s2);
    h_C.alloc(2 * s2);
    h_lam.alloc(smax);
    h_info.alloc(8);
    std::fill(h_info.p, h_info.p + 8, 0.0);
    cap = smax;
}

// Cyclic FP64 Jacobi on a small dense symmetric block (host, row-major n x n
// in a), eigenvectors accumulated in v (column j = eigenvector j).
static void host_jacobi(int n, std::vector<double> &a, std::vector<double> &v) {
    v.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) v[(size_t)i * n + i] = 1.0;
    for (int sweep = 0; sweep < 60; ++sweep) {
        double off = 0.0, tot = 0.0;
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                tot += a[(size_t)i * n + j] * a[(size_t)i * n + j];
                if (i != j) off += a[(size_t)i * n + j] * a[(size_t)i * n + j];
            }
        if (off <= 1e-34 * tot || off == 0.0) break;
        for (int p = 0; p < n - 1; ++p)
            for (int q = p + 1; q < n; ++q) {
                const double apq = a[(size_t)p * n + q];
                if (apq == 0.0) continue;
                const double app = a[(size_t)p * n + p], aqq = a[(size_t)q * n + q];
                const double tau = (aqq - app) / (2.0 * apq);
                const double tt = (tau >= 0 ? 1.0 : -1.0) / (std::fabs(tau) + std::hypot(1.0, tau));
                const double c = 1.0 / std::sqrt(1.0 + tt * tt), sv = tt * c;
                for (int k = 0; k < n; ++k) {  // A <- A J (columns p, q)
                    const double akp = a[(size_t)k * n + p], akq = a[(size_t)k * n + q];
                    a[(size_t)k * n + p] = c * akp - sv * akq;
                    a[(size_t)k * n + q] = sv * akp + c * akq;
                }
                for (int k = 0; k < n; ++k) {  // A <- J^T A (rows p, q)
                    const double apk = a[(size_t)p * n + k], aqk = a[(size_t)q * n + k];
                    a[(size_t)p * n + k] = c * apk - sv * aqk;
                    a[(size_t)q * n + k] = sv * apk + c * aqk;
                }
                for (int k = 0; k < n; ++k) {
                    const double vkp = v[(size_t)k * n + p], vkq = v[(size_t)k * n + q];
                    v[(size_t)k * n + p] = c * vkp - sv * vkq;
                    v[(size_t)k * n + q] = sv * vkp + c * vkq;
                }
            }
    }
}

void host_eigh(int n, const double *G, double *w, double *V) {
    std::vector<double> a(G, G + (size_t)n * n), v;
    for (int i = 0; i < n; ++i)  // symmetrise (column-major in, row-major work)
        for (int j = 0; j < i; ++j) {
            const double m = 0.5 * (a[(size_t)i * n + j] + a[(size_t)j * n + i]);
            a[(size_t)i * n + j] = a[(size_t)j * n + i] = m;
        }
    host_jacobi(n, a, v);
    std::vector<int> ord(n);
    for (int i = 0; i < n; ++i) ord[i] = i;
    std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) {
        return a[(size_t)x * n + x] < a[(size_t)y * n + y];
    });
    for (int j = 0; j < n; ++j) {
        w[j] = a[(size_t)ord[j] * n + ord[j]];
        for (int i = 0; i < n; ++i) V[i + (size_t)j * n] = v[(size_t)i * n + ord[j]];
    }
}

// Eigen-decomposition of the symmetric s x s matrix M (device, ld) into
// ascending eigenvalues eval (host) and eigenvectors Z (device, ldz).
//
// Refinement step (after Ogita & Aishima): with G = X^T X, R = I - G and
// S = X^T M X, lambda_i = S_ii / G_ii and X <- X (I + E), where
// E_ij = (S_ij + lambda_j R_ij) / (lambda_j - lambda_i) for well-separated
// pairs and R_ij / 2 inside a cluster.  A cluster is a connected set of
// pairs whose first-order correction is not small (|E_ij| > 1e-2) or whose
// gap is below 1e-5 max|lambda| (there E_ij would mostly amplify rounding);
// each cluster block of S is diagonalised exactly in FP64 in the same step,
// so near-degenerate pairs come out orthonormal and resolved to FP64
// accuracy.  The update of a step with max|E| < 1e-9 is the last (its error
// is of the order max|E|^2 / gap); that step folds the ascending sort into the
// update and writes Z.
int sym_eig(EigWork &wk, int s, const double *M, int ld, double *eval_host, double *Z, int ldz,
            int refine_steps, cudaStream_t st, bool emulated) {
    GCGE_REQUIRE(s >= 1 && s <= wk.cap, GCGE_ERR_ARG, "sym_eig: size");
    {  // counts of the previous call (its copy has completed by now: every
       // caller synchronises the stream between two eigensolves)
        const int *hi = reinterpret_cast<const int *>(wk.h_info.p);
        wk.last_rounds = hi[0];
        wk.last_sweeps = hi[1];
    }
    GCGE_REQUIRE(s <= jacobi_max_dim(), GCGE_ERR_TOO_LARGE,
                 "sym_eig: projected dimension exceeds the shared-memory Jacobi capacity");
    static PerDevice<bool> smem_set;  // allow the largest size once per device
    smem_set.get([] {
        GCGE_CUDA(cudaFuncSetAttribute(k_jacobi32, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)jacobi_dyn_limit()));
        return true;
    });
    const bool cluster = s >= kJacClusterMin && jacobi_cluster_usable() &&
                         jacobi_cluster_smem_bytes(s) <= jacobi_cluster_dyn_limit() &&
                         jc_slots(jac_m(s) / 2) <= kJacMaxLocal;
    if (cluster) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(kJC);
        cfg.blockDim = dim3(kJacobiThreads);
        cfg.dynamicSmemBytes = jacobi_cluster_smem_bytes(s);
        cfg.stream = st;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = kJC;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        GCGE_CUDA(cudaLaunchKernelEx(&cfg, k_jacobi32_cluster, s, M, ld, wk.log.p, wk.max_rounds,
                                     wk.info.p));
    } else {
        GCGE_REQUIRE(jacobi_smem_bytes(s) <= jacobi_dyn_limit(), GCGE_ERR_TOO_LARGE,
                     "sym_eig: projected dimension exceeds the one-CTA Jacobi capacity");
        k_jacobi32<<<1, kJacobiThreads, jacobi_smem_bytes(s), st>>>(s, M, ld, wk.log.p,
                                                                    wk.max_rounds, wk.info.p);
    }
    GCGE_CHECK_LAUNCH();
    switch ((jac_m(s) / 2 + 31) / 32) {
        case 1: launch_rotations<1>(s, wk.log.p, wk.info.p, wk.X.p, s, st); break;
        case 2: launch_rotations<2>(s, wk.log.p, wk.info.p, wk.X.p, s, st); break;
        case 3: launch_rotations<3>(s, wk.log.p, wk.info.p, wk.X.p, s, st); break;
        case 4: launch_rotations<4>(s, wk.log.p, wk.info.p, wk.X.p, s, st); break;
        case 5: launch_rotations<5>(s, wk.log.p, wk.info.p, wk.X.p, s, st); break;
        case 6: launch_rotations<6>(s, wk.log.p, wk.info.p, wk.X.p, s, st); break;
        case 7: launch_rotations<7>(s, wk.log.p, wk.info.p, wk.X.p, s, st); break;
        default: launch_rotations<8>(s, wk.log.p, wk.info.p, wk.X.p, s, st); break;
    }
    GCGE_CHECK_LAUNCH();
    count_launch(2);
    const int lds = s;
    double *X = wk.X.p, *Xn = wk.X2.p;
    // s x s products of the refinement: X^T P (ld s) and A B (ld of A given)
    auto sgram = [&](const double *P, double *C) {
        if (emulated)
            oz_gram(s, s, s, X, lds, P, lds, C, lds, wk.gscr.p, wk.gscr.n, st);
        else
            gram(s, s, s, X, lds, P, lds, C, lds, wk.gscr.p, wk.gscr.n, st);
    };
    auto slincomb = [&](const double *A, int lda, const double *B, double *Y, int ldy) {
        if (emulated)
            oz_lincomb(s, s, s, A, lda, B, lds, Y, ldy, nullptr, 0, st, 1.0, wk.ozb.p, wk.ozb.n);
        else
            lincomb(s, s, s, A, lda, B, lds, Y, ldy, nullptr, 0, st);
    };
    const size_t s2 = (size_t)s * s;
    double *hS = wk.h_S.p, *hG = wk.h_C.p + s2, *hC = wk.h_C.p;
    std::vector<double> lam(s);
    std::vector<int> ord(s), comp(s), parent(s);
    auto find = [&](int x) {
        while (parent[x] != x) {
            parent[x] = parent[parent[x]];
            x = parent[x];
        }
        return x;
    };
    const int steps = std::max(2, refine_steps);
    for (int step = 0; step < steps; ++step) {
        sgram(X, wk.G.p);
        slincomb(M, ld, X, wk.W.p, lds);
        sgram(wk.W.p, wk.S.p);
        GCGE_CUDA(cudaMemcpyAsync(hS, wk.S.p, sizeof(double) * s2, cudaMemcpyDeviceToHost, st));
        GCGE_CUDA(cudaMemcpyAsync(hG, wk.G.p, sizeof(double) * s2, cudaMemcpyDeviceToHost, st));
        GCGE_CUDA(cudaStreamSynchronize(st));
        double scale = 0.0;
        for (int i = 0; i < s; ++i) {
            lam[i] = hS[i + (size_t)i * s] / hG[i + (size_t)i * s];
            GCGE_REQUIRE(std::isfinite(lam[i]), GCGE_ERR_NUMERIC, "sym_eig: non-finite eigenvalue");
            scale = std::max(scale, std::fabs(lam[i]));
        }
        // E_ij = (S_ij + lam_j R_ij) / (lam_j - lam_i); pairs whose correction is
        // not small, or whose gap is below kClusterGap * scale, join one cluster
        for (int i = 0; i < s; ++i) parent[i] = i;
        for (int j = 0; j < s; ++j)
            for (int i = 0; i < s; ++i) {
                const double rij = (i == j ? 1.0 : 0.0) - hG[i + (size_t)j * s];
                double e = 0.5 * rij;
                if (i != j) {
                    const double gap = lam[j] - lam[i];
                    e = (hS[i + (size_t)j * s] + lam[j] * rij) / gap;
                    if (!(std::fabs(gap) > kClusterGap * scale) || !(std::fabs(e) <= kStrongCoupling)) {
                        const int a = find(i), b = find(j);
                        if (a != b) parent[a] = b;
                    }
                }
                hC[i + (size_t)j * s] = e;  // E for now
            }
        for (int i = 0; i < s; ++i) comp[i] = find(i);
        double emax = 0.0;
        for (int j = 0; j < s; ++j)
            for (int i = 0; i < s; ++i) {
                double &e = hC[i + (size_t)j * s];
                if (i != j && comp[i] == comp[j]) e = 0.5 * ((i == j ? 1.0 : 0.0) - hG[i + (size_t)j * s]);
                emax = std::max(emax, std::fabs(e));
                if (i == j) e += 1.0;  // C = I + E
            }
        // exact FP64 diagonalisation of each cluster block of S
        std::iota(ord.begin(), ord.end(), 0);
        std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) {
            return comp[a] != comp[b] ? comp[a] < comp[b] : a < b;
        });
        int k = 0;
        while (k < s) {
            int e = k + 1;
            while (e < s && comp[ord[e]] == comp[ord[k]]) ++e;
            const int c = e - k;
            if (c > 1) {
                // the cluster block of (I + E)^T S (I + E): its in-cluster part
                // T = I + E_c (first-order G_c^{-1/2}) carries the off-diagonal
                // Gram entries, so the block's eigenvalues are accurate to
                // second order in them; the cross terms through entries of E
                // outside the cluster are second order too
                std::vector<double> Sc((size_t)c * c), Tc((size_t)c * c), ST((size_t)c * c);
                std::vector<double> blk((size_t)c * c), vec;
                for (int a = 0; a < c; ++a)
                    for (int b = 0; b < c; ++b) {
                        const int ia = ord[k + a], ib = ord[k + b];
                        Sc[(size_t)a * c + b] = 0.5 * (hS[ia + (size_t)ib * s] + hS[ib + (size_t)ia * s]);
                        Tc[(size_t)a * c + b] = hC[ia + (size_t)ib * s];  // row a, column b
                    }
                for (int a = 0; a < c; ++a)  // ST = Sc Tc
                    for (int b = 0; b < c; ++b) {
                        double v = 0.0;
                        for (int u = 0; u < c; ++u) v += Sc[(size_t)a * c + u] * Tc[(size_t)u * c + b];
                        ST[(size_t)a * c + b] = v;
                    }
                for (int a = 0; a < c; ++a)  // blk = Tc^T ST
                    for (int b = 0; b < c; ++b) {
                        double v = 0.0;
                        for (int u = 0; u < c; ++u) v += Tc[(size_t)u * c + a] * ST[(size_t)u * c + b];
                        blk[(size_t)a * c + b] = v;
                    }
                for (int a = 0; a < c; ++a)
                    for (int b = 0; b < a; ++b) {
                        const double v = 0.5 * (blk[(size_t)a * c + b] + blk[(size_t)b * c + a]);
                        blk[(size_t)a * c + b] = blk[(size_t)b * c + a] = v;
                    }
                host_jacobi(c, blk, vec);
                std::vector<double> tmp((size_t)s * c, 0.0);
                for (int b = 0; b < c; ++b)
                    for (int a = 0; a < c; ++a) {
                        const double v = vec[(size_t)a * c + b];
                        if (v == 0.0) continue;
                        const double *src = hC + (size_t)ord[k + a] * s;
                        double *dst = tmp.data() + (size_t)b * s;
                        for (int i = 0; i < s; ++i) dst[i] += src[i] * v;
                    }
                for (int b = 0; b < c; ++b) {
                    std::copy(tmp.begin() + (size_t)b * s, tmp.begin() + (size_t)(b + 1) * s,
                              hC + (size_t)ord[k + b] * s);
                    lam[ord[k + b]] = blk[(size_t)b * c + b];
                }
            }
            k = e;
        }
        // the step's error is second order in emax (first order inside clusters,
        // which are diagonalised exactly), so once emax < 1e-9 this update is
        // the last one needed
        const bool last = (step == steps - 1) || emax < 1e-9;
        wk.last_steps = step + 1;
        if (!last) {
            GCGE_CUDA(cudaMemcpyAsync(wk.C.p, hC, sizeof(double) * s2, cudaMemcpyHostToDevice, st));
            slincomb(X, lds, wk.C.p, Xn, lds);
            std::swap(X, Xn);
            // hC is rewritten only after the next step's synchronisation, which
            // follows this copy on the stream
            continue;
        }
        // final: ascending order folded into the update
        std::iota(ord.begin(), ord.end(), 0);
        std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return lam[a] < lam[b]; });
        double *hP = wk.h_S.p;  // S is no longer needed
        for (int j = 0; j < s; ++j) {
            std::copy(hC + (size_t)ord[j] * s, hC + (size_t)(ord[j] + 1) * s, hP + (size_t)j * s);
            eval_host[j] = lam[ord[j]];
        }
        GCGE_CUDA(cudaMemcpyAsync(wk.C.p, hP, sizeof(double) * s2, cudaMemcpyHostToDevice, st));
        slincomb(X, lds, wk.C.p, Z, ldz);
        wk.last_delta = emax;
        break;
    }
    // the Jacobi's round and sweep counts reach the host with the caller's
    // next synchronisation (no wait here); the next call reads them
    GCGE_CUDA(cudaMemcpyAsync(wk.h_info.p, wk.info.p, sizeof(int) * 3, cudaMemcpyDeviceToHost,
                              st));
    return GCGE_OK;
}

}  // namespace gcge
