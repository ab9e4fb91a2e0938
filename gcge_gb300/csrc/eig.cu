// Dense symmetric eigensolver for the Rayleigh-Ritz projected matrix
// (replaces the reference's dsyevx call, src/ops_eig_sol_gcg.c:1145-1150 /
// :1207-1209: all eigenpairs, ascending).
//
// GB300 issues FP64 at ~1/58 of its FP32 rate, so an FP64 Jacobi on one SM
// would take tens of milliseconds for s = 200.  The solver therefore
//   1. runs a parallel-order (round-robin) two-sided cyclic Jacobi in FP32 in
//      one 1024-thread CTA, with the packed upper triangle of the matrix in
//      shared memory (s <= 336), logging each round's rotations;
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
#include <mutex>
#include <algorithm>
#include <cmath>
#include <numeric>

#include "common.cuh"
#include "eig.cuh"

namespace gcge {

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
int jacobi_max_dim() {
    const size_t lim = jacobi_dyn_limit();
    int s = 8;
    while (jacobi_smem_bytes(s + 1) <= lim) ++s;
    return s;
}

__global__ void __launch_bounds__(kJacobiThreads)
k_jacobi32(int s, const double *__restrict__ M, int ldm, float2 *__restrict__ log, int max_rounds,
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
                log[(size_t)round * np + i] = make_float2(cs[i], sn[i]);
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

// Largest dynamic shared memory the Jacobi kernel may request: the device's
// opt-in per-block limit minus the kernel's static shared memory.
static size_t jacobi_dyn_limit() {
    static std::once_flag once;
    static size_t lim = 0;
    std::call_once(once, [] {
        int dev = 0, optin = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        cudaFuncAttributes fa{};
        cudaFuncGetAttributes(&fa, k_jacobi32);
        lim = optin > 0 ? (size_t)optin - fa.sharedSizeBytes : 48 * 1024;
    });
    return lim;
}

// V = J_1 J_2 ... J_T, one warp per row of V: row r starts as e_r and every
// logged rotation (p, q, c, s) maps (v_p, v_q) -> (c v_p - s v_q, s v_p + c v_q).
// Lane l applies the rotations of pairs l, l + 32, ... (NS slots); the log of
// the next kRotGroup rounds is loaded while the current ones are applied, so
// the row's updates do not wait on the log's L2 latency.
constexpr int kRotGroup = 4;
template <int NS>
__global__ void __launch_bounds__(256)
k_apply_rotations(int s, const float2 *__restrict__ log, const int *__restrict__ info,
                  double *__restrict__ V, int ldv) {
    extern __shared__ float rows[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r = blockIdx.x * 8 + warp;
    if (r >= s) return;  // warp-uniform; the kernel has no block-wide barrier
    float *v = rows + (size_t)warp * s;
    const int m = jac_m(s), np = m / 2, m1 = m - 1;
    const int rounds = info[0];
    for (int j = lane; j < s; j += 32) v[j] = (j == r) ? 1.0f : 0.0f;
    __syncwarp();
    auto load = [&](float2 (&dst)[kRotGroup][NS], int t0) {
#pragma unroll
        for (int g = 0; g < kRotGroup; ++g)
#pragma unroll
            for (int k = 0; k < NS; ++k) {
                const int i = lane + 32 * k;
                dst[g][k] = (t0 + g < rounds && i < np) ? log[(size_t)(t0 + g) * np + i]
                                                        : make_float2(1.0f, 0.0f);
            }
    };
    float2 cur[kRotGroup][NS], nxt[kRotGroup][NS];
    load(cur, 0);
    int rr = 0;  // round within the sweep
    for (int t0 = 0; t0 < rounds; t0 += kRotGroup) {
        load(nxt, t0 + kRotGroup);
#pragma unroll
        for (int g = 0; g < kRotGroup; ++g) {
#pragma unroll
            for (int k = 0; k < NS; ++k) {
                const int i = lane + 32 * k;
                const float2 cs = cur[g][k];
                if (cs.y == 0.0f) continue;  // also every slot past np or past the last round
                int a, b;
                if (i == 0) {
                    a = m1;
                    b = rr;
                } else {
                    a = rr + i;
                    if (a >= m1) a -= m1;
                    b = rr - i;
                    if (b < 0) b += m1;
                }
                const int p = min(a, b), q = max(a, b);
                if (q >= s) continue;
                const float vp = v[p], vq = v[q];
                v[p] = cs.x * vp - cs.y * vq;
                v[q] = cs.y * vp + cs.x * vq;
            }
            __syncwarp();
            if (++rr == m1) rr = 0;
        }
#pragma unroll
        for (int g = 0; g < kRotGroup; ++g)
#pragma unroll
            for (int k = 0; k < NS; ++k) cur[g][k] = nxt[g][k];
    }
    for (int j = lane; j < s; j += 32) V[r + (size_t)j * ldv] = (double)v[j];
}

template <int NS>
static void launch_rotations(int s, const float2 *log, const int *info, double *V, int ldv,
                             cudaStream_t st) {
    k_apply_rotations<NS><<<(s + 7) / 8, 256, (size_t)8 * s * sizeof(float), st>>>(s, log, info,
                                                                                  V, ldv);
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
    log.alloc((size_t)max_rounds * (m / 2) + 1);
    gscr.alloc(gram_scratch_elems(smax, smax, smax));
    h_S.alloc(s2);
    h_C.alloc(2 * s2);
    h_lam.alloc(smax);
    h_info.alloc(8);
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
            int refine_steps, cudaStream_t st) {
    GCGE_REQUIRE(s >= 1 && s <= wk.cap, GCGE_ERR_ARG, "sym_eig: size");
    GCGE_REQUIRE(s <= jacobi_max_dim(), GCGE_ERR_TOO_LARGE,
                 "sym_eig: projected dimension exceeds the shared-memory Jacobi capacity");
    const size_t smem = jacobi_smem_bytes(s);
    static std::once_flag once;  // allow the largest size once, for every caller thread
    std::call_once(once, [] {
        GCGE_CUDA(cudaFuncSetAttribute(k_jacobi32, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)jacobi_dyn_limit()));
    });
    k_jacobi32<<<1, kJacobiThreads, smem, st>>>(s, M, ld, wk.log.p, wk.max_rounds, wk.info.p);
    GCGE_CHECK_LAUNCH();
    switch ((jac_m(s) / 2 + 31) / 32) {
        case 1: launch_rotations<1>(s, wk.log.p, wk.info.p, wk.X.p, s, st); break;
        case 2: launch_rotations<2>(s, wk.log.p, wk.info.p, wk.X.p, s, st); break;
        case 3: launch_rotations<3>(s, wk.log.p, wk.info.p, wk.X.p, s, st); break;
        case 4: launch_rotations<4>(s, wk.log.p, wk.info.p, wk.X.p, s, st); break;
        case 5: launch_rotations<5>(s, wk.log.p, wk.info.p, wk.X.p, s, st); break;
        default: launch_rotations<6>(s, wk.log.p, wk.info.p, wk.X.p, s, st); break;
    }
    GCGE_CHECK_LAUNCH();
    count_launch(2);
    const int lds = s;
    double *X = wk.X.p, *Xn = wk.X2.p;
    const size_t gs = wk.gscr.n;
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
        gram(s, s, s, X, lds, X, lds, wk.G.p, lds, wk.gscr.p, gs, st);
        lincomb(s, s, s, M, ld, X, lds, wk.W.p, lds, nullptr, 0, st);
        gram(s, s, s, X, lds, wk.W.p, lds, wk.S.p, lds, wk.gscr.p, gs, st);
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
                std::vector<double> blk((size_t)c * c), vec;
                for (int a = 0; a < c; ++a)
                    for (int b = 0; b < c; ++b) {
                        const int ia = ord[k + a], ib = ord[k + b];
                        blk[(size_t)a * c + b] = 0.5 * (hS[ia + (size_t)ib * s] + hS[ib + (size_t)ia * s]) /
                                                 std::sqrt(hG[ia + (size_t)ia * s] * hG[ib + (size_t)ib * s]);
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
            lincomb(s, s, s, X, lds, wk.C.p, lds, Xn, lds, nullptr, 0, st);
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
        lincomb(s, s, s, X, lds, wk.C.p, lds, Z, ldz, nullptr, 0, st);
        wk.last_delta = emax;
        break;
    }
    int hinfo[3] = {0, 0, 0};
    GCGE_CUDA(cudaMemcpyAsync(hinfo, wk.info.p, sizeof(int) * 3, cudaMemcpyDeviceToHost, st));
    GCGE_CUDA(cudaStreamSynchronize(st));
    wk.last_rounds = hinfo[0];
    wk.last_sweeps = hinfo[1];
    return GCGE_OK;
}

}  // namespace gcge
