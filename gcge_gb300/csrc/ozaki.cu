// FP64-accurate dense products on the bf16 tensor cores, for the
// mixed-precision GCG: the tall-skinny Gram products Q^T P (B-orthogonalisation,
// Rayleigh-Ritz) and the linear combinations Y = X C (orth updates, Ritz
// vectors, P), the calls the reference makes through DenseMatQtAP and
// MultiVecLinearComb (app/app_lapack.c:64-183, :463-534).  GB300's FP64 units
// run at about 1.2 TFLOP/s; these products dominate the FP64 solve.
//
// Method (error-free digit splitting, the Ozaki scheme): within each chunk of
// kBK = 64 consecutive k, every row of the left operand and every column of
// the right operand gets an exponent e with |x| < 2^e over the chunk, and each
// |x| becomes a 56-bit fixed-point integer X = |x| 2^(56 - e) (truncated)
// written with 7 digits of 8 bits, X = sum_i d_i 2^(8(6-i)): the leading digit
// d_0 in [0, 256] and balanced digits d_1..d_6 in [-128, 127] (the bytes of
// X + 0x808080808080, less 128), each carrying x's sign.  Digits are exact in
// bf16.  A chunk's product sum_k x_k y_k is 2^(ea+eb-112) * sum_l L_l
// 2^(8(12-l)) with level sums L_l = sum_{i+j=l} sum_k d_i(x_k) d_j(y_k),
// l = 0..6 (the 28 digit pairs with i + j <= 6).  |L_l| <= 64 (2 * 256 * 128
// + 5 * 128^2) < 2^24, so the level sums of bf16 products accumulated in FP32
// by mma.sync are exact integers.  After the chunk they are folded into two
// exact int64 words, converted exactly to FP64 and added, with the chunk
// scale, into FP64 accumulators.  The truncation error is below 2^-55 of the
// chunk's largest |x| |y| per product, the same order as FP64 rounding;
// non-finite inputs give NaN outputs.
//
// Tiles: a CTA computes a 64 x BN block of the result for a range of k; the
// operands' digit planes for one chunk sit in shared memory (7 planes each,
// rows padded to 72 bf16 so ldmatrix is conflict-free) and each warp owns a
// 16 x 8 tile: per 16-wide k step it loads 7 A and 7 B digit fragments and
// issues 28 MMAs into 7 level accumulators.  Gram products split k over CTAs
// (partials summed in a fixed order); linear combinations tile the long row
// dimension and keep k whole.
#include <cstdint>
#include <mutex>

#include "common.cuh"

namespace gcge {
namespace {

constexpr int kDigits = 7;
constexpr int kBK = 64;
constexpr int kBKP = kBK + 8;
constexpr int kBM = 64;
constexpr int kSuper = 8;  // chunks per shared exponent (int64 sums stay below 2^51)

template <int BN>
struct __align__(16) OzSmem {
    uint16_t a[kDigits][kBM][kBKP];
    uint16_t b[kDigits][BN][kBKP];
    int ea[kBM], eb[BN];  // chunk exponent fields (biased, >= 1)
};

template <int BN>
__host__ __device__ constexpr int oz_threads() {
    return (kBM / 16) * (BN / 8) * 32;
}

// biased exponent field, zero and subnormals counted as 1
__device__ __forceinline__ int exp_field(double x) {
    return max((int)((__double_as_longlong(x) >> 52) & 0x7FF), 1);
}

// x as a 56-bit fixed-point magnitude X relative to 2^(emax - 1022) (emax >=
// exp_field(x)), plus 128 in each of its six low bytes (so that byte - 128 is
// a balanced digit), split into 32-bit words, and the bias word of its digits:
// +2^23 or -2^23 as an FP32 bit pattern, carrying x's sign.
struct Fixed56 {
    uint32_t hi, lo;
    uint32_t magic;
};
__device__ __forceinline__ Fixed56 fixed56(double x, int emax) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int ef = (int)((b >> 52) & 0x7FF);
    unsigned long long mant = b & 0x000FFFFFFFFFFFFFull;
    if (ef != 0) mant |= 0x0010000000000000ull;
    const int sh = max(ef, 1) - emax + 3;  // <= 3: the value < 2^56 in fixed point
    const unsigned long long X = sh >= 0 ? (mant << sh) : (sh > -64 ? (mant >> (-sh)) : 0ull);
    const unsigned long long Y = X + 0x0000808080808080ull;  // < 2^57
    Fixed56 f;
    f.hi = (uint32_t)(Y >> 32);
    f.lo = (uint32_t)Y;
    f.magic = 0x4B000000u | ((uint32_t)(b >> 32) & 0x80000000u);
    return f;
}

// Digit i as an FP32 number: (bias | t) read as FP32 is +-(2^23 + t) for the
// field t (bits 48.. of the biased value for i = 0, else its byte 6 - i), and
// subtracting +-2^23 (i = 0) or +-(2^23 + 128) leaves +-d_i exactly.  Its
// upper 16 bits are its bf16 pattern.
template <int I>
__device__ __forceinline__ uint32_t digit_f32(const Fixed56 &f) {
    float v;
    if constexpr (I == 0) {
        v = __uint_as_float((f.hi >> 16) | f.magic) - __uint_as_float(f.magic);
    } else {
        constexpr int s = 48 - 8 * I;
        uint32_t t;
        if constexpr (s >= 32)
            t = f.hi >> (s - 32);
        else
            t = __funnelshift_r(f.lo, f.hi, s);
        v = __uint_as_float((t & 255u) | f.magic) - __uint_as_float(f.magic | 128u);
    }
    return __float_as_uint(v);
}

// The 8 digit planes of two values (consecutive k of one row): word i holds
// digit i of x0 in its low and of x1 in its high bf16 half.
template <int I = 0>
__device__ __forceinline__ void digit_pairs(const Fixed56 &a, const Fixed56 &b,
                                            uint32_t (&w)[kDigits]) {
    if constexpr (I < kDigits) {
        w[I] = __byte_perm(digit_f32<I>(a), digit_f32<I>(b), 0x7632);
        digit_pairs<I + 1>(a, b, w);
    }
}

// exact int64 -> double for |t| < 2^51
__device__ __forceinline__ double i64_to_f64(long long t) {
    return __longlong_as_double(t + 0x4338000000000000LL) - 6755399441055744.0;
}

__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], const void *p) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(a));
}
__device__ __forceinline__ void ldsm_x2(uint32_t (&r)[2], const void *p) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];"
                 : "=r"(r[0]), "=r"(r[1])
                 : "r"(a));
}
__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4],
                                         const uint32_t (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
        "{%8,%9}, {%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// Exponent fields (max over [k0, kend), at least 1) of R rows of a
// k-contiguous operand: warp w takes rows w, w + NW, ...; the loads of all of
// a warp's rows for one k are issued together, so their latencies overlap.
template <int R, int NW>
__device__ __forceinline__ void exps_kcontig(const double *__restrict__ p, size_t ld, int r0,
                                             int nrows, int k0, int kend, int *e, int warp,
                                             int lane) {
    constexpr int RPW = (R + NW - 1) / NW;
    int em[RPW];
    const double *q[RPW];
#pragma unroll
    for (int t = 0; t < RPW; ++t) {
        const int r = warp + t * NW;
        em[t] = 1;
        q[t] = (r < R && r0 + r < nrows) ? p + (size_t)(r0 + r) * ld : nullptr;
    }
#pragma unroll 2
    for (int k = k0 + lane; k < kend; k += 32) {
#pragma unroll
        for (int t = 0; t < RPW; ++t)
            if (q[t]) em[t] = max(em[t], exp_field(q[t][k]));
    }
#pragma unroll
    for (int t = 0; t < RPW; ++t) {
        const int r = warp + t * NW;
        const int m = (int)__reduce_max_sync(0xffffffffu, (unsigned)em[t]);
        if (lane == 0 && r < R) e[r] = m;
    }
}

// The same for the kBM rows of an m-contiguous operand: NT / kBM threads per
// row (consecutive threads read consecutive rows), shared-memory maximum.
// e[] must hold 1 for every row beforehand.
template <int NT>
__device__ __forceinline__ void exps_mcontig(const double *__restrict__ p, size_t ld, int m0,
                                             int nrows, int k0, int kend, int *e, int tid) {
    constexpr int groups = NT / kBM;
    const int r = tid % kBM, g0 = tid / kBM;
    const int gr = m0 + r;
    int em = 1;
    if (gr < nrows && g0 < groups)
        for (int k = k0 + g0; k < kend; k += groups) em = max(em, exp_field(p[gr + (size_t)k * ld]));
    atomicMax(&e[r], em);
}

// Digit planes of R rows of a k-contiguous operand (element (r, k) at
// p[k + r * ld]) for the chunk [k0, k0 + kBK) clipped to kend, relative to the
// exponent fields e[r]; rows at or past nrows are zero.  One warp per row,
// lane l takes k = k0 + 2l, k0 + 2l + 1.
template <int R, int NW>
__device__ __forceinline__ void planes_kcontig(const double *__restrict__ p, size_t ld, int r0,
                                               int nrows, int k0, int kend,
                                               uint16_t (*planes)[R][kBKP], int *e, int warp,
                                               int lane) {
    // all of the warp's rows are loaded before any is split, so the loads'
    // latencies overlap
    constexpr int RPW = (R + NW - 1) / NW;
    const int k = k0 + 2 * lane;
    double v0[RPW], v1[RPW];
#pragma unroll
    for (int t = 0; t < RPW; ++t) {
        const int r = warp + t * NW, gr = r0 + r;
        v0[t] = v1[t] = 0.0;
        if (r < R && gr < nrows) {
            const double *q = p + (size_t)gr * ld;
            if (k < kend) v0[t] = q[k];
            if (k + 1 < kend) v1[t] = q[k + 1];
        }
    }
#pragma unroll
    for (int t = 0; t < RPW; ++t) {
        const int r = warp + t * NW;
        if (r >= R) break;
        const int em = e[r];
        uint32_t w[kDigits];
        digit_pairs(fixed56(v0[t], em), fixed56(v1[t], em), w);
#pragma unroll
        for (int i = 0; i < kDigits; ++i)
            *reinterpret_cast<uint32_t *>(&planes[i][r][2 * lane]) = w[i];
    }
}

// Digit planes of kBM rows of an m-contiguous operand (element (m, k) at
// p[m + k * ld]) relative to the exponent fields e[r]; a work item is one row
// and 8 consecutive k.
template <int NT>
__device__ __forceinline__ void planes_mcontig(const double *__restrict__ p, size_t ld, int m0,
                                               int nrows, int k0, int kend,
                                               uint16_t (*planes)[kBM][kBKP], const int *e,
                                               int tid) {
    constexpr int items = kBM * (kBK / 8);
    for (int it = tid; it < items; it += NT) {
        const int r = it % kBM, k8 = it / kBM;
        const int gr = m0 + r;
        const int em = e[r];
        uint32_t w[kDigits][4];
#pragma unroll
        for (int q = 0; q < 8; q += 2) {
            const int k = k0 + k8 * 8 + q;
            double v0 = 0.0, v1 = 0.0;
            if (gr < nrows) {
                if (k < kend) v0 = p[gr + (size_t)k * ld];
                if (k + 1 < kend) v1 = p[gr + (size_t)(k + 1) * ld];
            }
            uint32_t wp[kDigits];
            digit_pairs(fixed56(v0, em), fixed56(v1, em), wp);
#pragma unroll
            for (int i = 0; i < kDigits; ++i) w[i][q / 2] = wp[i];
        }
#pragma unroll
        for (int i = 0; i < kDigits; ++i)
            *reinterpret_cast<uint4 *>(&planes[i][r][k8 * 8]) =
                make_uint4(w[i][0], w[i][1], w[i][2], w[i][3]);
    }
}

struct OzArgs {
    int M, N;
    const double *A;  // gram: Q (n x M, k-contiguous rows of Q^T); lincomb: X (M x K)
    size_t lda;
    const double *B;  // gram: P (n x N); lincomb: C (K x N); both k-contiguous
    size_t ldb;
    int kbeg_stride;  // k per CTA along blockIdx.z
    int K;
    // gram output: partials part[z][M x N]; lincomb output: Y
    double *out;
    size_t ldo;
    const double *beta;
    int incb;
    double alpha;
    // lincomb: the right operand's exponent fields and digit planes, prepared
    // once per call (k_oz_bprep) instead of by every CTA of the long operand
    const uint16_t *bplanes;  // [tile][chunk][kDigits][BN][kBKP]
    const int *bexps;         // [tile][super-chunk][BN]
    int nchunks, nsup;
};

// Exponent fields and digit planes of the right operand of a linear
// combination (C, K x N, k-contiguous), for every super-chunk and chunk of K
// and every BN-column tile: block (super-chunk, tile).  The same device
// functions as the product kernel fill shared memory, which is then copied
// out, so the planes are bit for bit those the product kernel would make.
template <int BN>
__global__ void __launch_bounds__(oz_threads<BN>()) k_oz_bprep(const double *__restrict__ C,
                                                              size_t ldc, int N, int K,
                                                              uint16_t *__restrict__ planes,
                                                              int *__restrict__ exps, int nchunks,
                                                              int nsup) {
    constexpr int NT = oz_threads<BN>();
    constexpr int nwarps = NT / 32;
    constexpr int PL = kDigits * BN * kBKP;  // uint16 per chunk
    __shared__ __align__(16) uint16_t b[kDigits][BN][kBKP];
    __shared__ int eb[BN];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int s = blockIdx.x, nt = blockIdx.y, nt0 = nt * BN;
    const int sk = s * kSuper * kBK, ske = min(K, sk + kSuper * kBK);
    exps_kcontig<BN, nwarps>(C, ldc, nt0, N, sk, ske, eb, warp, lane);
    __syncthreads();
    for (int i = tid; i < BN; i += NT) exps[((size_t)nt * nsup + s) * BN + i] = eb[i];
    for (int k0 = sk; k0 < ske; k0 += kBK) {
        planes_kcontig<BN, nwarps>(C, ldc, nt0, N, k0, ske, b, eb, warp, lane);
        __syncthreads();
        const uint4 *src = reinterpret_cast<const uint4 *>(&b[0][0][0]);
        uint4 *dst = reinterpret_cast<uint4 *>(planes + ((size_t)nt * nchunks + k0 / kBK) * PL);
        for (int i = tid; i < PL / 8; i += NT) dst[i] = src[i];
        __syncthreads();
    }
}

template <int BN, bool GRAM>
__global__ void __launch_bounds__(oz_threads<BN>(), 2) k_oz_gemm(OzArgs a) {
    constexpr int NT = oz_threads<BN>();
    constexpr int nwarps = NT / 32;
    extern __shared__ __align__(16) unsigned char oz_raw[];
    OzSmem<BN> &sm = *reinterpret_cast<OzSmem<BN> *>(oz_raw);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int mt0 = blockIdx.x * kBM, nt0 = blockIdx.y * BN;
    const int kb = blockIdx.z * a.kbeg_stride;
    const int ke = min(a.K, kb + a.kbeg_stride);
    const int wm = warp % (kBM / 16), wn = warp / (kBM / 16);
    const int m0 = wm * 16, n0 = wn * 8;
    const int g = lane >> 2, t4 = lane & 3;

    double acc[4] = {0.0, 0.0, 0.0, 0.0};  // NaN once a non-finite input was seen

    // super-chunks of kSuper chunks share one exponent per row and column, so
    // the exact level sums of their chunks add up in int64 and are folded into
    // FP64 once per super-chunk
    for (int sk = kb; sk < ke; sk += kSuper * kBK) {
        const int ske = min(ke, sk + kSuper * kBK);
        if constexpr (GRAM) {
            exps_kcontig<kBM, nwarps>(a.A, a.lda, mt0, a.M, sk, ske, sm.ea, warp, lane);
        } else {
            for (int r = tid; r < kBM; r += NT) sm.ea[r] = 1;
            __syncthreads();
            exps_mcontig<NT>(a.A, a.lda, mt0, a.M, sk, ske, sm.ea, tid);
        }
        if constexpr (GRAM) {
            exps_kcontig<BN, nwarps>(a.B, a.ldb, nt0, a.N, sk, ske, sm.eb, warp, lane);
        } else {
            const int *e = a.bexps + ((size_t)blockIdx.y * a.nsup + sk / (kSuper * kBK)) * BN;
            for (int i = tid; i < BN; i += NT) sm.eb[i] = e[i];
        }
        __syncthreads();
        long long thi[4] = {0, 0, 0, 0}, tlo[4] = {0, 0, 0, 0};
        for (int k0 = sk; k0 < ske; k0 += kBK) {
            if constexpr (GRAM)
                planes_kcontig<kBM, nwarps>(a.A, a.lda, mt0, a.M, k0, ske, sm.a, sm.ea, warp, lane);
            else
                planes_mcontig<NT>(a.A, a.lda, mt0, a.M, k0, ske, sm.a, sm.ea, tid);
            if constexpr (GRAM) {
                planes_kcontig<BN, nwarps>(a.B, a.ldb, nt0, a.N, k0, ske, sm.b, sm.eb, warp, lane);
            } else {
                constexpr int PL = kDigits * BN * kBKP;
                const uint4 *src = reinterpret_cast<const uint4 *>(
                    a.bplanes + ((size_t)blockIdx.y * a.nchunks + k0 / kBK) * PL);
                uint4 *dst = reinterpret_cast<uint4 *>(&sm.b[0][0][0]);
                for (int i = tid; i < PL / 8; i += NT) dst[i] = src[i];
            }
            __syncthreads();

            float lv[kDigits][4];
#pragma unroll
            for (int l = 0; l < kDigits; ++l) lv[l][0] = lv[l][1] = lv[l][2] = lv[l][3] = 0.f;
#pragma unroll
            for (int ks = 0; ks < kBK / 16; ++ks) {
                uint32_t bf[kDigits][2];
#pragma unroll
                for (int j = 0; j < kDigits; ++j)
                    ldsm_x2(bf[j], &sm.b[j][n0 + (lane & 7)][ks * 16 + ((lane >> 3) & 1) * 8]);
#pragma unroll
                for (int i = 0; i < kDigits; ++i) {
                    uint32_t af[4];
                    ldsm_x4(af, &sm.a[i][m0 + (lane & 15)][ks * 16 + (lane >> 4) * 8]);
#pragma unroll
                    for (int j = 0; j < kDigits - i; ++j) mma_bf16(lv[i + j], af, bf[j]);
                }
            }
            // the exact level sums as two int64 words, hi = levels 0..3 in units
            // of level 3 and lo = levels 4..6 in units of level 6 (|hi| < 2^47.3,
            // |lo| < 2^39.3 per chunk)
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                int L[kDigits];
#pragma unroll
                for (int l = 0; l < kDigits; ++l) L[l] = __float2int_rn(lv[l][q]);
                thi[q] += ((long long)L[0] << 24) + ((long long)L[1] << 16) +
                          ((long long)L[2] << 8) + (long long)L[3];
                tlo[q] += ((long long)L[4] << 16) + ((long long)L[5] << 8) + (long long)L[6];
            }
            __syncthreads();
        }
        // fold into the FP64 accumulators: value = 2^(ea-1022 + eb-1022 - 64) (hi 2^24 + lo)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int rl = m0 + g + ((q >> 1) << 3);
            const int cl = n0 + 2 * t4 + (q & 1);
            const int ea = sm.ea[rl], eb = sm.eb[cl];
            if (ea == 0x7FF || eb == 0x7FF) {
                acc[q] = __longlong_as_double(0x7FF8000000000000LL);
            } else {
                const int fld = ea + eb - 1085;  // exponent field of the scale
                if (fld > 0) {
                    const double s = fld >= 2047 ? __longlong_as_double(0x7FF0000000000000LL)
                                                 : __longlong_as_double((long long)fld << 52);
                    const double v = fma(i64_to_f64(thi[q]), 16777216.0, i64_to_f64(tlo[q]));
                    acc[q] = fma(v, s, acc[q]);
                }
            }
        }
        __syncthreads();
    }

#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int row = mt0 + m0 + g + ((q >> 1) << 3);
        const int col = nt0 + n0 + 2 * t4 + (q & 1);
        if (row >= a.M || col >= a.N) continue;
        const double v = acc[q];
        if constexpr (GRAM) {
            a.out[(size_t)blockIdx.z * a.M * a.N + row + (size_t)col * a.M] = v;
        } else {
            double y = a.alpha * v;
            if (a.beta != nullptr) {
                const double b = a.beta[a.incb == 0 ? 0 : (size_t)col * a.incb];
                if (b != 0.0) y = fma(b, a.out[row + (size_t)col * a.ldo], y);
            }
            a.out[row + (size_t)col * a.ldo] = y;
        }
    }
}

// Split-k partial sums in a fixed order: block b sums outputs
// [32 b, 32 b + 32); thread (o, g) adds chunks g, g + 8, ... of output o
// (consecutive o read consecutive addresses), then the 8 groups are added in
// a fixed tree.
__global__ void __launch_bounds__(256) k_oz_reduce(const double *__restrict__ part, int chunks,
                                                   int m, int w, double *__restrict__ C, int ldc) {
    __shared__ double red[8][33];
    const int total = m * w;
    const int o = threadIdx.x & 31, grp = threadIdx.x >> 5;
    const int e = blockIdx.x * 32 + o;
    double s0 = 0.0, s1 = 0.0;
    if (e < total) {
        int c = grp;
        for (; c + 8 < chunks; c += 16) {
            s0 += part[(size_t)c * total + e];
            s1 += part[(size_t)(c + 8) * total + e];
        }
        if (c < chunks) s0 += part[(size_t)c * total + e];
    }
    red[grp][o] = s0 + s1;
    __syncthreads();
    if (grp == 0 && e < total) {
        const double v = ((red[0][o] + red[1][o]) + (red[2][o] + red[3][o])) +
                         ((red[4][o] + red[5][o]) + (red[6][o] + red[7][o]));
        C[e % m + (size_t)(e / m) * ldc] = v;
    }
}

int oz_num_sms() { return device_sms(); }

template <int BN, bool GRAM>
void launch_oz(const OzArgs &a, dim3 grid, cudaStream_t st) {
    static PerDevice<bool> smem_set;
    const int smem = (int)sizeof(OzSmem<BN>);
    smem_set.get([smem] {
        GCGE_CUDA(cudaFuncSetAttribute(k_oz_gemm<BN, GRAM>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        return true;
    });
    k_oz_gemm<BN, GRAM><<<grid, oz_threads<BN>(), smem, st>>>(a);
    GCGE_CHECK_LAUNCH();
    count_launch();
}

int oz_tile_n(int n) { return n <= 8 ? 8 : (n <= 16 ? 16 : 24); }

// Bytes of the right-operand planes and exponent fields of a linear
// combination with k terms and m columns in tiles of bn columns.
size_t bprep_bytes(int k, int m, int bn) {
    const size_t ntiles = (size_t)(m + bn - 1) / bn;
    const size_t nchunks = (size_t)(k + kBK - 1) / kBK;
    const size_t nsup = (size_t)(k + kSuper * kBK - 1) / (kSuper * kBK);
    return ntiles * nchunks * kDigits * bn * kBKP * sizeof(uint16_t) +
           ntiles * nsup * bn * sizeof(int) + 256;
}

template <int BN>
void prep_b(OzArgs &a, int ntiles, void *scratch, cudaStream_t st) {
    a.nchunks = (a.K + kBK - 1) / kBK;
    a.nsup = (a.K + kSuper * kBK - 1) / (kSuper * kBK);
    uint16_t *planes = static_cast<uint16_t *>(scratch);
    const size_t pl = (size_t)ntiles * a.nchunks * kDigits * BN * kBKP;
    int *exps = reinterpret_cast<int *>(
        (reinterpret_cast<uintptr_t>(planes + pl) + 255) & ~(uintptr_t)255);
    k_oz_bprep<BN><<<dim3(a.nsup, ntiles), oz_threads<BN>(), 0, st>>>(
        a.B, a.ldb, a.N, a.K, planes, exps, a.nchunks, a.nsup);
    GCGE_CHECK_LAUNCH();
    count_launch();
    a.bplanes = planes;
    a.bexps = exps;
}

template <bool GRAM>
void launch_oz_bn(const OzArgs &a, int bn, dim3 grid, cudaStream_t st) {
    switch (bn) {
        case 8: launch_oz<8, GRAM>(a, grid, st); break;
        case 16: launch_oz<16, GRAM>(a, grid, st); break;
        default: launch_oz<24, GRAM>(a, grid, st); break;
    }
}

}  // namespace

// C (m x w, ldc) = Q^T P for Q n x m (ldq), P n x w (ldp); scratch holds the
// split-k partials (scratch_elems doubles).
void oz_gram(int n, int m, int w, const double *Q, int ldq, const double *P, int ldp, double *C,
             int ldc, double *scratch, size_t scratch_elems, cudaStream_t st,
             TcExpCache *cache) {
    if (m <= 0 || w <= 0) return;
    if (tc_digits_available()) {
        tc_gram(n, m, w, Q, ldq, P, ldp, C, ldc, scratch, scratch_elems, st, cache);
        return;
    }
    if (n <= 0) {
        GCGE_CUDA(cudaMemset2DAsync(C, sizeof(double) * ldc, 0, sizeof(double) * m, w, st));
        return;
    }
    const int bn = oz_tile_n(w);
    const int mt = (m + kBM - 1) / kBM, nt = (w + bn - 1) / bn;
    const int chunks = (n + kBK - 1) / kBK;
    // one wave of two CTAs per SM over the whole grid, at least two chunks each
    long long z = std::max(1, (2 * oz_num_sms() + mt * nt - 1) / (mt * nt));
    z = std::min<long long>(z, std::max(1, chunks / 2));
    z = std::min<long long>(z, (long long)(scratch_elems / ((size_t)m * w)));
    GCGE_REQUIRE(z >= 1, GCGE_ERR_ARG, "oz_gram: scratch too small");
    const int per = (int)((chunks + z - 1) / z) * kBK;
    const int zz = (n + per - 1) / per;
    OzArgs a{};
    a.M = m;
    a.N = w;
    a.A = Q;
    a.lda = (size_t)ldq;
    a.B = P;
    a.ldb = (size_t)ldp;
    a.kbeg_stride = per;
    a.K = n;
    a.out = scratch;
    launch_oz_bn<true>(a, bn, dim3(mt, nt, zz), st);
    const int tot = m * w;
    k_oz_reduce<<<(tot + 31) / 32, 256, 0, st>>>(scratch, zz, m, w, C, ldc);
    GCGE_CHECK_LAUNCH();
    count_launch();
}

// Y (n x m, ldy) = alpha X C + Y diag(beta) for X n x k (ldx), C k x m (ldc);
// beta == nullptr overwrites Y; incb == 0 broadcasts beta[0].
size_t oz_lincomb_scratch_bytes(int k, int m) {
    return std::max(bprep_bytes(k, m, oz_tile_n(m)), tc_lincomb_scratch_bytes(k, m));
}

void oz_lincomb(int n, int k, int m, const double *X, int ldx, const double *C, int ldc,
                double *Y, int ldy, const double *beta_dev, int incb, cudaStream_t st,
                double alpha, void *scratch, size_t scratch_bytes, TcExpCache *cache) {
    if (n <= 0 || m <= 0) return;
    if (k <= 0) {
        lincomb(n, k, m, X, ldx, C, ldc, Y, ldy, beta_dev, incb, st, alpha);
        return;
    }
    if (tc_digits_available()) {
        tc_lincomb(n, k, m, X, ldx, C, ldc, Y, ldy, beta_dev, incb, st, alpha, scratch,
                   scratch_bytes, cache);
        return;
    }
    const int bn = oz_tile_n(m);
    OzArgs a{};
    a.M = n;
    a.N = m;
    a.A = X;
    a.lda = (size_t)ldx;
    a.B = C;
    a.ldb = (size_t)ldc;
    a.kbeg_stride = k;
    a.K = k;
    a.out = Y;
    a.ldo = (size_t)ldy;
    a.beta = beta_dev;
    a.incb = incb;
    a.alpha = alpha;
    const int ntiles = (m + bn - 1) / bn;
    GCGE_REQUIRE(scratch && scratch_bytes >= bprep_bytes(k, m, bn), GCGE_ERR_ARG,
                 "oz_lincomb: scratch too small");
    switch (bn) {
        case 8: prep_b<8>(a, ntiles, scratch, st); break;
        case 16: prep_b<16>(a, ntiles, scratch, st); break;
        default: prep_b<24>(a, ntiles, scratch, st); break;
    }
    launch_oz_bn<false>(a, bn, dim3((n + kBM - 1) / kBM, ntiles, 1), st);
}

}  // namespace gcge
