// FP64-accurate tall-skinny products on the 5th-generation tensor cores
// (tcgen05.mma, accumulators in tensor memory), for the mixed-precision GCG:
// the Gram products Q^T P and the linear combinations Y = alpha X C + Y
// diag(beta) that the reference computes with DenseMatQtAP and
// MultiVecLinearComb (app/app_lapack.c:64-183, :463-534).
//
// Method (error-free digit splitting, the Ozaki scheme), as in ozaki.cu:
// within a super-chunk of consecutive k every row of the left operand and
// every column of the right operand gets an exponent e with |x| < 2^e, |x|
// becomes the 56-bit fixed-point integer X = |x| 2^(56-e) (truncated), written
// as 7 digits of 8 bits with x's sign: the leading digit in [0, 256], the
// others balanced in [-128, 127].  Digits are exact in FP16, the 28 digit
// pairs with i + j <= 6 are multiplied on the tensor cores and summed into 7
// level accumulators L_l = sum_{i+j=l} d_i d'_j, which are exact FP32 integers
// as long as |L_l| < 2^24: 96 consecutive k at most (|L_6| <= 96 (2 * 256 *
// 128 + 5 * 128^2) < 2^23.8).  Every 96 k ("drain") the levels are read out of
// tensor memory and folded into two exact int64 words; every super-chunk the
// words are converted to FP64 with the super-chunk's scale and added.  Error:
// below 2^-55 of the super-chunk's largest |x| |y| per product.
//
// Data path, per CTA (one per SM, persistent over work items):
//  * exponent fields come from a streaming pre-pass (k_tc_expcols /
//    k_tc_exprows: per column of the Gram operands over each 384-row
//    super-chunk, per row of the linear combination's left operand over each
//    480-column super-chunk);
//  * one producer thread issues bulk tensor copies (cp.async.bulk.tensor.2d,
//    TMA) of the raw FP64 tiles of each 32-k raw stage, two raw stages ahead,
//    into shared memory (Gram tiles: 16 k x rows boxes with the 128-byte
//    swizzle, so that a lane per row reads them without bank conflicts);
//  * 7 producer warps turn each 16-k half of a raw stage into the 7 FP16
//    digit planes of a digit stage (two digit stages, K-major core-matrix
//    layout: 8 rows x 16 bytes per core matrix); the right operand of a linear
//    combination is prepared once per call (k_tc_bprep) and copied into each
//    digit stage with cp.async.bulk;
//  * one thread of warp 0 issues the 28 MMAs of each digit stage (M = 128 rows,
//    N = BN, K = 16, f16 x f16 -> f32 into 7 level accumulators in tensor
//    memory, 7 x BN of its 512 columns) and commits each stage to an mbarrier;
//  * 12 drain warps read the levels of each 96-k chunk from tensor memory
//    (warp w reads lanes 32 (w % 4) .. + 31), fold them into int64 registers,
//    and at each super-chunk end into FP64 accumulators in shared memory; at
//    the end of a work item they write the result.
// Every wait on an mbarrier is bounded; a wait that runs out sets the error
// word and every role stops at its next wait, so the kernel always returns.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstdint>
#include <mutex>

#include "common.cuh"

namespace gcge {
namespace {

constexpr int kTcDigits = 7;
constexpr int kTcM = 128;      // output rows per tile (tensor-memory lanes)
constexpr int kTcStageK = 16;  // k per digit stage (one MMA step)
constexpr int kTcRawK = 32;    // k per raw (TMA) stage: two digit stages
constexpr int kTcDrainStages = 6;
constexpr int kTcDrainK = kTcStageK * kTcDrainStages;  // 96: exact FP32 level sums
constexpr int kTcKGroups = kTcStageK / 8;              // core matrices along k per stage
constexpr int kTcProdWarps = 7, kTcDrainWarps = 12;
constexpr int kTcWarps = 1 + kTcProdWarps + kTcDrainWarps;
constexpr int kTcThreads = kTcWarps * 32;  // 640
constexpr int kTcProdThreads = kTcProdWarps * 32;
constexpr int kTcDrainThreads = kTcDrainWarps * 32;
constexpr uint32_t kTcTmemCols = 512;
// bounded mbarrier waits: 4 s of device clock, or this many suspended tests
constexpr unsigned long long kTcWaitNs = 4000000000ull;
constexpr long long kTcWaitPolls = 1LL << 22;
// exponent-field slots: the producers fill super-chunk j + 1's while the
// drain folds super-chunk j - 1 with its own
constexpr int kTcExpSlots = 3;
constexpr int kTcSuperGram = 4 * kTcDrainK;     // 384 rows of the Gram operands
constexpr int kTcSuperLincomb = 5 * kTcDrainK;  // 480: K up to 480 in one super-chunk

// Byte layout of one operand tile of R rows in a digit stage: plane i
// (digit), k-group g (8 consecutive k), row r: i * plane + g * lbo +
// (r / 8) * 128 + (r % 8) * 16, with lbo = R * 16 + 16 (the pad keeps the
// producers' 16-byte stores of the k-groups of a row on different banks).
__host__ __device__ constexpr uint32_t tc_lbo(int rows) { return (uint32_t)rows * 16u + 16u; }
__host__ __device__ constexpr uint32_t tc_plane(int rows) { return kTcKGroups * tc_lbo(rows); }
__host__ __device__ constexpr uint32_t tc_tile_bytes(int rows) {
    return kTcDigits * tc_plane(rows);
}
__host__ __device__ constexpr uint32_t tc_round(uint32_t x, uint32_t a) { return (x + a - 1) / a * a; }
// The right operand's 7 digit planes form ONE tile of 7 BN rows (plane j at
// rows [j BN, (j + 1) BN)), so that a single MMA with N = (7 - i) BN
// multiplies left plane i by right planes 0 .. 6 - i and adds each product
// into its level's accumulator columns (level l = i + j at columns l BN):
// k-group g, row r at g * lbo_b + (r / 8) * 128 + (r % 8) * 16.
__host__ __device__ constexpr uint32_t tc_lbo_b(int bn) {
    return (uint32_t)kTcDigits * bn * 16u + 16u;
}
__host__ __device__ constexpr uint32_t tc_tile_b_bytes(int bn) { return kTcKGroups * tc_lbo_b(bn); }

// Shared memory (offsets from a 1024-byte aligned base).  Raw stage of a
// Gram: A boxes [2][128 rows][16 k] and B boxes [2][BN rows][16 k] of FP64 in
// the 128-byte swizzle; of a linear combination: A box [32 k][128 rows] and
// the right operand's prepared digit planes of its two digit stages.  A
// linear combination covers at most one super-chunk per work item (the host
// splits longer contractions), so only the Gram keeps FP64 accumulators.
template <int BN, bool GRAM>
struct TcLayout {
    static constexpr uint32_t a_bytes = tc_tile_bytes(kTcM);
    static constexpr uint32_t b_bytes = tc_tile_b_bytes(BN);
    static constexpr uint32_t a_box = GRAM ? 16u * kTcM * 8u : (uint32_t)kTcRawK * kTcM * 8u;
    static constexpr uint32_t b_box = GRAM ? 16u * BN * 8u : b_bytes;  // lincomb: planes
    // gram: two A boxes and two B boxes; lincomb: one A box and two planes
    static constexpr uint32_t raw_bytes =
        GRAM ? 2 * (a_box + b_box) : tc_round(a_box + 2 * b_box, 1024);
    static constexpr uint32_t raw_off = 0;  // [2] raw stages
    static constexpr uint32_t stage_bytes = a_bytes + b_bytes;
    static constexpr uint32_t dig_off = tc_round(raw_off + 2 * raw_bytes, 1024);  // [2] digit stages
    static constexpr uint32_t acc_off = dig_off + 2 * stage_bytes;  // double acc[BN][kTcM]
    static constexpr uint32_t ea_off = acc_off + (GRAM ? (uint32_t)BN * kTcM * 8 : 0u);  // int ea[3][kTcM]
    static constexpr uint32_t eb_off = ea_off + kTcExpSlots * kTcM * 4;     // int eb[3][BN]
    static constexpr uint32_t bar_off = tc_round(eb_off + kTcExpSlots * BN * 4, 16);
    // full[2] empty[2] rfull[2] accf tfree exfull[3] exfree[3] final
    static constexpr int nbars = 9 + 2 * kTcExpSlots;
    static constexpr uint32_t misc_off = bar_off + nbars * 8;  // tmem slot, abort flag
    static constexpr uint32_t bytes = misc_off + 16;
    static constexpr uint32_t alloc_bytes = bytes + 1024;  // room to align the base
    // what the bulk copies of one raw stage write fits the stage
    static_assert((GRAM ? 2 * (a_box + b_box) : a_box + 2 * b_box) <= raw_bytes,
                  "raw stage too small for its bulk copies");
    static_assert(raw_off + 2 * raw_bytes <= dig_off, "raw stages overlap the digit stages");
    static_assert(alloc_bytes <= 232448, "shared memory beyond the per-CTA limit");
};

struct TcArgs {
    int M, N, K;
    const double *A;  // gram: Q (k, r) at A[k + r lda]; lincomb: X (r, k) at A[r + k lda]
    size_t lda;
    int super_k;      // k per shared exponent (multiple of kTcDrainK)
    int kchunk;       // gram: k per work item (multiple of super_k)
    int items;        // work items
    int mtiles, ntiles;
    double *out;      // gram: partials [kz][M x N]; lincomb: Y (ldo)
    size_t ldo;
    const double *beta;
    int incb;
    double alpha;
    // exponent fields: gram: eA [super][M], eB [super][N]; lincomb: eA
    // [super][M] (rows of X), eB = the prepared right operand's [ntile][super][BN]
    const int *eA, *eB;
    const uint8_t *bplanes;  // lincomb: [ntile][digit stage][b_bytes]
    int nstages, nsup;       // lincomb: digit stages and super-chunks of K
    int accumulate;          // lincomb: add to Y (later blocks of a split contraction)
    int *error;
};

__device__ __forceinline__ uint32_t su32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// ---------------------------------------------------------------- mbarriers
__device__ __forceinline__ void mbar_init(uint64_t *b, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *b) {
    asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(su32(b)) : "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t *b, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(su32(b)), "r"(parity)
        : "memory");
    return done != 0;
}
// The same test, suspending the thread in hardware until the phase completes
// or about `hint_ns` have passed, so that a waiting warp takes no issue slots
// from the warps doing the work.
__device__ __forceinline__ bool mbar_test_suspend(uint64_t *b, uint32_t parity, uint32_t hint_ns) {
    uint32_t done;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2, %3;\n"
        "selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(su32(b)), "r"(parity), "r"(hint_ns)
        : "memory");
    return done != 0;
}
__device__ __forceinline__ unsigned long long tc_global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Waits for the phase of `parity` to complete; false when the wait ran out
// (kTcWaitNs on the device clock, or kTcWaitPolls tests) or another role
// gave up (abort flag set).  All lanes of the calling warp must call it
// together; lane 0 waits and the result is broadcast.
__device__ __forceinline__ bool mbar_wait_warp(uint64_t *b, uint32_t parity,
                                               volatile int *abort_flag, int *gerror) {
    int ok = 1;
    if ((threadIdx.x & 31) == 0 && !mbar_test(b, parity)) {
        const unsigned long long t0 = tc_global_ns();
        long long polls = 0;
        while (!mbar_test_suspend(b, parity, 20000u)) {
            if (*abort_flag) {
                ok = 0;
                break;
            }
            if (++polls > kTcWaitPolls || tc_global_ns() - t0 > kTcWaitNs) {
                *abort_flag = 1;
                atomicExch(gerror, 1);
                ok = 0;
                break;
            }
        }
    }
    ok = __shfl_sync(0xffffffffu, ok, 0);
    // every lane takes the phase's acquire itself (the phase cannot move on
    // without this warp, so the test succeeds at once)
    if (ok) mbar_test(b, parity);
    return ok != 0;
}

// ---------------------------------------------------------------- tcgen05
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    // start address, leading (k-direction) and stride (8-row) byte offsets in
    // 16-byte units, descriptor version 1, no swizzle
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) |
           ((uint64_t)(sbo >> 4) << 32) | (1ull << 46);
}
// kind::f16 instruction descriptor: f32 accumulate (bit 4), f16 A and B
// (format 0 at bits 7 and 10), both K-major, N >> 3 at bit 17, M >> 4 at bit 24
__host__ __device__ constexpr uint32_t tc_idesc(int m, int n) {
    return (1u << 4) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}
__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                       uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void tc_commit(uint64_t *b) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            su32(b))
        : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_ld8(uint32_t taddr, uint32_t (&r)[8]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7])
        : "r"(taddr));
}
__device__ __forceinline__ void tc_wait_ld() {
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// ---------------------------------------------------------------- digits
__device__ __forceinline__ int tc_exp_field(double x) {
    return max((int)(((unsigned)__double2hiint(x) >> 20) & 0x7FFu), 1);
}

// X = |x| 2^(1078 - emax) as a 56-bit fixed-point integer (truncated; the
// caller guarantees emax >= the exponent field of x), plus 0x808080808080,
// as two words: the 53-bit significand shifted left by 3, then right by
// emax - field with clamped funnel shifts (no branches).  sgn = x's sign bit.
__device__ __forceinline__ void tc_fixed56(double x, uint32_t emax, uint32_t &yh, uint32_t &yl,
                                           uint32_t &sgn) {
    const uint32_t hi = (uint32_t)__double2hiint(x), lo = (uint32_t)__double2loint(x);
    const uint32_t ef = (hi >> 20) & 0x7FFu;
    const uint32_t mhi = (hi & 0xFFFFFu) | (min(ef, 1u) << 20);
    uint32_t xh = __funnelshift_l(lo, mhi, 3);
    uint32_t xl = lo << 3;
    const uint32_t r = emax - max(ef, 1u);
    const uint32_t r1 = min(r, 32u), r2 = min(r - r1, 32u);
    xl = __funnelshift_rc(xl, xh, r1);
    xh = __funnelshift_rc(xh, 0u, r1);
    xl = __funnelshift_rc(xl, xh, r2);
    xh = __funnelshift_rc(xh, 0u, r2);
    asm("add.cc.u32 %0, %2, 0x80808080;\n\taddc.u32 %1, %3, 0x8080;"
        : "=r"(yl), "=r"(yh)
        : "r"(xl), "r"(xh));
    sgn = hi & 0x80000000u;
}

// (a - b) on two packed FP16 values
__device__ __forceinline__ uint32_t tc_hsub2(uint32_t a, uint32_t b) {
    uint32_t d;
    asm("sub.rn.f16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
    return d;
}

// The 7 FP16 digits of 8 values (one row, 8 consecutive k) relative to the
// exponent field emax: out[i] holds digit i of the 8 values, two per word
// (lower k in the low half).  With Y = X + 0x808080808080 (tc_fixed56),
// digit 0 is Y >> 48 (in [0, 256]) and digit i >= 1 is byte 6 - i of Y less
// 128 (in [-128, 127]), so that X = sum_i d_i 2^(8 (6 - i)); each carries x's
// sign.  A digit is formed for two values at once: the FP16 pattern
// sign | 0x6400 | field is +-(1024 + field) exactly (ulp 1 on [1024, 2048)),
// and subtracting +-1024 (digit 0) or +-(1024 + 128) leaves +-d exactly.
__device__ __forceinline__ void tc_digits8(const double (&v)[8], int emax, uint4 (&out)[kTcDigits]) {
    uint32_t w[kTcDigits][4];
#pragma unroll
    for (int e = 0; e < 8; e += 2) {
        uint32_t yh0, yl0, s0, yh1, yl1, s1;
        tc_fixed56(v[e], (uint32_t)emax, yh0, yl0, s0);
        tc_fixed56(v[e + 1], (uint32_t)emax, yh1, yl1, s1);
        const uint32_t M = 0x64006400u | (s0 >> 16) | s1;  // +-1024 in each half
        const uint32_t Mb = M | 0x00800080u;                // +-(1024 + 128)
        w[0][e / 2] = tc_hsub2((yh0 >> 16) | (yh1 & 0xFFFF0000u) | M, M);
        // byte 6 - i of Y: bytes 4, 5 in the high word, 0..3 in the low word;
        // the permutation puts value 0's byte in half 0 and value 1's in half 1
        w[1][e / 2] = tc_hsub2((__byte_perm(yh0, yh1, 0x0501) & 0x00FF00FFu) | M, Mb);
        w[2][e / 2] = tc_hsub2((__byte_perm(yh0, yh1, 0x0400) & 0x00FF00FFu) | M, Mb);
        w[3][e / 2] = tc_hsub2((__byte_perm(yl0, yl1, 0x0703) & 0x00FF00FFu) | M, Mb);
        w[4][e / 2] = tc_hsub2((__byte_perm(yl0, yl1, 0x0602) & 0x00FF00FFu) | M, Mb);
        w[5][e / 2] = tc_hsub2((__byte_perm(yl0, yl1, 0x0501) & 0x00FF00FFu) | M, Mb);
        w[6][e / 2] = tc_hsub2((__byte_perm(yl0, yl1, 0x0400) & 0x00FF00FFu) | M, Mb);
    }
#pragma unroll
    for (int i = 0; i < kTcDigits; ++i) out[i] = make_uint4(w[i][0], w[i][1], w[i][2], w[i][3]);
}

// ---------------------------------------------------------------- bulk copies
__device__ __forceinline__ void mbar_expect_tx(uint64_t *b, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(
                     su32(b)),
                 "r"(bytes)
                 : "memory");
}
// contiguous bytes (16-byte aligned, a multiple of 16) into shared memory,
// completing on an mbarrier
__device__ __forceinline__ void bulk_load(uint32_t dst, const void *src, uint32_t bytes,
                                          uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, "
        "[%3];" ::"r"(dst),
        "l"(src), "r"(bytes), "r"(su32(bar))
        : "memory");
}
// 2D tile of a tensor map into shared memory, completing on an mbarrier
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y,
                                            uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(su32(bar))
        : "memory");
}

// exact int64 -> double for |t| < 2^51
__device__ __forceinline__ double tc_i64_to_f64(long long t) {
    return __longlong_as_double(t + 0x4338000000000000LL) - 6755399441055744.0;
}

// Waits, with a bound of its own and regardless of the abort flag, for a
// phase that asynchronous work of this CTA still completes (bulk copies or
// MMAs in flight at teardown).  Lane 0 of the calling warp waits.
__device__ __forceinline__ void mbar_wait_teardown(uint64_t *b, uint32_t parity) {
    if ((threadIdx.x & 31) == 0) {
        const unsigned long long t0 = tc_global_ns();
        while (!mbar_test_suspend(b, parity, 20000u))
            if (tc_global_ns() - t0 > 1000000000ull) break;
    }
    __syncwarp();
}

// ---------------------------------------------------------------- work items
// Work item `it`: gram: (m tile, n tile, k range); lincomb: (m tile = 128
// rows of X and Y, n tile).
struct TcItem {
    int mt0, nt, kb, ke;
};
template <bool GRAM>
__device__ __forceinline__ TcItem tc_item(const TcArgs &a, int it) {
    TcItem w;
    const int mn = a.mtiles * a.ntiles;
    const int z = it / mn, r = it % mn;
    w.mt0 = (r % a.mtiles) * kTcM;
    w.nt = r / a.mtiles;
    if (GRAM) {
        w.kb = z * a.kchunk;
        w.ke = min(a.K, w.kb + a.kchunk);
    } else {
        w.kb = 0;
        w.ke = a.K;
    }
    return w;
}
// A position in this CTA's sequence of raw stages: work item, super-chunk
// start, raw stage start.
struct TcCursor {
    TcItem w;
    int it, sk, k0;
    bool valid;
};
template <bool GRAM>
__device__ __forceinline__ void cur_init(const TcArgs &a, TcCursor &c) {
    c.it = blockIdx.x;
    c.valid = c.it < a.items;
    if (c.valid) {
        c.w = tc_item<GRAM>(a, c.it);
        c.sk = c.k0 = c.w.kb;
    }
}
template <bool GRAM>
__device__ __forceinline__ void cur_next(const TcArgs &a, TcCursor &c) {
    const int ske = min(c.w.ke, c.sk + a.super_k);
    c.k0 += kTcRawK;
    if (c.k0 < ske) return;
    c.sk += a.super_k;
    if (c.sk < c.w.ke) {
        c.k0 = c.sk;
        return;
    }
    c.it += gridDim.x;
    c.valid = c.it < a.items;
    if (c.valid) {
        c.w = tc_item<GRAM>(a, c.it);
        c.sk = c.k0 = c.w.kb;
    }
}

// ---------------------------------------------------------------- kernel
template <int BN, bool GRAM>
__global__ void __launch_bounds__(kTcThreads, 1)
    k_tc_digits(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
                TcArgs a) {
    using L = TcLayout<BN, GRAM>;
    extern __shared__ __align__(1024) uint8_t sm_raw[];
    // 1024-byte aligned base (the 128-byte swizzle of the bulk copies needs it)
    uint8_t *sm = sm_raw + ((1024u - (su32(sm_raw) & 1023u)) & 1023u);
    double *acc = reinterpret_cast<double *>(sm + L::acc_off);  // [BN][kTcM]
    int *ea = reinterpret_cast<int *>(sm + L::ea_off);           // [3][kTcM]
    int *eb = reinterpret_cast<int *>(sm + L::eb_off);           // [3][BN]
    uint64_t *bars = reinterpret_cast<uint64_t *>(sm + L::bar_off);
    uint64_t *full = bars, *empty = bars + 2, *rfull = bars + 4, *accf = bars + 6;
    uint64_t *tfree = bars + 7, *exfull = bars + 8, *exfree = bars + 8 + kTcExpSlots;
    uint64_t *fin = bars + 8 + 2 * kTcExpSlots;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(sm + L::misc_off);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(sm + L::misc_off + 4);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t sbase = su32(sm);

    if (tid == 0) {
        for (int s = 0; s < 2; ++s) {
            mbar_init(&full[s], kTcProdThreads);
            mbar_init(&empty[s], 1);
            mbar_init(&rfull[s], 1);
        }
        for (int s = 0; s < kTcExpSlots; ++s) {
            mbar_init(&exfull[s], kTcProdThreads);
            mbar_init(&exfree[s], kTcDrainThreads);
        }
        mbar_init(accf, 1);
        mbar_init(tfree, kTcDrainThreads);
        mbar_init(fin, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         su32(tmem_slot)),
                     "r"(kTcTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const int super_k = a.super_k;

    if (warp == 0) {
        // ------------------------------------------------------------ MMA issuer
        uint32_t t = 0, d = 0;  // digit stages and drain chunks issued so far
        bool ok = true;
        for (int it = blockIdx.x; it < a.items && ok; it += gridDim.x) {
            const TcItem w = tc_item<GRAM>(a, it);
            for (int k0 = w.kb; k0 < w.ke && ok; k0 += kTcDrainK, ++d) {
                if (d > 0 && !mbar_wait_warp(tfree, (d - 1) & 1, abort_flag, a.error)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                const int nst = min(kTcDrainStages, (w.ke - k0 + kTcStageK - 1) / kTcStageK);
                for (int st = 0; st < nst; ++st, ++t) {
                    const uint32_t s = t & 1;
                    if (!mbar_wait_warp(&full[s], (t >> 1) & 1, abort_flag, a.error)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    if (lane == 0) {
                        const uint32_t abase = sbase + L::dig_off + s * L::stage_bytes;
                        const uint32_t bbase = abase + L::a_bytes;
                        // left plane i times right planes j = 0 .. 6 - i, into
                        // levels l = i + j, in MMAs of at most kLvl levels (N <= 256)
                        constexpr int kLvl = 256 / BN < kTcDigits ? 256 / BN : kTcDigits;
#pragma unroll
                        for (int i = 0; i < kTcDigits; ++i) {
                            const uint64_t ad =
                                smem_desc(abase + i * tc_plane(kTcM), tc_lbo(kTcM), 128);
#pragma unroll
                            for (int l0 = i; l0 < kTcDigits; l0 += kLvl) {
                                const int nl = min(kLvl, kTcDigits - l0);
                                const uint64_t bd = smem_desc(
                                    bbase + (uint32_t)((l0 - i) * BN / 8) * 128u, tc_lbo_b(BN), 128);
                                // the first product into a level in a drain chunk
                                // overwrites it (level l first meets i = 0)
                                tc_mma(tmem + (uint32_t)(l0 * BN), ad, bd, tc_idesc(kTcM, nl * BN),
                                       (st > 0 || i > 0) ? 1u : 0u);
                            }
                        }
                        tc_commit(&empty[s]);
                        if (st == nst - 1) tc_commit(accf);
                    }
                    __syncwarp();
                }
            }
        }
        // all issued MMAs complete before tensor memory is freed
        if (lane == 0) tc_commit(fin);
        __syncwarp();
        mbar_wait_teardown(fin, 0);
    } else if (warp >= 4 && warp < 4 + kTcDrainWarps) {
        // ------------------------------------------------------------ drain
        const int q = warp & 3;             // tensor-memory lane quarter
        const int third = (warp - 4) >> 2;  // column-group share
        const int row = q * 32 + lane;      // output row within the tile
        constexpr int NG = BN / 8;          // 8-column groups
        constexpr int GPT = (NG + 2) / 3;   // groups per drain thread (at most)
        long long thi[GPT * 8], tlo[GPT * 8];
#pragma unroll
        for (int c = 0; c < GPT * 8; ++c) thi[c] = tlo[c] = 0;
        uint32_t d = 0, sc = 0;  // drain chunks and super-chunks consumed so far
        bool ok = true;
        for (int it = blockIdx.x; it < a.items && ok; it += gridDim.x) {
            const TcItem w = tc_item<GRAM>(a, it);
            const int grow = w.mt0 + row;
            if (GRAM)
                for (int c = third; c < NG; c += 3)
                    for (int cc = 0; cc < 8; ++cc) acc[(c * 8 + cc) * kTcM + row] = 0.0;
            for (int sk = w.kb; sk < w.ke && ok; sk += super_k, ++sc) {
                const int ske = min(w.ke, sk + super_k);
                for (int k0 = sk; k0 < ske; k0 += kTcDrainK, ++d) {
                    if (!mbar_wait_warp(accf, d & 1, abort_flag, a.error)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
#pragma unroll
                    for (int l = 0; l < kTcDigits; ++l) {
#pragma unroll
                        for (int gi = 0; gi < GPT; ++gi) {
                            const int g = third + 3 * gi;
                            if (g >= NG) break;
                            uint32_t v[8];
                            tc_ld8(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(l * BN + g * 8),
                                   v);
                            tc_wait_ld();
#pragma unroll
                            for (int cc = 0; cc < 8; ++cc) {
                                const long long L =
                                    (long long)__float2int_rn(__uint_as_float(v[cc]));
                                // hi: levels 0..3 in units of level 3; lo: 4..6 in units of 6
                                if (l <= 3) thi[gi * 8 + cc] += L << (8 * (3 - l));
                                else tlo[gi * 8 + cc] += L << (8 * (6 - l));
                            }
                        }
                    }
                    tc_fence_before();
                    mbar_arrive(tfree);
                }
                if (!ok) break;
                // fold the super-chunk: into the FP64 accumulators (Gram), or
                // straight into Y (a linear combination's single super-chunk)
                const uint32_t b = sc % kTcExpSlots;
                if (!mbar_wait_warp(&exfull[b], (sc / kTcExpSlots) & 1, abort_flag, a.error)) {
                    ok = false;
                    break;
                }
                const int er = ea[b * kTcM + row];
#pragma unroll
                for (int gi = 0; gi < GPT; ++gi) {
                    const int g = third + 3 * gi;
                    if (g >= NG) break;
#pragma unroll
                    for (int cc = 0; cc < 8; ++cc) {
                        const int c = g * 8 + cc;
                        const int ec = eb[b * BN + c];
                        // the super-chunk's sum: v 2^(er + ec - 2108), or NaN
                        const bool nan = er == 0x7FF || ec == 0x7FF;
                        const int fld = er + ec - 1085;  // exponent field of the scale
                        const double sc2 = fld <= 0 ? 0.0
                                           : fld >= 2047
                                               ? __longlong_as_double(0x7FF0000000000000LL)
                                               : __longlong_as_double((long long)fld << 52);
                        const double v = fma(tc_i64_to_f64(thi[gi * 8 + cc]), 16777216.0,
                                             tc_i64_to_f64(tlo[gi * 8 + cc]));
                        thi[gi * 8 + cc] = tlo[gi * 8 + cc] = 0;
                        if (GRAM) {
                            double &A = acc[c * kTcM + row];
                            if (nan) A = __longlong_as_double(0x7FF8000000000000LL);
                            else if (fld > 0) A = fma(v, sc2, A);
                        } else {
                            const double val =
                                nan ? __longlong_as_double(0x7FF8000000000000LL) : v * sc2;
                            const int col = w.nt * BN + c;
                            if (grow < a.M && col < a.N) {
                                double *dst = a.out + grow + (size_t)col * a.ldo;
                                double y = a.alpha * val;
                                if (a.accumulate) {
                                    y += *dst;
                                } else if (a.beta != nullptr) {
                                    const double bb =
                                        a.beta[a.incb == 0 ? 0 : (size_t)col * a.incb];
                                    if (bb != 0.0) y = fma(bb, *dst, y);
                                }
                                *dst = y;
                            }
                        }
                    }
                }
                mbar_arrive(&exfree[b]);
            }
            if (!ok) break;
            // the work item's result (Gram: split-k partials)
            if (GRAM && grow < a.M) {
                const int z = it / (a.mtiles * a.ntiles);
                for (int g = third; g < NG; g += 3) {
                    for (int cc = 0; cc < 8; ++cc) {
                        const int col = w.nt * BN + g * 8 + cc;
                        if (col < a.N)
                            a.out[(size_t)z * a.M * a.N + grow + (size_t)col * a.M] =
                                acc[(g * 8 + cc) * kTcM + row];
                    }
                }
            }
        }
    } else {
        // ------------------------------------------------------------ producers
        const int pw = warp < 4 ? warp - 1 : warp - (4 + kTcDrainWarps) + 3;  // 0..6
        const int p = pw * 32 + lane;                                          // 0..223
        auto prod_sync = [] { asm volatile("bar.sync 1, %0;" ::"n"(kTcProdThreads) : "memory"); };
        // bulk tensor copies of raw stage q (cursor c) into raw buffer q % 2
        auto issue = [&](uint32_t q, const TcCursor &c) {
            const uint32_t r = q & 1;
            const uint32_t base = sbase + L::raw_off + r * L::raw_bytes;
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            if (GRAM) {
                mbar_expect_tx(&rfull[r], 2 * (L::a_box + L::b_box));
                tma_load_2d(base, &mapA, c.k0, c.w.mt0, &rfull[r]);
                tma_load_2d(base + L::a_box, &mapA, c.k0 + 16, c.w.mt0, &rfull[r]);
                tma_load_2d(base + 2 * L::a_box, &mapB, c.k0, c.w.nt * BN, &rfull[r]);
                tma_load_2d(base + 2 * L::a_box + L::b_box, &mapB, c.k0 + 16, c.w.nt * BN,
                            &rfull[r]);
            } else {
                // the A box and the prepared planes of the stage's digit stages
                const int ske = min(c.w.ke, c.sk + super_k);
                const int nd = min(2, (ske - c.k0 + kTcStageK - 1) / kTcStageK);
                mbar_expect_tx(&rfull[r], L::a_box + nd * L::b_box);
                tma_load_2d(base, &mapA, c.w.mt0, c.k0, &rfull[r]);
                const uint8_t *src =
                    a.bplanes +
                    ((size_t)c.w.nt * a.nstages + (c.k0 - c.w.kb) / kTcStageK) * L::b_bytes;
                for (int dd = 0; dd < nd; ++dd)
                    bulk_load(base + L::a_box + dd * L::b_box, src + (size_t)dd * L::b_bytes,
                              L::b_bytes, &rfull[r]);
            }
        };
        // exponent fields of super-chunk (w, sk) into slot b
        auto load_exps = [&](const TcItem &w, int sk, uint32_t b) {
            const int sidx = (sk - (GRAM ? 0 : w.kb)) / super_k;
            for (int r = p; r < kTcM; r += kTcProdThreads) {
                const int gr = w.mt0 + r;
                ea[b * kTcM + r] = gr < a.M ? a.eA[(size_t)sidx * a.M + gr] : 1;
            }
            for (int c = p; c < BN; c += kTcProdThreads) {
                const int gc = w.nt * BN + c;
                if (GRAM) eb[b * BN + c] = gc < a.N ? a.eB[(size_t)sidx * a.N + gc] : 1;
                else eb[b * BN + c] = a.eB[((size_t)w.nt * a.nsup + sidx) * BN + c];
            }
        };

        TcCursor cons, tma;
        cur_init<GRAM>(a, cons);
        tma = cons;
        uint32_t issued = 0;  // raw stages issued
        if (p == 0) {
            for (int i = 0; i < 2 && tma.valid; ++i) {
                issue(issued++, tma);
                cur_next<GRAM>(a, tma);
            }
        }
        // the first super-chunk's exponent fields
        load_exps(cons.w, cons.sk, 0);
        prod_sync();
        mbar_arrive(&exfull[0]);
        uint32_t q = 0, t = 0, j = 0;  // raw stages, digit stages, super-chunks consumed
        bool ok = true;
        while (ok && cons.valid) {
            const int ske = min(cons.w.ke, cons.sk + super_k);
            if (cons.k0 == cons.sk) {
                // at a super-chunk start: the next super-chunk's exponent fields
                TcCursor nx = cons;
                nx.k0 = ske - kTcRawK;  // the super-chunk's last raw stage
                if (nx.k0 < nx.sk) nx.k0 = nx.sk;
                cur_next<GRAM>(a, nx);
                while (nx.valid && nx.k0 != nx.sk) cur_next<GRAM>(a, nx);
                if (nx.valid) {
                    const uint32_t b1 = (j + 1) % kTcExpSlots;
                    // every producer wait is followed by a producer barrier and a
                    // check of the abort flag, so that all producer warps leave
                    // together (none is left waiting at a barrier the others skip)
                    if (j + 1 >= kTcExpSlots)
                        mbar_wait_warp(&exfree[b1], ((j + 1 - kTcExpSlots) / kTcExpSlots) & 1,
                                       abort_flag, a.error);
                    prod_sync();
                    if (*abort_flag) break;
                    load_exps(nx.w, nx.sk, b1);
                    prod_sync();
                    mbar_arrive(&exfull[b1]);
                }
            }
            const uint32_t r = q & 1;
            mbar_wait_warp(&rfull[r], (q >> 1) & 1, abort_flag, a.error);
            const uint8_t *raw = sm + L::raw_off + r * L::raw_bytes;
            const int *ebuf_a = ea + (j % kTcExpSlots) * kTcM;
            const int *ebuf_b = eb + (j % kTcExpSlots) * BN;
            const int nd = min(2, (ske - cons.k0 + kTcStageK - 1) / kTcStageK);
            for (int dd = 0; dd < nd; ++dd, ++t) {
                const uint32_t s = t & 1;
                mbar_wait_warp(&empty[s], ((t >> 1) & 1) ^ 1, abort_flag, a.error);
                prod_sync();
                if (*abort_flag) {
                    ok = false;
                    break;
                }
                uint8_t *abuf = sm + L::dig_off + s * L::stage_bytes;
                uint8_t *bbuf = abuf + L::a_bytes;
                if (!GRAM) {
                    // the right operand's prepared planes of this digit stage, from
                    // the raw stage (the digit stage's full barrier covers them like
                    // the producers' own stores)
                    const uint4 *src =
                        reinterpret_cast<const uint4 *>(raw + L::a_box + dd * L::b_box);
                    uint4 *dst = reinterpret_cast<uint4 *>(bbuf);
                    for (int i = p; i < (int)(L::b_bytes / 16); i += kTcProdThreads)
                        dst[i] = src[i];
                }
                // digit planes of this 16-k half of the raw stage, two items
                // at a time (independent instruction streams)
                constexpr int a_items = kTcM * kTcKGroups;
                constexpr int b_items = GRAM ? BN * kTcKGroups : 0;
                constexpr int n_items = a_items + b_items;
                for (int item0 = p; item0 < n_items; item0 += 2 * kTcProdThreads) {
                    double v[2][8];
                    int em[2] = {1, 1};
                    uint8_t *dstb[2] = {nullptr, nullptr};
                    uint32_t pl[2] = {0, 0};
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const int item = item0 + h * kTcProdThreads;
                        const bool live = item < n_items;
                        const int it2 = live ? item : item0;
                        const bool isb = it2 >= a_items;
                        const int ii = isb ? it2 - a_items : it2;
                        const int rows = isb ? BN : kTcM;
                        const int rr = ii % rows, g = ii / rows;
                        if (GRAM) {
                            // box dd of the operand: rr's 16 k as 8 chunks of 16
                            // bytes, chunk c stored at chunk c ^ (rr % 8)
                            const uint8_t *box = raw + (isb ? 2 * L::a_box + dd * L::b_box
                                                            : dd * L::a_box) +
                                                 (uint32_t)rr * 128u;
#pragma unroll
                            for (int qq = 0; qq < 4; ++qq) {
                                const int c = 4 * g + qq;
                                const double2 u = *reinterpret_cast<const double2 *>(
                                    box + (uint32_t)((c ^ (rr & 7)) << 4));
                                v[h][2 * qq] = u.x;
                                v[h][2 * qq + 1] = u.y;
                            }
                        } else {
                            // box [32 k][128 rows]
                            const double *col = reinterpret_cast<const double *>(raw) +
                                                (size_t)(dd * kTcStageK + g * 8) * kTcM + rr;
#pragma unroll
                            for (int qq = 0; qq < 8; ++qq) v[h][qq] = col[(size_t)qq * kTcM];
                        }
                        em[h] = isb ? ebuf_b[rr] : ebuf_a[rr];
                        if (live) {
                            dstb[h] = (isb ? bbuf : abuf) +
                                      (uint32_t)g * (isb ? tc_lbo_b(BN) : tc_lbo(kTcM)) +
                                      (uint32_t)(rr >> 3) * 128u + (uint32_t)(rr & 7) * 16u;
                            pl[h] = isb ? (uint32_t)BN * 16u : tc_plane(kTcM);
                        }
                    }
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        if (dstb[h] == nullptr) continue;
                        uint4 dg[kTcDigits];
                        tc_digits8(v[h], em[h], dg);
#pragma unroll
                        for (int i = 0; i < kTcDigits; ++i)
                            *reinterpret_cast<uint4 *>(dstb[h] + (uint32_t)i * pl[h]) = dg[i];
                    }
                }
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                mbar_arrive(&full[s]);
            }
            if (!ok) break;
            // raw buffer r is read: refill it with raw stage q + 2
            prod_sync();
            if (*abort_flag) break;
            if (p == 0 && tma.valid) {
                issue(issued++, tma);
                cur_next<GRAM>(a, tma);
            }
            ++q;
            const int sk_before = cons.sk, it_before = cons.it;
            cur_next<GRAM>(a, cons);
            if (cons.valid && (cons.sk != sk_before || cons.it != it_before)) ++j;
        }
        // raw stages still in flight (an abort) land before the CTA exits
        if (pw == 0)
            for (uint32_t qq = q; qq < issued; ++qq)
                mbar_wait_teardown(&rfull[qq & 1], (qq >> 1) & 1);
    }

    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(kTcTmemCols)
                     : "memory");
    }
}

// Exponent fields for the Gram operands: out[s * ncols + c] = the largest
// exponent field (at least 1) of column c of X (n x ncols, leading dimension
// ld, 16-byte aligned columns) over rows [s super, (s + 1) super).  One warp
// per (super-chunk, column), 16-byte loads.
__global__ void __launch_bounds__(256) k_tc_expcols(const double *__restrict__ X, size_t ld,
                                                    int n, int ncols, int super, int nsup,
                                                    int *__restrict__ out) {
    const int lane = threadIdx.x & 31;
    const long long nw = (long long)gridDim.x * 8;
    for (long long wid = (long long)blockIdx.x * 8 + (threadIdx.x >> 5);
         wid < (long long)nsup * ncols; wid += nw) {
        const int c = (int)(wid / nsup), s = (int)(wid % nsup);
        const int r0 = s * super, r1 = min(n, r0 + super);
        const double *col = X + (size_t)c * ld;
        int em = 1;
        for (int r = r0 + 2 * lane; r < r1; r += 64) {
            if (r + 1 < r1) {
                const double2 u = __ldg(reinterpret_cast<const double2 *>(col + r));
                em = max(em, max(tc_exp_field(u.x), tc_exp_field(u.y)));
            } else {
                em = max(em, tc_exp_field(__ldg(col + r)));
            }
        }
        em = (int)__reduce_max_sync(0xffffffffu, (unsigned)em);
        if (lane == 0) out[(size_t)s * ncols + c] = em;
    }
}

// Exponent fields for the left operand of a linear combination:
// out[s * n + r] = the largest exponent field (at least 1) of row r of X
// (n x K, leading dimension ld) over columns [s super, (s + 1) super).
__global__ void __launch_bounds__(256) k_tc_exprows(const double *__restrict__ X, size_t ld,
                                                    int n, int K, int super,
                                                    int *__restrict__ out) {
    const int r = blockIdx.x * 256 + threadIdx.x, s = blockIdx.y;
    if (r >= n) return;
    const int k0 = s * super, k1 = min(K, k0 + super);
    int em = 1;
    int k = k0;
    for (; k + 8 <= k1; k += 8) {
        double v[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) v[q] = __ldg(X + r + (size_t)(k + q) * ld);
#pragma unroll
        for (int q = 0; q < 8; ++q) em = max(em, tc_exp_field(v[q]));
    }
    for (; k < k1; ++k) em = max(em, tc_exp_field(__ldg(X + r + (size_t)k * ld)));
    out[(size_t)s * n + r] = em;
}

// Right operand of a linear combination (C, K x N, element (k, c) at
// C[k + c ldc]) prepared once per call: block (super-chunk, n tile) writes the
// exponent fields of its BN columns and the digit planes of each 16-k digit
// stage of the super-chunk in the stage layout of the product kernel.
template <int BN>
__global__ void __launch_bounds__(256) k_tc_bprep(const double *__restrict__ C, size_t ldc, int N,
                                                  int K, int super_k, uint8_t *__restrict__ planes,
                                                  int *__restrict__ exps, int nstages, int nsup) {
    constexpr uint32_t bb = tc_tile_b_bytes(BN);
    __shared__ int em_s[BN];
    const int sidx = blockIdx.x, nt = blockIdx.y;
    const int sk = sidx * super_k, ske = min(K, sk + super_k);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int c = warp; c < BN; c += 8) {
        const int gc = nt * BN + c;
        int em = 1;
        if (gc < N)
            for (int k = sk + lane; k < ske; k += 32) em = max(em, tc_exp_field(C[k + (size_t)gc * ldc]));
        em = (int)__reduce_max_sync(0xffffffffu, (unsigned)em);
        if (lane == 0) {
            em_s[c] = em;
            exps[((size_t)nt * nsup + sidx) * BN + c] = em;
        }
    }
    __syncthreads();
    for (int k0 = sk; k0 < ske; k0 += kTcStageK) {
        uint8_t *dst = planes + ((size_t)nt * nstages + k0 / kTcStageK) * bb;
        for (int item = threadIdx.x; item < BN * kTcKGroups; item += 256) {
            const int c = item % BN, g = item / BN;
            const int gc = nt * BN + c, k = k0 + g * 8;
            double v[8];
#pragma unroll
            for (int q = 0; q < 8; ++q)
                v[q] = (gc < N && k + q < ske) ? C[k + q + (size_t)gc * ldc] : 0.0;
            uint4 dg[kTcDigits];
            tc_digits8(v, em_s[c], dg);
            uint8_t *base = dst + (uint32_t)g * tc_lbo_b(BN) + (uint32_t)(c >> 3) * 128u +
                            (uint32_t)(c & 7) * 16u;
#pragma unroll
            for (int i = 0; i < kTcDigits; ++i)
                *reinterpret_cast<uint4 *>(base + (uint32_t)i * BN * 16u) = dg[i];
        }
    }
}

// Split-k partial sums in a fixed order: block b sums outputs
// [32 b, 32 b + 32); thread (o, grp) adds partials grp, grp + 8, ... of output
// o, then the 8 groups are added in a fixed tree.
__global__ void __launch_bounds__(256) k_tc_reduce(const double *__restrict__ part, int chunks,
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

int tc_bn(int n) { return n <= 16 ? 16 : (n <= 32 ? 32 : 48); }

template <int BN, bool GRAM>
void launch_tc(const CUtensorMap &ma, const CUtensorMap &mb, const TcArgs &a, int grid,
               cudaStream_t st) {
    using L = TcLayout<BN, GRAM>;
    static PerDevice<bool> smem_set;
    smem_set.get([] {
        GCGE_CUDA(cudaFuncSetAttribute(k_tc_digits<BN, GRAM>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)L::alloc_bytes));
        return true;
    });
    k_tc_digits<BN, GRAM><<<grid, kTcThreads, L::alloc_bytes, st>>>(ma, mb, a);
    GCGE_CHECK_LAUNCH();
    count_launch();
}

template <bool GRAM>
void launch_tc_bn(const CUtensorMap &ma, const CUtensorMap &mb, const TcArgs &a, int bn, int grid,
                  cudaStream_t st) {
    switch (bn) {
        case 16: launch_tc<16, GRAM>(ma, mb, a, grid, st); break;
        case 32: launch_tc<32, GRAM>(ma, mb, a, grid, st); break;
        default: launch_tc<48, GRAM>(ma, mb, a, grid, st); break;
    }
}

// Device error word of the product kernels (a wait that ran out), one per
// device; read and cleared by tc_check_error.
int *tc_error_word() {
    static PerDevice<int *> word;
    return word.get([] {
        int *p = nullptr;
        GCGE_CUDA(cudaMalloc((void **)&p, sizeof(int)));
        GCGE_CUDA(cudaMemset(p, 0, sizeof(int)));
        return p;
    });
}

// cuTensorMapEncodeTiled from the driver (the library links the static
// runtime, not the driver library)
PFN_cuTensorMapEncodeTiled_v12000 tc_encode_fn() {
    static std::once_flag once;
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                             cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        else
            cudaGetLastError();
    });
    return fn;
}

// 2D FP64 tensor map of a column-major block: dim0 (contiguous) x dim1 with
// row pitch ld doubles, box0 x box1 elements; false where the layout cannot
// be described (the caller then uses the FP64 kernels).
bool tc_map(CUtensorMap *map, const double *base, int dim0, int dim1, size_t ld, int box0,
            int box1, bool swizzle) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = tc_encode_fn();
    if (!enc || (reinterpret_cast<uintptr_t>(base) & 15) || (ld * 8) % 16 || dim0 < 1 || dim1 < 1)
        return false;
    const cuuint64_t dims[2] = {(cuuint64_t)dim0, (cuuint64_t)dim1};
    const cuuint64_t strides[1] = {(cuuint64_t)ld * 8};
    const cuuint32_t box[2] = {(cuuint32_t)box0, (cuuint32_t)box1};
    const cuuint32_t estr[2] = {1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, const_cast<double *>(base), dims, strides,
               box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
               swizzle ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
               CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

size_t tc_bprep_bytes(int k, int m) {
    const int bn = tc_bn(m);
    const size_t nt = (size_t)(m + bn - 1) / bn;
    const size_t nst = (size_t)(k + kTcStageK - 1) / kTcStageK;
    const size_t nsup = (size_t)(k + kTcSuperLincomb - 1) / kTcSuperLincomb;
    const size_t bb = tc_tile_b_bytes(bn);
    return nt * nst * bb + 256 + nt * nsup * bn * sizeof(int) + 256;
}

}  // namespace

bool tc_digits_available() {
    static PerDevice<int> ok;
    return ok.get([] {
        int major = 0, minor = 0;
        const int dev = current_device();
        cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
        cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
        return (major == 10 && minor == 3 && tc_encode_fn() != nullptr) ? 1 : 0;
    }) != 0;
}

void tc_check_error(cudaStream_t st) {
    int *w = tc_error_word();
    int h = 0;
    GCGE_CUDA(cudaMemcpyAsync(&h, w, sizeof(int), cudaMemcpyDeviceToHost, st));
    GCGE_CUDA(cudaStreamSynchronize(st));
    if (h != 0) {
        GCGE_CUDA(cudaMemsetAsync(w, 0, sizeof(int), st));
        GCGE_CUDA(cudaStreamSynchronize(st));
        throw CudaError{GCGE_ERR_CUDA, "tensor-core digit product: an mbarrier wait timed out"};
    }
}

// C (m x w, ldc) = Q^T P for Q n x m (ldq), P n x w (ldp): split-k partials
// in scratch (scratch_elems doubles), then a fixed-order sum.  Operands that a
// tensor map cannot describe (an odd leading dimension, a base not 16-byte
// aligned) go through the FP64 kernel.
void tc_gram(int n, int m, int w, const double *Q, int ldq, const double *P, int ldp, double *C,
             int ldc, double *scratch, size_t scratch_elems, cudaStream_t st) {
    if (m <= 0 || w <= 0) return;
    if (n <= 0) {
        GCGE_CUDA(cudaMemset2DAsync(C, sizeof(double) * ldc, 0, sizeof(double) * m, w, st));
        return;
    }
    const int bn = tc_bn(w);
    CUtensorMap ma, mb;
    if (!tc_map(&ma, Q, n, m, (size_t)ldq, 16, kTcM, true) ||
        !tc_map(&mb, P, n, w, (size_t)ldp, 16, bn, true)) {
        gram(n, m, w, Q, ldq, P, ldp, C, ldc, scratch, scratch_elems, st);
        return;
    }
    TcArgs a{};
    a.M = m;
    a.N = w;
    a.K = n;
    a.A = Q;
    a.lda = (size_t)ldq;
    a.super_k = kTcSuperGram;
    a.mtiles = (m + kTcM - 1) / kTcM;
    a.ntiles = (w + bn - 1) / bn;
    const int mn = a.mtiles * a.ntiles;
    const int sms = device_sms();
    // exponent fields of both operands per 384-row super-chunk
    const int nsup = (n + kTcSuperGram - 1) / kTcSuperGram;
    DevBuf<int> &eb = slot_stage().tc_exps;
    eb.alloc((size_t)nsup * (m + w));
    int *eA = eb.p, *eB = eb.p + (size_t)nsup * m;
    const int gx = std::min<long long>(4 * sms, ((long long)nsup * std::max(m, w) + 7) / 8);
    k_tc_expcols<<<gx, 256, 0, st>>>(Q, (size_t)ldq, n, m, kTcSuperGram, nsup, eA);
    k_tc_expcols<<<gx, 256, 0, st>>>(P, (size_t)ldp, n, w, kTcSuperGram, nsup, eB);
    GCGE_CHECK_LAUNCH();
    count_launch(2);
    a.eA = eA;
    a.eB = eB;
    // one wave of one CTA per SM over all work items
    int z = std::max(1, sms / mn);
    long long kc = ((long long)(n + z - 1) / z + kTcSuperGram - 1) / kTcSuperGram * kTcSuperGram;
    GCGE_REQUIRE((size_t)m * w <= scratch_elems, GCGE_ERR_ARG, "tc_gram: scratch too small");
    // fewer, longer k ranges until the partials fit the scratch
    while ((size_t)((n + kc - 1) / kc) * m * w > scratch_elems) kc *= 2;
    z = (int)((n + kc - 1) / kc);
    a.kchunk = (int)kc;
    a.items = z * mn;
    a.out = scratch;
    a.error = tc_error_word();
    launch_tc_bn<true>(ma, mb, a, bn, std::min(a.items, sms), st);
    const int tot = m * w;
    k_tc_reduce<<<(tot + 31) / 32, 256, 0, st>>>(scratch, z, m, w, C, ldc);
    GCGE_CHECK_LAUNCH();
    count_launch();
}

size_t tc_lincomb_scratch_bytes(int k, int m) {
    return tc_bprep_bytes(std::min(k, kTcSuperLincomb), m);
}

// Y (n x m, ldy) = alpha X C + Y diag(beta) for X n x k (ldx), C k x m (ldc);
// beta == nullptr overwrites Y; incb == 0 broadcasts beta[0].  Contractions
// longer than one super-chunk (480) run as several launches, each later one
// adding its block's product to Y.
void tc_lincomb(int n, int k, int m, const double *X, int ldx, const double *C, int ldc, double *Y,
                int ldy, const double *beta_dev, int incb, cudaStream_t st, double alpha,
                void *scratch, size_t scratch_bytes) {
    if (n <= 0 || m <= 0) return;
    const int bn = tc_bn(m);
    CUtensorMap ma;
    if (!tc_map(&ma, X, n, std::min(k, kTcSuperLincomb), (size_t)ldx, kTcM, kTcRawK, false)) {
        lincomb(n, k, m, X, ldx, C, ldc, Y, ldy, beta_dev, incb, st, alpha);
        return;
    }
    GCGE_REQUIRE(scratch && scratch_bytes >= tc_lincomb_scratch_bytes(k, m), GCGE_ERR_ARG,
                 "tc_lincomb: scratch too small");
    for (int k0 = 0; k0 < k; k0 += kTcSuperLincomb) {
        const int kb = std::min(kTcSuperLincomb, k - k0);
        const double *Xb = X + (size_t)k0 * ldx;
        // (the first block's map was made above; Xb keeps its 16-byte alignment)
        if (k0 > 0 && !tc_map(&ma, Xb, n, kb, (size_t)ldx, kTcM, kTcRawK, false))
            throw CudaError{GCGE_ERR_ARG, "tc_lincomb: operand layout"};
        TcArgs a{};
        a.M = n;
        a.N = m;
        a.K = kb;
        a.A = Xb;
        a.lda = (size_t)ldx;
        a.super_k = kTcSuperLincomb;
        a.mtiles = (n + kTcM - 1) / kTcM;
        a.ntiles = (m + bn - 1) / bn;
        a.items = a.mtiles * a.ntiles;
        a.out = Y;
        a.ldo = (size_t)ldy;
        a.beta = beta_dev;
        a.incb = incb;
        a.alpha = alpha;
        a.accumulate = k0 > 0 ? 1 : 0;
        a.nstages = (kb + kTcStageK - 1) / kTcStageK;
        a.nsup = 1;
        a.error = tc_error_word();
        uint8_t *planes = static_cast<uint8_t *>(scratch);
        const size_t pbytes = (size_t)a.ntiles * a.nstages * tc_tile_b_bytes(bn);
        int *bexps = reinterpret_cast<int *>(
            (reinterpret_cast<uintptr_t>(planes + pbytes) + 255) & ~(uintptr_t)255);
        const dim3 pg(1, a.ntiles);
        const double *Cb = C + k0;
        switch (bn) {
            case 16: k_tc_bprep<16><<<pg, 256, 0, st>>>(Cb, (size_t)ldc, m, kb, kTcSuperLincomb, planes, bexps, a.nstages, 1); break;
            case 32: k_tc_bprep<32><<<pg, 256, 0, st>>>(Cb, (size_t)ldc, m, kb, kTcSuperLincomb, planes, bexps, a.nstages, 1); break;
            default: k_tc_bprep<48><<<pg, 256, 0, st>>>(Cb, (size_t)ldc, m, kb, kTcSuperLincomb, planes, bexps, a.nstages, 1); break;
        }
        // exponent fields of the rows of X over the block's columns
        DevBuf<int> &eb = slot_stage().tc_exps;
        eb.alloc((size_t)n);
        k_tc_exprows<<<dim3((n + 255) / 256, 1), 256, 0, st>>>(Xb, (size_t)ldx, n, kb,
                                                             kTcSuperLincomb, eb.p);
        GCGE_CHECK_LAUNCH();
        count_launch(2);
        a.bplanes = planes;
        a.eA = eb.p;
        a.eB = bexps;
        launch_tc_bn<false>(ma, ma, a, bn, std::min(a.items, device_sms()), st);
    }
}

}  // namespace gcge
