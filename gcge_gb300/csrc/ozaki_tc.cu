// FP64-accurate tall-skinny products on the 5th-generation tensor cores
// (tcgen05.mma, accumulators in tensor memory), for the mixed-precision GCG:
// the Gram products Q^T P and the linear combinations Y = alpha X C + Y
// diag(beta) that the reference computes with DenseMatQtAP and
// MultiVecLinearComb (app/app_lapack.c:64-183, :463-534).
//
// Method (error-free digit splitting, the Ozaki scheme), as in ozaki.cu:
// within an exponent window of consecutive k every row of the left operand
// and every column of the right operand gets an exponent e with |x| < 2^e,
// |x| becomes the 55-bit fixed-point integer X = |x| 2^(55-e) (truncated),
// written as 7 digits of 8 bits with x's sign: the leading digit in [0, 128],
// the others balanced in [-128, 127].  Digits are exact in FP16, the 28 digit
// pairs with i + j <= 6 are multiplied on the tensor cores and summed into 7
// level accumulators L_l = sum_{i+j=l} d_i d'_j, which are exact FP32 integers
// as long as |L_l| < 2^24: 144 consecutive k at most (|L_6| <= 144 * 7 * 128^2
// < 2^23.98).  Every 144 k ("drain") the levels are read out of tensor memory
// into one exact 96-bit integer per output; at the end of a window it is
// converted to FP64 (integer instructions, round to nearest) with the window's
// scale.  A Gram work item has one window over its whole k range (error below
// 2^-53 sqrt(K) |x| |y| per entry, under the FP64 dot product's bound
// K 2^-53 |x| |y|); a linear combination has one per 432 k.
//
// Data path, per CTA (one per SM, persistent over work items, 16 warps):
//  * exponent fields come from a streaming pre-pass (k_tc_expcols /
//    k_tc_exprows: per column of the Gram operands over each window, per row
//    of the linear combination's left operand);
//  * bulk tensor copies (cp.async.bulk.tensor.2d, TMA) bring the raw FP64
//    tiles of each 32-k raw stage into shared memory two raw stages ahead
//    (Gram tiles: 16 k x rows boxes with the 128-byte swizzle, so that lanes
//    reading rows hit distinct banks); the right operand of a linear
//    combination is prepared once per call (k_tc_bprep) and copied in with
//    cp.async.bulk;
//  * 16 worker warps turn their core matrices (8 rows x 8 k) of each 16-k
//    half of a raw stage into the 7 FP16 digit planes of a digit stage (a
//    ring of two digit stages, K-major core-matrix layout); the last worker
//    to finish reading a raw stage issues the bulk copies of the raw stage
//    two ahead;
//  * one warp issues the MMAs of each digit stage (M = 128 rows, N = up to
//    256, K = 16, f16 x f16 -> f32 into the 7 level accumulators, 7 x BN of
//    the 512 tensor-memory columns) and commits them to mbarriers;
//  * every worker drains its slice of the levels after each 144-k chunk (warp
//    w reads lanes 32 (w % 4) .. + 31, BN / 4 columns) and folds it at the
//    end of each window (a Gram work item longer than one window adds its
//    windows into its split-k partial).
// Every wait on an mbarrier is bounded; a wait that runs out sets the error
// word and every warp stops at its next wait, so the kernel always returns.
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
constexpr int kTcDrainStages = 9;
constexpr int kTcDrainK = kTcStageK * kTcDrainStages;  // 144: exact FP32 level sums
constexpr int kTcKGroups = kTcStageK / 8;              // core matrices along k per stage
constexpr int kTcDigStages = 2;                         // ring of digit stages
constexpr int kTcWarps = 16;  // worker warps: digit conversion and drain
constexpr int kTcThreads = (kTcWarps + 1) * 32;  // and one warp issuing the MMAs
constexpr uint32_t kTcTmemCols = 512;
// bounded mbarrier waits: 4 s of device clock, or this many suspended tests
constexpr unsigned long long kTcWaitNs = 4000000000ull;
constexpr long long kTcWaitPolls = 1LL << 22;
// A Gram work item shares one exponent per column over its whole k range
// (at most this many rows: the 96-bit level sums stay below 2^86)
constexpr int kTcSuperGramMax = 16384 * kTcDrainK;
constexpr int kTcSuperLincomb = 3 * kTcDrainK;  // 432: K up to 432 in one window

// Byte layout of one operand tile of R rows in a digit stage: plane i
// (digit), k-group g (8 consecutive k), row r: i * plane + g * lbo +
// (r / 8) * 128 + (r % 8) * 16, with lbo = R * 16 + 16 (the pad keeps the
// 16-byte core-matrix rows of different k-groups on different banks).
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
// the right operand's prepared digit planes of its two digit stages.  The
// digit stages form a ring of kTcDigStages.
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
    static constexpr uint32_t dig_off = tc_round(raw_off + 2 * raw_bytes, 1024);
    static constexpr uint32_t bar_off = tc_round(dig_off + kTcDigStages * stage_bytes, 16);
    // mbarriers empty[3] full[3] rfull[2] accf fin
    static constexpr int nbars = 2 * kTcDigStages + 4;
    // tmem slot, abort flag, arrival counters rempty[2], raw stages issued
    static constexpr uint32_t misc_off = bar_off + nbars * 8;
    static constexpr uint32_t bytes = misc_off + 48;
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
    int super_k;      // k per exponent window (multiple of kTcDrainK)
    int kchunk;       // gram: k per work item (multiple of super_k)
    int items;        // work items
    int mtiles, ntiles;
    double *out;      // gram: partials [kz][M x N]; lincomb: Y (ldo)
    size_t ldo;
    const double *beta;
    int incb;
    double alpha;
    // exponent fields: gram: eA [window][M], eB [window][N]; lincomb: eA
    // [window][M] (rows of X), eB = the prepared right operand's [ntile][window][BN]
    const int *eA, *eB;
    const uint8_t *bplanes;  // lincomb: [ntile][digit stage][b_bytes]
    int nstages, nsup;       // lincomb: digit stages and exponent windows of K
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

// Arrival on a shared-memory counter (release and acquire at CTA scope);
// returns the count before it.
__device__ __forceinline__ uint32_t smem_arrive(uint32_t *ctr) {
    uint32_t old;
    asm volatile("atom.acq_rel.cta.shared::cta.add.u32 %0, [%1], 1;"
                 : "=r"(old)
                 : "r"(su32(ctr))
                 : "memory");
    return old;
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
__device__ __forceinline__ void tc_ld4(uint32_t taddr, uint32_t (&r)[4]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(taddr));
}
__device__ __forceinline__ void tc_wait_ld() {
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// ---------------------------------------------------------------- digits
__device__ __forceinline__ int tc_exp_field(double x) {
    return max((int)(((unsigned)__double2hiint(x) >> 20) & 0x7FFu), 1);
}

// X = |x| 2^(1077 - emax) as a 55-bit fixed-point integer (truncated; the
// caller guarantees emax >= the exponent field of x), plus 0x808080808080,
// as two words: the 53-bit significand shifted left by 2, then right by
// r = emax - field (at most 63: everything past 55 bits is gone), a 64-bit
// shift made of one wrapping and one clamping funnel shift.  hi = x's high
// word (its sign bit is the sign).
__device__ __forceinline__ void tc_fixed55(double x, uint32_t emax, uint32_t &yh, uint32_t &yl,
                                           uint32_t &hi) {
    hi = (uint32_t)__double2hiint(x);
    const uint32_t lo = (uint32_t)__double2loint(x);
    const uint32_t eb = hi & 0x7FF00000u;  // exponent field << 20
    // the hidden bit, absent for zeros and subnormals (which count as field 1)
    const uint32_t mhi = (hi & 0x000FFFFFu) | min(eb, 0x00100000u);
    const uint32_t xh = __funnelshift_l(lo, mhi, 2);
    const uint32_t xl = lo << 2;
    const uint32_t r = min(emax - (max(eb, 0x00100000u) >> 20), 63u);
    const bool big = r >= 32u;
    const uint32_t sl = __funnelshift_r(big ? xh : xl, big ? 0u : xh, r);  // shift r mod 32
    const uint32_t sh = __funnelshift_rc(xh, 0u, r);                       // 0 for r >= 32
    asm("add.cc.u32 %0, %2, 0x80808080;\n\taddc.u32 %1, %3, 0x8080;"
        : "=r"(yl), "=r"(yh)
        : "r"(sl), "r"(sh));
}

// (a - b) on two packed FP16 values
__device__ __forceinline__ uint32_t tc_hsub2(uint32_t a, uint32_t b) {
    uint32_t d;
    asm("sub.rn.f16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
    return d;
}

// The 7 FP16 digits of 8 values (one row, 8 consecutive k) relative to the
// exponent field emax: out[i] holds digit i of the 8 values, two per word
// (lower k in the low half).  With Y = X + 0x808080808080 (tc_fixed55),
// digit 0 is Y >> 48 (in [0, 128]) and digit i >= 1 is byte 6 - i of Y less
// 128 (in [-128, 127]), so that X = sum_i d_i 2^(8 (6 - i)); each carries x's
// sign.  A digit is formed for two values at once: the FP16 pattern
// sign | 0x6400 | field is +-(1024 + field) exactly (ulp 1 on [1024, 2048)),
// and subtracting +-1024 (digit 0) or +-(1024 + 128) leaves +-d exactly.
__device__ __forceinline__ void tc_digit_pair(double x0, double x1, uint32_t emax,
                                              uint32_t (&w)[kTcDigits]) {
    uint32_t yh0, yl0, h0, yh1, yl1, h1;
    tc_fixed55(x0, emax, yh0, yl0, h0);
    tc_fixed55(x1, emax, yh1, yl1, h1);
    // +-1024 in each half: the sign bits of the two values at bits 15 and 31
    const uint32_t M = (__byte_perm(h0, h1, 0x7030) & 0x80008000u) | 0x64006400u;
    const uint32_t Mb = M | 0x00800080u;                // +-(1024 + 128)
    w[0] = tc_hsub2((yh0 >> 16) | (yh1 & 0xFFFF0000u) | M, M);
    // byte 6 - i of Y: bytes 4, 5 in the high word, 0..3 in the low word; the
    // permutation puts value 0's byte in half 0 and value 1's in half 1
    w[1] = tc_hsub2((__byte_perm(yh0, yh1, 0x0501) & 0x00FF00FFu) | M, Mb);
    w[2] = tc_hsub2((__byte_perm(yh0, yh1, 0x0400) & 0x00FF00FFu) | M, Mb);
    w[3] = tc_hsub2((__byte_perm(yl0, yl1, 0x0703) & 0x00FF00FFu) | M, Mb);
    w[4] = tc_hsub2((__byte_perm(yl0, yl1, 0x0602) & 0x00FF00FFu) | M, Mb);
    w[5] = tc_hsub2((__byte_perm(yl0, yl1, 0x0501) & 0x00FF00FFu) | M, Mb);
    w[6] = tc_hsub2((__byte_perm(yl0, yl1, 0x0400) & 0x00FF00FFu) | M, Mb);
}
__device__ __forceinline__ void tc_digits8(const double (&v)[8], int emax, uint4 (&out)[kTcDigits]) {
    uint32_t w[4][kTcDigits];
#pragma unroll
    for (int e = 0; e < 4; ++e) tc_digit_pair(v[2 * e], v[2 * e + 1], (uint32_t)emax, w[e]);
#pragma unroll
    for (int i = 0; i < kTcDigits; ++i) out[i] = make_uint4(w[0][i], w[1][i], w[2][i], w[3][i]);
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


// (vh 2^64 + vl) 2^e as a double, rounded to nearest (ties to even), with
// integer instructions only (FP64 arithmetic is a slow pipe on this part).
// Results below the normal range flush to zero; above it they are +-inf.
__device__ __forceinline__ double tc_i128_f64(long long vh, unsigned long long vl, int e) {
    // vh 2^64 + vl, a two's-complement 128-bit integer
    const bool neg = vh < 0;
    if (neg) {
        vl = ~vl + 1ull;
        vh = ~vh + (vl == 0 ? 1 : 0);
    }
    const unsigned long long mh = (unsigned long long)vh;  // magnitude mh 2^64 + vl
    if ((mh | vl) == 0) return 0.0;
    // the leading 64 bits th (top bit set) and the rest tl
    int lz;
    unsigned long long th, tl;
    if (mh != 0) {
        lz = __clzll((long long)mh);
        th = lz ? (mh << lz) | (vl >> (64 - lz)) : mh;
        tl = vl << lz;
    } else {
        lz = 64 + __clzll((long long)vl);
        th = vl << (lz - 64);
        tl = 0;
    }
    // 53 bits kept, 11 rounded, tl sticky; the magnitude is mant 2^(75 - lz)
    const unsigned long long mant = th >> 11, rb = th & 0x7FFull;
    const bool up = rb > 0x400ull || (rb == 0x400ull && (tl != 0 || (mant & 1ull)));
    const int field = 1023 + 127 - lz + e;
    unsigned long long bits;
    if (field <= 0) {
        bits = 0;
    } else if (field >= 2047) {
        bits = 0x7FF0000000000000ull;
    } else {
        // mant holds the hidden bit, so it adds one to field - 1; a carry of
        // the rounding moves into the exponent
        bits = ((unsigned long long)(field - 1) << 52) + mant + (up ? 1ull : 0ull);
        if (bits > 0x7FF0000000000000ull) bits = 0x7FF0000000000000ull;
    }
    return __longlong_as_double((long long)(bits | (neg ? 0x8000000000000000ull : 0ull)));
}
// A 96-bit two's-complement accumulator (w0 least significant): += (a0, a1, a2)
__device__ __forceinline__ void tc_acc96(uint32_t &w0, uint32_t &w1, uint32_t &w2, uint32_t a0,
                                         uint32_t a1, uint32_t a2) {
    asm("add.cc.u32 %0, %0, %3;\n\taddc.cc.u32 %1, %1, %4;\n\taddc.u32 %2, %2, %5;"
        : "+r"(w0), "+r"(w1), "+r"(w2)
        : "r"(a0), "r"(a1), "r"(a2));
}
__device__ __forceinline__ void tc_acc64(uint32_t &w1, uint32_t &w2, uint32_t a1, uint32_t a2) {
    asm("add.cc.u32 %0, %0, %2;\n\taddc.u32 %1, %1, %3;" : "+r"(w1), "+r"(w2) : "r"(a1), "r"(a2));
}
// += v 2^(8 (6 - l)) for a level sum v (|v| < 2^31)
__device__ __forceinline__ void tc_acc_level(uint32_t &w0, uint32_t &w1, uint32_t &w2, int v, int l) {
    const uint32_t sx = (uint32_t)(v >> 31);
    const int sh = 8 * (6 - l);
    if (sh == 0) tc_acc96(w0, w1, w2, (uint32_t)v, sx, sx);
    else if (sh < 32) tc_acc96(w0, w1, w2, (uint32_t)v << sh, (uint32_t)(v >> (32 - sh)), sx);
    else if (sh == 32) tc_acc64(w1, w2, (uint32_t)v, sx);
    else tc_acc64(w1, w2, (uint32_t)v << (sh - 32), (uint32_t)(v >> (64 - sh)));
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
// A position in this CTA's sequence of raw stages: work item, window start,
// raw stage start.
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
// Warps 0 .. 15 are the workers.  Per digit stage a worker thread converts
// one pair of consecutive k in each of two core matrices of the left operand
// and, for a Gram, one of the right operand's when it is its warp's turn (those
// rotate over the warps from stage to stage); after each drain chunk it moves
// its slice of the level accumulators (tensor-memory lane quarter warp % 4,
// BN / 4 columns) into 96-bit integers, and after an exponent window it folds
// them into FP64.  The last worker to finish reading a raw stage issues the
// bulk copies of the raw stage two ahead into its buffer.  Warp 16 issues the
// MMAs of each digit stage once every worker has finished it (a dedicated
// warp: the issue blocks while the tensor core works through the previous
// stage, ~700 cycles of MMAs per stage).
//
// The waits form no cycle: digit stage t is produced after the MMAs of stage
// t - 2 completed (a ring of two digit stages); a worker drains the chunk that
// ends at stage e before it finishes stage e + 1, so the MMAs of stage e + 1,
// the next chunk's first (which overwrite the accumulators), are issued after
// every worker drained it.
template <int BN, bool GRAM>
__global__ void __launch_bounds__(kTcThreads, 1)
    k_tc_digits(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
                TcArgs a) {
    using L = TcLayout<BN, GRAM>;
    static_assert(BN % 16 == 0 && BN <= 64, "tile width: a multiple of 16, at most 64");
    extern __shared__ __align__(1024) uint8_t sm_raw[];
    // 1024-byte aligned base (the 128-byte swizzle of the bulk copies needs it)
    uint8_t *sm = sm_raw + ((1024u - (su32(sm_raw) & 1023u)) & 1023u);
    uint64_t *bars = reinterpret_cast<uint64_t *>(sm + L::bar_off);
    uint64_t *empty = bars, *full = bars + kTcDigStages, *rfull = bars + 2 * kTcDigStages;
    uint64_t *accf = rfull + 2, *fin = rfull + 3;
    uint32_t *misc = reinterpret_cast<uint32_t *>(sm + L::misc_off);
    uint32_t *tmem_slot = misc;
    volatile int *abort_flag = reinterpret_cast<volatile int *>(misc + 1);
    uint32_t *rcnt = misc + 2;
    int *n_raw = reinterpret_cast<int *>(misc + 4);  // raw stages issued
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t sbase = su32(sm);
    const int super_k = a.super_k;

    if (tid == 0) {
        for (int s = 0; s < kTcDigStages; ++s) {
            mbar_init(&empty[s], 1);
            mbar_init(&full[s], kTcWarps);
        }
        for (int s = 0; s < 2; ++s) {
            mbar_init(&rfull[s], 1);
            rcnt[s] = 0;
        }
        mbar_init(accf, 1);
        mbar_init(fin, 1);
        *abort_flag = 0;
        *n_raw = 0;
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

    // bulk copies of raw stage q (cursor c) into raw buffer q % 2
    auto issue_raw = [&](uint32_t q, const TcCursor &c) {
        const uint32_t r = q & 1;
        const uint32_t base = sbase + L::raw_off + r * L::raw_bytes;
        if (GRAM) {
            mbar_expect_tx(&rfull[r], 2 * (L::a_box + L::b_box));
            tma_load_2d(base, &mapA, c.k0, c.w.mt0, &rfull[r]);
            tma_load_2d(base + L::a_box, &mapA, c.k0 + 16, c.w.mt0, &rfull[r]);
            tma_load_2d(base + 2 * L::a_box, &mapB, c.k0, c.w.nt * BN, &rfull[r]);
            tma_load_2d(base + 2 * L::a_box + L::b_box, &mapB, c.k0 + 16, c.w.nt * BN, &rfull[r]);
        } else {
            // the A box and the prepared planes of the stage's digit stages
            const int ske = min(c.w.ke, c.sk + super_k);
            const int nd = min(2, (ske - c.k0 + kTcStageK - 1) / kTcStageK);
            mbar_expect_tx(&rfull[r], L::a_box + nd * L::b_box);
            tma_load_2d(base, &mapA, c.w.mt0, c.k0, &rfull[r]);
            const uint8_t *src =
                a.bplanes + ((size_t)c.w.nt * a.nstages + (c.k0 - c.w.kb) / kTcStageK) * L::b_bytes;
            for (int dd = 0; dd < nd; ++dd)
                bulk_load(base + L::a_box + dd * L::b_box, src + (size_t)dd * L::b_bytes, L::b_bytes,
                          &rfull[r]);
        }
        atomicMax(n_raw, (int)q + 1);
    };
    // the MMAs of digit stage t (buffer s, stage st of its drain chunk)
    auto issue_mma = [&](uint32_t s, int st, bool last_of_chunk) {
        const uint32_t abase = sbase + L::dig_off + s * L::stage_bytes;
        const uint32_t bbase = abase + L::a_bytes;
        // left plane i times right planes j = 0 .. 6 - i, into levels l = i + j,
        // in MMAs of at most kLvl levels (N <= 256)
        constexpr int kLvl = 256 / BN < kTcDigits ? 256 / BN : kTcDigits;
#pragma unroll
        for (int i = 0; i < kTcDigits; ++i) {
            const uint64_t ad = smem_desc(abase + i * tc_plane(kTcM), tc_lbo(kTcM), 128);
#pragma unroll
            for (int l0 = i; l0 < kTcDigits; l0 += kLvl) {
                const int nl = min(kLvl, kTcDigits - l0);
                const uint64_t bd =
                    smem_desc(bbase + (uint32_t)((l0 - i) * BN / 8) * 128u, tc_lbo_b(BN), 128);
                // the first product into a level in a drain chunk overwrites it
                // (level l first meets i = 0)
                tc_mma(tmem + (uint32_t)(l0 * BN), ad, bd, tc_idesc(kTcM, nl * BN),
                       (st > 0 || i > 0) ? 1u : 0u);
            }
        }
        tc_commit(&empty[s]);
        if (last_of_chunk) tc_commit(accf);
    };

    if (warp == kTcWarps) {
        // ------------------------------------------------------------ MMA issuer
        uint32_t s = 0, ph = 0;  // ring position and phase of the next digit stage
        bool ok = true;
        for (int it = blockIdx.x; it < a.items && ok; it += gridDim.x) {
            const TcItem w = tc_item<GRAM>(a, it);
            for (int k0 = w.kb; k0 < w.ke && ok; k0 += kTcDrainK) {
                const int nst = min(kTcDrainStages, (w.ke - k0 + kTcStageK - 1) / kTcStageK);
                for (int st = 0; st < nst; ++st) {
                    // every worker finished the stage (and drained the previous
                    // chunk before the first stage of this one)
                    if (!mbar_wait_warp(&full[s], ph, abort_flag, a.error)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    if (lane == 0) issue_mma(s, st, st == nst - 1);
                    __syncwarp();
                    if (++s == kTcDigStages) s = 0, ph ^= 1;
                }
            }
        }
        // all issued MMAs complete before tensor memory is freed
        if (lane == 0) tc_commit(fin);
        __syncwarp();
        mbar_wait_teardown(fin, 0);
    } else {
        if (tid == 0) {
            TcCursor c;
            cur_init<GRAM>(a, c);
            for (uint32_t q = 0; q < 2 && c.valid; ++q) {
                issue_raw(q, c);
                cur_next<GRAM>(a, c);
            }
        }

        // Work units of a digit stage: core matrices (8 rows x 8 k), one pair of
        // consecutive k per lane: lane = 8 pp + r, row r of the core matrix, k
        // pair pp.  The 4-byte digit stores of a warp fill one 128-byte line,
        // and the 16-byte reads of a quarter-warp from a swizzled box (row r's
        // chunk 4 g + pp at (4 g + pp) ^ r) hit distinct banks.  Warp w converts
        // the left operand's row group w in both k-groups; the right operand's
        // units (Gram) rotate over the warps from stage to stage.
        const int r7 = lane & 7, pp = lane >> 3;
        const int ra = warp * 8 + r7;  // left-operand row of this thread
        const uint32_t a_dst = (uint32_t)warp * 128u + (uint32_t)r7 * 16u + (uint32_t)pp * 4u;
        constexpr int BU = BN / 4;  // right-operand units: BN / 8 row groups x 2 k-groups
        // drain slice: row q 32 + lane, columns [cp CPW, (cp + 1) CPW)
        constexpr int CPW = BN / 4;
        const int q = warp & 3, cp = warp >> 2;
        const int drow = q * 32 + lane;
        // per column the level sums of the current window, sum over l of
        // L_l 2^(8 (6 - l)), as a 96-bit integer (w0 least significant)
        uint32_t w0[CPW], w1[CPW], w2[CPW];
#pragma unroll
        for (int c = 0; c < CPW; ++c) w0[c] = w1[c] = w2[c] = 0;

        // the next chunk to drain: work item, window start, chunk start,
        // index of its last digit stage
        TcItem dw{0, 0, 0, 0};
        int dit = blockIdx.x, dsk = 0, dk0 = 0, dlast = 0;
        bool dvalid = dit < a.items;
        uint32_t dn = 0;  // chunks drained
        auto dstages = [&]() { return min(kTcDrainStages, (dw.ke - dk0 + kTcStageK - 1) / kTcStageK); };
        if (dvalid) {
            dw = tc_item<GRAM>(a, dit);
            dsk = dk0 = dw.kb;
            dlast = dstages() - 1;
        }
        auto drain = [&]() -> bool {
            if (!mbar_wait_warp(accf, dn & 1, abort_flag, a.error)) return false;
            tc_fence_after();
            const uint32_t tb = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(cp * CPW);
            // levels 0 and 1, 2 and 3 pair up exactly in 32 bits (|L_0 2^8 + L_1|
            // < 2^30.2, |L_2 2^8 + L_3| < 2^30.9): each pair is read with one
            // wait and added once; levels 4, 5 and 6 are added alone
            auto f2i = [](uint32_t u) { return __float2int_rn(__uint_as_float(u)); };
#pragma unroll
            for (int l = 0; l < 4; l += 2) {
                uint32_t u[CPW / 4][4], v[CPW / 4][4];
#pragma unroll
                for (int j = 0; j < CPW / 4; ++j) {
                    tc_ld4(tb + (uint32_t)(l * BN + 4 * j), u[j]);
                    tc_ld4(tb + (uint32_t)((l + 1) * BN + 4 * j), v[j]);
                }
                tc_wait_ld();
#pragma unroll
                for (int c = 0; c < CPW; ++c)
                    tc_acc_level(w0[c], w1[c], w2[c],
                                 f2i(u[c >> 2][c & 3]) * 256 + f2i(v[c >> 2][c & 3]), l + 1);
            }
#pragma unroll
            for (int l = 4; l < kTcDigits; ++l) {
                uint32_t u[CPW / 4][4];
#pragma unroll
                for (int j = 0; j < CPW / 4; ++j) tc_ld4(tb + (uint32_t)(l * BN + 4 * j), u[j]);
                tc_wait_ld();
#pragma unroll
                for (int c = 0; c < CPW; ++c) tc_acc_level(w0[c], w1[c], w2[c], f2i(u[c >> 2][c & 3]), l);
            }
            ++dn;
            const int ske = min(dw.ke, dsk + super_k);
            if (dk0 + kTcDrainK >= ske) {
                // the window ends: its sums, w 2^(er + ec - 2106)
                // converted with integer instructions, go into the work item's
                // split-k partial (Gram; a work item of several windows adds
                // them there) or straight into Y (a linear combination)
                const int sidx = (dsk - (GRAM ? 0 : dw.kb)) / super_k;
                const int grow = dw.mt0 + drow;
                const int er = grow < a.M ? __ldg(a.eA + (size_t)sidx * a.M + grow) : 1;
                const bool first = dsk == dw.kb;
                const int z = dit / (a.mtiles * a.ntiles);
#pragma unroll
                for (int c = 0; c < CPW; ++c) {
                    const int col = cp * CPW + c, gcol = dw.nt * BN + col;
                    const int ec = GRAM ? (gcol < a.N ? __ldg(a.eB + (size_t)sidx * a.N + gcol) : 1)
                                        : __ldg(a.eB + ((size_t)dw.nt * a.nsup + sidx) * BN + col);
                    const double val = (er == 0x7FF || ec == 0x7FF)
                                           ? __longlong_as_double(0x7FF8000000000000LL)
                                           : tc_i128_f64((long long)(int)w2[c],
                                                         ((unsigned long long)w1[c] << 32) | w0[c],
                                                         er + ec - 2106);
                    w0[c] = w1[c] = w2[c] = 0;
                    if (GRAM) {
                        // the work item's split-k partial: its first window
                        // writes it, later windows add to it
                        if (grow < a.M && gcol < a.N) {
                            double *dst = a.out + (size_t)z * a.M * a.N + grow + (size_t)gcol * a.M;
                            *dst = first ? val : *dst + val;
                        }
                    } else if (grow < a.M && gcol < a.N) {
                        double *dst = a.out + grow + (size_t)gcol * a.ldo;
                        // alpha = +-1 needs no FP64 multiply (the sign folds
                        // into the beta fma or the store)
                        double y = a.alpha == 1.0 ? val : a.alpha == -1.0 ? -val : a.alpha * val;
                        if (a.accumulate) {
                            y += *dst;
                        } else if (a.beta != nullptr) {
                            const double bb = a.beta[a.incb == 0 ? 0 : (size_t)gcol * a.incb];
                            if (bb != 0.0) y = fma(bb, *dst, y);
                        }
                        *dst = y;
                    }
                }
            }
            // the next chunk
            const int tnext = dlast + 1;
            dk0 += kTcDrainK;
            if (dk0 >= ske) {
                dsk += super_k;
                if (dsk >= dw.ke) {
                    dit += gridDim.x;
                    dvalid = dit < a.items;
                    if (dvalid) {
                        dw = tc_item<GRAM>(a, dit);
                        dsk = dw.kb;
                    }
                }
                dk0 = dsk;
            }
            if (dvalid) dlast = tnext + dstages() - 1;
            return true;
        };

        // ---- production
        TcCursor cons;
        cur_init<GRAM>(a, cons);
        int t = 0;        // digit stages produced
        int sidx = 0;     // window of the current raw stage
        uint32_t s = 0, ph = 0;  // ring position and phase of stage t
        uint32_t qr = 0;  // raw stages read
        int em_a = 1;
        bool ok = true;
        while (ok && cons.valid) {
            const int ske = min(cons.w.ke, cons.sk + super_k);
            if (cons.k0 == cons.sk) {
                // a window starts: its index and the exponent field of this
                // thread's row
                sidx = (cons.sk - (GRAM ? 0 : cons.w.kb)) / super_k;
                const int gr = cons.w.mt0 + ra;
                em_a = gr < a.M ? __ldg(a.eA + (size_t)sidx * a.M + gr) : 1;
            }
            const uint32_t r = qr & 1;
            const uint8_t *raw = sm + L::raw_off + r * L::raw_bytes;
            const int nd = min(2, (ske - cons.k0 + kTcStageK - 1) / kTcStageK);
            for (int dd = 0; dd < nd; ++dd, ++t) {
                // the right-operand unit of this warp at stage t (Gram): unit b goes
                // to warp (b + t BU) mod 16
                const int bu = (warp - (int)(((uint32_t)t * BU) & 15u)) & 15;
                const bool hasb = GRAM && bu < BU;
                const int rb = (bu >> 1) * 8 + r7, gb = bu & 1;
                int emb = 1;
                if (hasb) {
                    const int gc = cons.w.nt * BN + rb;
                    emb = gc < a.N ? __ldg(a.eB + (size_t)sidx * a.N + gc) : 1;
                }
                if (dd == 0 && !mbar_wait_warp(&rfull[r], (qr >> 1) & 1, abort_flag, a.error)) {
                    ok = false;
                    break;
                }
                // the MMAs of stage t - kTcDigStages read this buffer
                if (t >= kTcDigStages && !mbar_wait_warp(&empty[s], ph ^ 1, abort_flag, a.error)) {
                    ok = false;
                    break;
                }
                uint8_t *abuf = sm + L::dig_off + s * L::stage_bytes;
                uint8_t *bbuf = abuf + L::a_bytes;
                if (!GRAM) {
                    // the right operand's prepared planes of this digit stage, from
                    // the raw stage
                    const uint4 *src = reinterpret_cast<const uint4 *>(raw + L::a_box + dd * L::b_box);
                    uint4 *dst = reinterpret_cast<uint4 *>(bbuf);
                    for (int i = tid; i < (int)(L::b_bytes / 16); i += kTcWarps * 32) dst[i] = src[i];
                }
                // the pairs: left operand k-groups 0 and 1, and the right-operand unit
                double2 v0, v1, vb = make_double2(0.0, 0.0);
                if (GRAM) {
                    // box dd: row ra's 16 k as 8 chunks of 16 bytes, chunk c at c ^ (ra % 8)
                    const uint8_t *box = raw + dd * L::a_box + (uint32_t)ra * 128u;
                    v0 = *reinterpret_cast<const double2 *>(box + ((uint32_t)(pp ^ r7) << 4));
                    v1 = *reinterpret_cast<const double2 *>(box + ((uint32_t)((4 + pp) ^ r7) << 4));
                    if (hasb) {
                        const uint8_t *bx = raw + 2 * L::a_box + dd * L::b_box + (uint32_t)rb * 128u;
                        vb = *reinterpret_cast<const double2 *>(
                            bx + ((uint32_t)((4 * gb + pp) ^ r7) << 4));
                    }
                } else {
                    // box [32 k][128 rows]
                    const double *col = reinterpret_cast<const double *>(raw) +
                                        (size_t)(dd * kTcStageK + 2 * pp) * kTcM + ra;
                    v0 = make_double2(col[0], col[kTcM]);
                    v1 = make_double2(col[8 * kTcM], col[9 * kTcM]);
                }
                // row groups past the operand's last row hold zero digits: the
                // conversion is skipped (warp-uniform)
                const bool live_a = cons.w.mt0 + warp * 8 < a.M;
                const bool live_b = !GRAM || cons.w.nt * BN + (bu >> 1) * 8 < a.N;
                uint32_t d0[kTcDigits], d1[kTcDigits], db[kTcDigits];
#pragma unroll
                for (int i = 0; i < kTcDigits; ++i) d0[i] = d1[i] = db[i] = 0u;
                if (live_a) {
                    tc_digit_pair(v0.x, v0.y, (uint32_t)em_a, d0);
                    tc_digit_pair(v1.x, v1.y, (uint32_t)em_a, d1);
                }
                if (hasb && live_b) tc_digit_pair(vb.x, vb.y, (uint32_t)emb, db);
#pragma unroll
                for (int i = 0; i < kTcDigits; ++i) {
                    uint8_t *pa = abuf + (uint32_t)i * tc_plane(kTcM) + a_dst;
                    *reinterpret_cast<uint32_t *>(pa) = d0[i];
                    *reinterpret_cast<uint32_t *>(pa + tc_lbo(kTcM)) = d1[i];
                }
                if (hasb) {
                    const uint32_t b_dst = (uint32_t)gb * tc_lbo_b(BN) + (uint32_t)(bu >> 1) * 128u +
                                           (uint32_t)r7 * 16u + (uint32_t)pp * 4u;
#pragma unroll
                    for (int i = 0; i < kTcDigits; ++i)
                        *reinterpret_cast<uint32_t *>(bbuf + b_dst + (uint32_t)i * BN * 16u) = db[i];
                }
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                // chunks that ended at stage t - 1 or earlier
                while (dvalid && dlast < t) {
                    if (!drain()) {
                        ok = false;
                        break;
                    }
                }
                if (!ok) break;
                // arrival (release; the stores and drains above come first)
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(&full[s]);
                if (++s == kTcDigStages) s = 0, ph ^= 1;
            }
            if (!ok) break;
            // raw stage qr is read; the last warp copies raw stage qr + 2 into its buffer
            __syncwarp();
            if (lane == 0 && smem_arrive(&rcnt[r]) == kTcWarps - 1) {
                rcnt[r] = 0;
                TcCursor c2 = cons;
                cur_next<GRAM>(a, c2);
                if (c2.valid) cur_next<GRAM>(a, c2);
                if (c2.valid) issue_raw(qr + 2, c2);
            }
            __syncwarp();
            ++qr;
            cur_next<GRAM>(a, cons);
        }
        // the remaining chunks
        while (ok && dvalid)
            if (!drain()) ok = false;

    }
    // teardown: the bulk copies still in flight (after an abort) land before
    // the CTA exits; the MMA warp waited for its MMAs
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        const int nr = *n_raw;
        for (int qq = max(nr - 2, 0); qq < nr; ++qq)
            mbar_wait_teardown(&rfull[qq & 1], (qq >> 1) & 1);
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(kTcTmemCols)
                     : "memory");
    }
}

// Exponent fields for the Gram operands: out[s * ncols + c] = the largest
// exponent field (at least 1) of column c of X (n x ncols, leading dimension
// ld, 16-byte aligned columns) over rows [s super, (s + 1) super).  One warp
// per (column, piece of at most kTcExpPiece rows of one window), 16-byte
// loads, merged with atomicMax into `out`, which starts at 0.
constexpr int kTcExpPiece = 4096;
__global__ void __launch_bounds__(256) k_tc_expcols(const double *__restrict__ X, size_t ld,
                                                    int n, int ncols, int super, int nsup,
                                                    int *__restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int pieces = (super + kTcExpPiece - 1) / kTcExpPiece;  // per window
    const long long units = (long long)nsup * pieces * ncols;
    const long long nw = (long long)gridDim.x * 8;
    for (long long wid = (long long)blockIdx.x * 8 + (threadIdx.x >> 5); wid < units; wid += nw) {
        const int c = (int)(wid % ncols);
        const long long sp = wid / ncols;
        const int s = (int)(sp / pieces), pc = (int)(sp % pieces);
        const int r0 = s * super + pc * kTcExpPiece;
        const int r1 = (int)std::min<long long>(std::min<long long>(n, (long long)(s + 1) * super),
                                                r0 + kTcExpPiece);
        const double *col = X + (size_t)c * ld;
        int em = 1;
#pragma unroll 4
        for (int r = r0 + 2 * lane; r < r1; r += 64) {
            if (r + 1 < r1) {
                const double2 u = __ldg(reinterpret_cast<const double2 *>(col + r));
                em = max(em, max(tc_exp_field(u.x), tc_exp_field(u.y)));
            } else {
                em = max(em, tc_exp_field(__ldg(col + r)));
            }
        }
        em = (int)__reduce_max_sync(0xffffffffu, (unsigned)em);
        if (lane == 0) {
            if (pieces == 1) out[(size_t)s * ncols + c] = em;
            else atomicMax(out + (size_t)s * ncols + c, em);
        }
    }
}
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
// C[k + c ldc]) prepared once per call: block (window, n tile) writes the
// exponent fields of its BN columns and the digit planes of each 16-k digit
// stage of the window in the stage layout of the product kernel.
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
             int ldc, double *scratch, size_t scratch_elems, cudaStream_t st, TcExpCache *cache) {
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
    a.mtiles = (m + kTcM - 1) / kTcM;
    a.ntiles = (w + bn - 1) / bn;
    const int mn = a.mtiles * a.ntiles;
    const int sms = device_sms();
    // one wave of one CTA per SM over all work items (k ranges of a multiple
    // of the drain chunk), fewer and longer ranges until the partials fit
    // the scratch
    int z = std::max(1, sms / mn);
    long long kc = ((long long)(n + z - 1) / z + kTcDrainK - 1) / kTcDrainK * kTcDrainK;
    GCGE_REQUIRE((size_t)m * w <= scratch_elems, GCGE_ERR_ARG, "tc_gram: scratch too small");
    while ((size_t)((n + kc - 1) / kc) * m * w > scratch_elems) kc *= 2;
    // the exponent window: the whole k range of a work item, or windows of
    // the largest size when the range is longer.  One
    // exponent per column over K rows bounds the error of an entry by
    // 2^-54 sqrt(K) |x| |y|, below the FP64 dot product's K 2^-53 |x| |y|.
    if (kc > kTcSuperGramMax) kc = (kc + kTcSuperGramMax - 1) / kTcSuperGramMax * kTcSuperGramMax;
    const int super_k = (int)std::min<long long>(kc, kTcSuperGramMax);
    z = (int)((n + kc - 1) / kc);
    a.super_k = super_k;
    const int nsup = (n + super_k - 1) / super_k;
    const long long pieces = (super_k + kTcExpPiece - 1) / kTcExpPiece;
    auto expcols = [&](const double *X, int ld, int cols, int *out) {
        if (pieces > 1) GCGE_CUDA(cudaMemsetAsync(out, 0, sizeof(int) * (size_t)nsup * cols, st));
        const int gx = (int)std::min<long long>(8 * sms, (nsup * pieces * cols + 7) / 8);
        k_tc_expcols<<<gx, 256, 0, st>>>(X, (size_t)ld, n, cols, super_k, nsup, out);
        GCGE_CHECK_LAUNCH();
        count_launch();
    };
    DevBuf<int> &eb = slot_stage().tc_exps;
    int *eA, *eB;
    if (cache) {
        // Q's fields from the cache (computed there on first use)
        if (!cache->matches(Q, (size_t)ldq, n, m, super_k, 0)) {
            cache->e.alloc((size_t)nsup * m);
            expcols(Q, ldq, m, cache->e.p);
            cache->set(Q, (size_t)ldq, n, m, super_k, 0);
        }
        eA = cache->e.p;
        eb.alloc((size_t)nsup * w);
        eB = eb.p;
    } else {
        eb.alloc((size_t)nsup * (m + w));
        eA = eb.p;
        eB = eb.p + (size_t)nsup * m;
        expcols(Q, ldq, m, eA);
    }
    expcols(P, ldp, w, eB);
    a.eA = eA;
    a.eB = eB;
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
// longer than one window (432) run as several launches, each later one
// adding its block's product to Y.
void tc_lincomb(int n, int k, int m, const double *X, int ldx, const double *C, int ldc, double *Y,
                int ldy, const double *beta_dev, int incb, cudaStream_t st, double alpha,
                void *scratch, size_t scratch_bytes, TcExpCache *cache) {
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
        // exponent fields of the rows of X over the block's columns (kept in
        // the cache when the whole contraction is one block)
        const bool cached = cache != nullptr && k <= kTcSuperLincomb;
        DevBuf<int> &eb = cached ? cache->e : slot_stage().tc_exps;
        count_launch();
        if (!cached || !cache->matches(Xb, (size_t)ldx, n, kb, kTcSuperLincomb, 1)) {
            eb.alloc((size_t)n);
            k_tc_exprows<<<dim3((n + 255) / 256, 1), 256, 0, st>>>(Xb, (size_t)ldx, n, kb,
                                                                 kTcSuperLincomb, eb.p);
            GCGE_CHECK_LAUNCH();
            count_launch();
            if (cached) cache->set(Xb, (size_t)ldx, n, kb, kTcSuperLincomb, 1);
        }
        a.bplanes = planes;
        a.eA = eb.p;
        a.eB = bexps;
        launch_tc_bn<false>(ma, ma, a, bn, std::min(a.items, device_sms()), st);
    }
}

}  // namespace gcge
