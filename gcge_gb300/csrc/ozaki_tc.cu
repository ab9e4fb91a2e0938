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
// Kernel structure (one CTA per SM, persistent over work items):
//  * warp 0 allocates tensor memory (512 columns: 7 levels x BN) and one of
//    its threads issues the MMAs (M = 128 rows, N = BN, K = 16 per
//    instruction, f16 x f16 -> f32), committing each stage to an mbarrier;
//  * 7 producer warps compute exponents and digit planes of the next 32-k
//    stage into shared memory (two stages, K-major core-matrix layout:
//    8 rows x 16 bytes per core matrix, padded so stores are conflict-free);
//  * 12 drain warps read the level accumulators of each 96-k chunk from
//    tensor memory (warp w reads lanes 32 (w % 4) .. + 31), fold them into
//    int64 registers, and at each super-chunk end into FP64 accumulators in
//    shared memory; at the end of a work item they write the result.
// Every wait on an mbarrier is bounded; a wait that runs out sets the error
// word and every role stops at its next wait, so the kernel always returns.
#include <cstdint>

#include "common.cuh"

namespace gcge {
namespace {

constexpr int kTcDigits = 7;
constexpr int kTcM = 128;      // output rows per tile (tensor-memory lanes)
constexpr int kTcStageK = 32;  // k per pipeline stage (two 16-k MMA steps)
constexpr int kTcDrainStages = 3;
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
// Exponent-field slots: the producers fill super-chunk j + 1's while they
// write super-chunk j's digits and the drain folds super-chunk j - 1 with its
// own, so three slots keep the producers from waiting on the drain.
constexpr int kTcExpSlots = 3;

// Byte layout of one operand tile of R rows in a stage: plane i (digit),
// k-group g (8 consecutive k), row r: i * plane + g * lbo + (r / 8) * 128 +
// (r % 8) * 16, with lbo = R * 16 + 16 (the pad keeps the producers' 16-byte
// stores of the 8 k-groups of a row on different banks).
__host__ __device__ constexpr uint32_t tc_lbo(int rows) { return (uint32_t)rows * 16u + 16u; }
__host__ __device__ constexpr uint32_t tc_plane(int rows) { return kTcKGroups * tc_lbo(rows); }
__host__ __device__ constexpr uint32_t tc_tile_bytes(int rows) {
    return kTcDigits * tc_plane(rows);
}

template <int BN>
struct TcLayout {
    static constexpr uint32_t a_bytes = tc_tile_bytes(kTcM);
    static constexpr uint32_t b_bytes = tc_tile_bytes(BN);
    static constexpr uint32_t stage_bytes = a_bytes + b_bytes;
    static constexpr uint32_t stages_off = 0;
    static constexpr uint32_t acc_off = 2 * stage_bytes;  // double acc[BN][kTcM]
    static constexpr uint32_t ea_off = acc_off + (uint32_t)BN * kTcM * 8;  // int ea[3][kTcM]
    static constexpr uint32_t eb_off = ea_off + kTcExpSlots * kTcM * 4;     // int eb[3][BN]
    static constexpr uint32_t bar_off = (eb_off + kTcExpSlots * BN * 4 + 15) / 16 * 16;
    // full[2] empty[2] accf tfree exfull[3] exfree[3] final
    static constexpr int nbars = 7 + 2 * kTcExpSlots;
    static constexpr uint32_t misc_off = bar_off + nbars * 8;  // tmem slot, abort flag
    static constexpr uint32_t bytes = misc_off + 16;
};

struct TcArgs {
    int M, N, K;
    // gram: A = Q, element (k, r) at A[k + r lda]; B = P, element (k, c) at
    // B[k + c ldb].  lincomb: A = X, element (r, k) at A[r + k lda]; B = C,
    // whose digit planes and exponents were prepared by k_tc_bprep.
    const double *A;
    size_t lda;
    const double *B;
    size_t ldb;
    int super_k;    // k per shared exponent (multiple of kTcDrainK)
    int kchunk;     // gram: k per work item (multiple of super_k)
    int items;      // work items
    int mtiles, ntiles;
    double *out;    // gram: partials [kz][M x N]; lincomb: Y (ldo)
    size_t ldo;
    const double *beta;
    int incb;
    double alpha;
    const uint8_t *bplanes;  // lincomb: [ntile][stage][b_bytes]
    const int *bexps;        // lincomb: [ntile][super][BN]
    int nstages, nsup;       // lincomb: stages and super-chunks of K
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

// exact int64 -> double for |t| < 2^51
__device__ __forceinline__ double tc_i64_to_f64(long long t) {
    return __longlong_as_double(t + 0x4338000000000000LL) - 6755399441055744.0;
}

// ---------------------------------------------------------------- kernel
// Work item `it`: gram: (m tile, n tile, k range); lincomb: (m tile = 128
// rows of X and Y, n tile).  Fills its output tile coordinates and k range.
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

template <int BN, bool GRAM>
__global__ void __launch_bounds__(kTcThreads, 1) k_tc_digits(TcArgs a) {
    using L = TcLayout<BN>;
    extern __shared__ __align__(1024) uint8_t sm[];
    double *acc = reinterpret_cast<double *>(sm + L::acc_off);  // [BN][kTcM]
    int *ea = reinterpret_cast<int *>(sm + L::ea_off);           // [3][kTcM]
    int *eb = reinterpret_cast<int *>(sm + L::eb_off);           // [3][BN]
    uint64_t *bars = reinterpret_cast<uint64_t *>(sm + L::bar_off);
    uint64_t *full = bars, *empty = bars + 2, *accf = bars + 4, *tfree = bars + 5;
    uint64_t *exfull = bars + 6, *exfree = bars + 6 + kTcExpSlots, *fin = bars + 6 + 2 * kTcExpSlots;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(sm + L::misc_off);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(sm + L::misc_off + 4);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t sbase = su32(sm);

    if (tid == 0) {
        for (int s = 0; s < 2; ++s) {
            mbar_init(&full[s], kTcProdThreads);
            mbar_init(&empty[s], 1);
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
        constexpr uint32_t idesc = tc_idesc(kTcM, BN);
        uint32_t t = 0, d = 0;  // stages and drain chunks issued so far
        bool ok = true;
        for (int it = blockIdx.x; it < a.items && ok; it += gridDim.x) {
            const TcItem w = tc_item<GRAM>(a, it);
            for (int k0 = w.kb; k0 < w.ke && ok; k0 += kTcDrainK, ++d) {
                if (d > 0 && !mbar_wait_warp(tfree, (d - 1) & 1, abort_flag, a.error)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                uint32_t started = 0;  // levels written in this drain chunk
                const int nst = min(kTcDrainStages, (w.ke - k0 + kTcStageK - 1) / kTcStageK);
                for (int st = 0; st < nst; ++st, ++t) {
                    const uint32_t s = t & 1;
                    if (!mbar_wait_warp(&full[s], (t >> 1) & 1, abort_flag, a.error)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    if (lane == 0) {
                        const uint32_t abase = sbase + L::stages_off + s * L::stage_bytes;
                        const uint32_t bbase = abase + L::a_bytes;
#pragma unroll
                        for (int ks = 0; ks < kTcStageK / 16; ++ks) {
#pragma unroll
                            for (int i = 0; i < kTcDigits; ++i) {
                                const uint64_t ad =
                                    smem_desc(abase + i * tc_plane(kTcM) + 2 * ks * tc_lbo(kTcM),
                                              tc_lbo(kTcM), 128);
#pragma unroll
                                for (int j = 0; j + i < kTcDigits; ++j) {
                                    const uint64_t bd =
                                        smem_desc(bbase + j * tc_plane(BN) + 2 * ks * tc_lbo(BN),
                                                  tc_lbo(BN), 128);
                                    const int l = i + j;
                                    tc_mma(tmem + (uint32_t)(l * BN), ad, bd, idesc,
                                           (started >> l) & 1u);
                                    started |= 1u << l;
                                }
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
        mbar_wait_warp(fin, 0, abort_flag, a.error);
    } else if (warp >= 4 && warp < 4 + kTcDrainWarps) {
        // ------------------------------------------------------------ drain
        const int q = warp & 3;                 // tensor-memory lane quarter
        const int third = (warp - 4) >> 2;      // column-group share
        const int row = q * 32 + lane;          // output row within the tile
        constexpr int NG = BN / 8;              // 8-column groups
        constexpr int GPT = (NG + 2) / 3;       // groups per drain thread (at most)
        long long thi[GPT * 8], tlo[GPT * 8];
#pragma unroll
        for (int c = 0; c < GPT * 8; ++c) thi[c] = tlo[c] = 0;
        uint32_t d = 0, sc = 0;  // drain chunks and super-chunks consumed so far
        bool ok = true;
        for (int it = blockIdx.x; it < a.items && ok; it += gridDim.x) {
            const TcItem w = tc_item<GRAM>(a, it);
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
                                const long long L = (long long)__float2int_rn(__uint_as_float(v[cc]));
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
                // fold the super-chunk into the FP64 accumulators
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
                        double &A = acc[c * kTcM + row];
                        if (er == 0x7FF || ec == 0x7FF) {
                            A = __longlong_as_double(0x7FF8000000000000LL);
                        } else {
                            const int fld = er + ec - 1085;  // exponent field of the scale
                            if (fld > 0) {
                                const double sc2 = fld >= 2047
                                                       ? __longlong_as_double(0x7FF0000000000000LL)
                                                       : __longlong_as_double((long long)fld << 52);
                                const double v = fma(tc_i64_to_f64(thi[gi * 8 + cc]), 16777216.0,
                                                     tc_i64_to_f64(tlo[gi * 8 + cc]));
                                A = fma(v, sc2, A);
                            }
                        }
                        thi[gi * 8 + cc] = tlo[gi * 8 + cc] = 0;
                    }
                }
                mbar_arrive(&exfree[b]);
            }
            if (!ok) break;
            // the work item's result
            const int grow = w.mt0 + row;
            if (grow < a.M) {
                for (int g = third; g < NG; g += 3) {
                    for (int cc = 0; cc < 8; ++cc) {
                        const int col = w.nt * BN + g * 8 + cc;
                        if (col >= a.N) continue;
                        const double v = acc[(g * 8 + cc) * kTcM + row];
                        if (GRAM) {
                            const int z = it / (a.mtiles * a.ntiles);
                            a.out[(size_t)z * a.M * a.N + grow + (size_t)col * a.M] = v;
                        } else {
                            double y = a.alpha * v;
                            double *dst = a.out + grow + (size_t)col * a.ldo;
                            if (a.beta != nullptr) {
                                const double bb = a.beta[a.incb == 0 ? 0 : (size_t)col * a.incb];
                                if (bb != 0.0) y = fma(bb, *dst, y);
                            }
                            *dst = y;
                        }
                    }
                }
            }
        }
    } else {
        // ------------------------------------------------------------ producers
        // The super-chunks of this CTA's work items form one sequence j = 0, 1,
        // ...; while the producers write the digit planes of super-chunk j,
        // each stage also takes a slice of the exponent pass of super-chunk
        // j + 1 (its first reads of those data from HBM), so the exponent pass
        // overlaps the digit work instead of stalling it, and the digit pass
        // reads data the exponent pass brought into L2.
        const int pw = warp < 4 ? warp - 1 : warp - (4 + kTcDrainWarps) + 3;  // 0..6
        const int p = pw * 32 + lane;                                          // 0..223
        auto prod_sync = [] { asm volatile("bar.sync 1, %0;" ::"n"(kTcProdThreads) : "memory"); };
        constexpr int RX = GRAM ? kTcM + BN : kTcM;  // rows of the exponent pass
        // exponent items [e0, e1) of super-chunk (w, sk, ske) into slot buffers
        auto exp_items = [&](const TcItem &w, int sk, int ske, int e0, int e1, int *ebuf_a,
                             int *ebuf_b) {
            for (int e = e0 + p; e < e1; e += 2 * kTcProdThreads) {
                int em2[2] = {1, 1};
                int rr2[2] = {-1, -1};
                double v[2][8];
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int ee = e + h * kTcProdThreads;
#pragma unroll
                    for (int q = 0; q < 8; ++q) v[h][q] = 0.0;
                    if (ee >= e1) continue;
                    const int r = ee % RX, g = ee / RX;
                    const int k = sk + g * 8;
                    rr2[h] = r;
                    if (GRAM) {
                        const bool isb = r >= kTcM;
                        const int gr = isb ? w.nt * BN + (r - kTcM) : w.mt0 + r;
                        if (gr >= (isb ? a.N : a.M)) continue;
                        const double *src =
                            isb ? a.B + (size_t)gr * a.ldb : a.A + (size_t)gr * a.lda;
                        if (k + 8 <= ske && (reinterpret_cast<uintptr_t>(src + k) & 15) == 0) {
                            const double2 *s2 = reinterpret_cast<const double2 *>(src + k);
#pragma unroll
                            for (int q = 0; q < 4; ++q) {
                                const double2 u = __ldg(s2 + q);
                                v[h][2 * q] = u.x;
                                v[h][2 * q + 1] = u.y;
                            }
                        } else {
#pragma unroll
                            for (int q = 0; q < 8; ++q)
                                if (k + q < ske) v[h][q] = __ldg(src + k + q);
                        }
                    } else {
                        const int gr = w.mt0 + r;
                        if (gr >= a.M) continue;
#pragma unroll
                        for (int q = 0; q < 8; ++q)
                            if (k + q < ske) v[h][q] = __ldg(a.A + gr + (size_t)(k + q) * a.lda);
                    }
                }
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    if (rr2[h] < 0) continue;
#pragma unroll
                    for (int q = 0; q < 8; ++q) em2[h] = max(em2[h], tc_exp_field(v[h][q]));
                    const int r = rr2[h];
                    if (GRAM && r >= kTcM) atomicMax(&ebuf_b[r - kTcM], em2[h]);
                    else atomicMax(&ebuf_a[r], em2[h]);
                }
            }
        };
        // slot buffers of super-chunk (w, sk): set to 1 (the minimum field),
        // or, for the right operand of a linear combination, its prepared fields
        auto exp_init = [&](const TcItem &w, int sk, int *ebuf_a, int *ebuf_b) {
            for (int r = p; r < kTcM; r += kTcProdThreads) ebuf_a[r] = 1;
            if (GRAM) {
                for (int c = p; c < BN; c += kTcProdThreads) ebuf_b[c] = 1;
            } else {
                const int sidx = (sk - w.kb) / super_k;
                for (int c = p; c < BN; c += kTcProdThreads)
                    ebuf_b[c] = a.bexps[((size_t)w.nt * a.nsup + sidx) * BN + c];
            }
        };
        auto n_exp_items = [&](int sk, int ske) { return RX * ((ske - sk + 7) / 8); };

        uint32_t t = 0, j = 0;
        bool ok = true;
        int it = blockIdx.x;
        TcItem w = tc_item<GRAM>(a, it);
        int sk = w.kb;
        // prologue: the exponent pass of the first super-chunk on its own
        {
            const int ske = min(w.ke, sk + super_k);
            exp_init(w, sk, ea, eb);
            prod_sync();
            exp_items(w, sk, ske, 0, n_exp_items(sk, ske), ea, eb);
            prod_sync();
            mbar_arrive(&exfull[0]);
        }
        while (ok) {
            const int ske = min(w.ke, sk + super_k);
            const uint32_t b = j % kTcExpSlots;
            // the next super-chunk of the sequence (same work item, or the
            // CTA's next one)
            int it1 = it, sk1 = ske;
            if (sk1 >= w.ke) {
                it1 = it + gridDim.x;
                sk1 = -1;
            }
            const bool has_next = it1 < a.items;
            TcItem w1 = w;
            if (has_next && sk1 < 0) {
                w1 = tc_item<GRAM>(a, it1);
                sk1 = w1.kb;
            }
            const int ske1 = has_next ? min(w1.ke, sk1 + super_k) : 0;
            const uint32_t b1 = (j + 1) % kTcExpSlots;
            int *ea1 = ea + b1 * kTcM, *eb1 = eb + b1 * BN;
            // every producer wait is followed by a producer barrier and a check
            // of the abort flag, so that all producer warps leave together
            // (none is left waiting at a barrier the others skip)
            if (has_next && j + 1 >= kTcExpSlots)
                mbar_wait_warp(&exfree[b1], ((j + 1 - kTcExpSlots) / kTcExpSlots) & 1, abort_flag,
                               a.error);
            prod_sync();
            if (*abort_flag) break;
            if (has_next) exp_init(w1, sk1, ea1, eb1);
            const int nst = (ske - sk + kTcStageK - 1) / kTcStageK;
            const int ne1 = has_next ? n_exp_items(sk1, ske1) : 0;
            const int per = (ne1 + nst - 1) / nst;
            const int *ebuf_a = ea + b * kTcM, *ebuf_b = eb + b * BN;
            for (int st = 0; st < nst; ++st, ++t) {
                const int k0 = sk + st * kTcStageK;
                const uint32_t s = t & 1;
                mbar_wait_warp(&empty[s], ((t >> 1) & 1) ^ 1, abort_flag, a.error);
                prod_sync();
                if (*abort_flag) {
                    ok = false;
                    break;
                }
                // a slice of the next super-chunk's exponent pass
                if (has_next)
                    exp_items(w1, sk1, ske1, st * per, min(ne1, (st + 1) * per), ea1, eb1);
                uint8_t *abuf = sm + L::stages_off + s * L::stage_bytes;
                uint8_t *bbuf = abuf + L::a_bytes;
                constexpr int a_items = kTcM * kTcKGroups;
                constexpr int b_items = GRAM ? BN * kTcKGroups : 0;
                // digit planes of this stage, two items' loads in flight
                for (int item = p; item < a_items + b_items; item += 2 * kTcProdThreads) {
                    double v[2][8];
                    int em[2] = {1, 1};
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const int ii0 = item + h * kTcProdThreads;
#pragma unroll
                        for (int q = 0; q < 8; ++q) v[h][q] = 0.0;
                        if (ii0 >= a_items + b_items) continue;
                        const bool isb = ii0 >= a_items;
                        const int ii = isb ? ii0 - a_items : ii0;
                        const int rows = isb ? BN : kTcM;
                        const int r = ii % rows, g = ii / rows;
                        const int k = k0 + g * 8;
                        em[h] = isb ? ebuf_b[r] : ebuf_a[r];
                        if (GRAM) {
                            const int gr = isb ? w.nt * BN + r : w.mt0 + r;
                            if (gr >= (isb ? a.N : a.M)) continue;
                            const double *src =
                                isb ? a.B + (size_t)gr * a.ldb : a.A + (size_t)gr * a.lda;
                            if (k + 8 <= ske && (reinterpret_cast<uintptr_t>(src + k) & 15) == 0) {
                                const double2 *s2 = reinterpret_cast<const double2 *>(src + k);
#pragma unroll
                                for (int q = 0; q < 4; ++q) {
                                    const double2 u = __ldg(s2 + q);
                                    v[h][2 * q] = u.x;
                                    v[h][2 * q + 1] = u.y;
                                }
                            } else {
#pragma unroll
                                for (int q = 0; q < 8; ++q)
                                    if (k + q < ske) v[h][q] = __ldg(src + k + q);
                            }
                        } else {
                            const int gr = w.mt0 + r;
                            if (gr >= a.M) continue;
#pragma unroll
                            for (int q = 0; q < 8; ++q)
                                if (k + q < ske)
                                    v[h][q] = __ldg(a.A + gr + (size_t)(k + q) * a.lda);
                        }
                    }
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const int ii0 = item + h * kTcProdThreads;
                        if (ii0 >= a_items + b_items) continue;
                        const bool isb = ii0 >= a_items;
                        const int ii = isb ? ii0 - a_items : ii0;
                        const int rows = isb ? BN : kTcM;
                        const int r = ii % rows, g = ii / rows;
                        uint4 dg[kTcDigits];
                        tc_digits8(v[h], em[h], dg);
                        uint8_t *base = (isb ? bbuf : abuf) + (uint32_t)g * tc_lbo(rows) +
                                        (uint32_t)(r >> 3) * 128u + (uint32_t)(r & 7) * 16u;
#pragma unroll
                        for (int i = 0; i < kTcDigits; ++i)
                            *reinterpret_cast<uint4 *>(base + (uint32_t)i * tc_plane(rows)) = dg[i];
                    }
                }
                if (!GRAM) {
                    // the right operand's prepared planes for this stage
                    const int sidx = (k0 - w.kb) / kTcStageK;
                    const uint4 *src = reinterpret_cast<const uint4 *>(
                        a.bplanes + ((size_t)w.nt * a.nstages + sidx) * L::b_bytes);
                    uint4 *dst = reinterpret_cast<uint4 *>(bbuf);
                    for (int i = p; i < (int)(L::b_bytes / 16); i += kTcProdThreads)
                        dst[i] = __ldg(src + i);
                }
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                mbar_arrive(&full[s]);
            }
            if (!ok || !has_next) break;
            // the next super-chunk's exponent fields are complete
            prod_sync();
            mbar_arrive(&exfull[b1]);
            it = it1;
            w = w1;
            sk = sk1;
            ++j;
        }
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

// Right operand of a linear combination (C, K x N, element (k, c) at
// C[k + c ldc]) prepared once per call: block (super-chunk, n tile) writes the
// exponent fields of its BN columns and the digit planes of each 32-k stage
// of the super-chunk in the stage layout of the product kernel.
template <int BN>
__global__ void __launch_bounds__(256) k_tc_bprep(const double *__restrict__ C, size_t ldc, int N,
                                                  int K, int super_k, uint8_t *__restrict__ planes,
                                                  int *__restrict__ exps, int nstages, int nsup) {
    using L = TcLayout<BN>;
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
        uint8_t *dst = planes + ((size_t)nt * nstages + k0 / kTcStageK) * L::b_bytes;
        for (int item = threadIdx.x; item < BN * kTcKGroups; item += 256) {
            const int c = item % BN, g = item / BN;
            const int gc = nt * BN + c, k = k0 + g * 8;
            double v[8];
#pragma unroll
            for (int q = 0; q < 8; ++q)
                v[q] = (gc < N && k + q < ske) ? C[k + q + (size_t)gc * ldc] : 0.0;
            uint4 dg[kTcDigits];
            tc_digits8(v, em_s[c], dg);
            uint8_t *base = dst + (uint32_t)g * tc_lbo(BN) + (uint32_t)(c >> 3) * 128u +
                            (uint32_t)(c & 7) * 16u;
#pragma unroll
            for (int i = 0; i < kTcDigits; ++i)
                *reinterpret_cast<uint4 *>(base + (uint32_t)i * tc_plane(BN)) = dg[i];
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

constexpr int kTcSuperGram = 4 * kTcDrainK;     // 384
constexpr int kTcSuperLincomb = 5 * kTcDrainK;  // 480: K up to 480 in one super-chunk

template <int BN, bool GRAM>
void launch_tc(const TcArgs &a, int grid, cudaStream_t st) {
    using L = TcLayout<BN>;
    static PerDevice<bool> smem_set;
    smem_set.get([] {
        GCGE_CUDA(cudaFuncSetAttribute(k_tc_digits<BN, GRAM>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L::bytes));
        return true;
    });
    k_tc_digits<BN, GRAM><<<grid, kTcThreads, L::bytes, st>>>(a);
    GCGE_CHECK_LAUNCH();
    count_launch();
}

template <bool GRAM>
void launch_tc_bn(const TcArgs &a, int bn, int grid, cudaStream_t st) {
    switch (bn) {
        case 16: launch_tc<16, GRAM>(a, grid, st); break;
        case 32: launch_tc<32, GRAM>(a, grid, st); break;
        default: launch_tc<48, GRAM>(a, grid, st); break;
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

size_t tc_bprep_bytes(int k, int m) {
    const int bn = tc_bn(m);
    const size_t nt = (size_t)(m + bn - 1) / bn;
    const size_t nst = (size_t)(k + kTcStageK - 1) / kTcStageK;
    const size_t nsup = (size_t)(k + kTcSuperLincomb - 1) / kTcSuperLincomb;
    const size_t bb = tc_tile_bytes(bn);
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
        return (major == 10 && minor == 3) ? 1 : 0;
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
// in scratch (scratch_elems doubles), then a fixed-order sum.
void tc_gram(int n, int m, int w, const double *Q, int ldq, const double *P, int ldp, double *C,
             int ldc, double *scratch, size_t scratch_elems, cudaStream_t st) {
    if (m <= 0 || w <= 0) return;
    if (n <= 0) {
        GCGE_CUDA(cudaMemset2DAsync(C, sizeof(double) * ldc, 0, sizeof(double) * m, w, st));
        return;
    }
    const int bn = tc_bn(w);
    TcArgs a{};
    a.M = m;
    a.N = w;
    a.K = n;
    a.A = Q;
    a.lda = (size_t)ldq;
    a.B = P;
    a.ldb = (size_t)ldp;
    a.super_k = kTcSuperGram;
    a.mtiles = (m + kTcM - 1) / kTcM;
    a.ntiles = (w + bn - 1) / bn;
    const int mn = a.mtiles * a.ntiles;
    const int sms = device_sms();
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
    launch_tc_bn<true>(a, bn, std::min(a.items, sms), st);
    const int tot = m * w;
    k_tc_reduce<<<(tot + 31) / 32, 256, 0, st>>>(scratch, z, m, w, C, ldc);
    GCGE_CHECK_LAUNCH();
    count_launch();
}

size_t tc_lincomb_scratch_bytes(int k, int m) { return tc_bprep_bytes(k, m); }

// Y (n x m, ldy) = alpha X C + Y diag(beta) for X n x k (ldx), C k x m (ldc);
// beta == nullptr overwrites Y; incb == 0 broadcasts beta[0].
void tc_lincomb(int n, int k, int m, const double *X, int ldx, const double *C, int ldc, double *Y,
                int ldy, const double *beta_dev, int incb, cudaStream_t st, double alpha,
                void *scratch, size_t scratch_bytes) {
    if (n <= 0 || m <= 0) return;
    const int bn = tc_bn(m);
    GCGE_REQUIRE(scratch && scratch_bytes >= tc_bprep_bytes(k, m), GCGE_ERR_ARG,
                 "tc_lincomb: scratch too small");
    TcArgs a{};
    a.M = n;
    a.N = m;
    a.K = k;
    a.A = X;
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
    a.nstages = (k + kTcStageK - 1) / kTcStageK;
    a.nsup = (k + kTcSuperLincomb - 1) / kTcSuperLincomb;
    a.error = tc_error_word();
    uint8_t *planes = static_cast<uint8_t *>(scratch);
    const size_t pbytes = (size_t)a.ntiles * a.nstages * tc_tile_bytes(bn);
    int *exps = reinterpret_cast<int *>(
        (reinterpret_cast<uintptr_t>(planes + pbytes) + 255) & ~(uintptr_t)255);
    const dim3 pg(a.nsup, a.ntiles);
    switch (bn) {
        case 16: k_tc_bprep<16><<<pg, 256, 0, st>>>(C, (size_t)ldc, m, k, kTcSuperLincomb, planes, exps, a.nstages, a.nsup); break;
        case 32: k_tc_bprep<32><<<pg, 256, 0, st>>>(C, (size_t)ldc, m, k, kTcSuperLincomb, planes, exps, a.nstages, a.nsup); break;
        default: k_tc_bprep<48><<<pg, 256, 0, st>>>(C, (size_t)ldc, m, k, kTcSuperLincomb, planes, exps, a.nstages, a.nsup); break;
    }
    GCGE_CHECK_LAUNCH();
    count_launch();
    a.bplanes = planes;
    a.bexps = exps;
    launch_tc_bn<false>(a, bn, std::min(a.items, device_sms()), st);
}

}  // namespace gcge
