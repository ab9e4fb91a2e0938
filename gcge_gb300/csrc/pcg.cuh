// Block conjugate gradient of the W step (pcg.cu).
#pragma once
#include "common.cuh"

namespace gcge {

constexpr int kPcgMaxCols = 64;

// Per-column state of one block-PCG solve, resident in device memory.
struct PcgScalars {
    double rho1[kPcgMaxCols], rho2[kPcgMaxCols], ptw[kPcgMaxCols], alpha[kPcgMaxCols];
    double beta[kPcgMaxCols], init_res[kPcgMaxCols], last_res[kPcgMaxCols];
    double norm_b[kPcgMaxCols];
    int active[kPcgMaxCols];
    // iteration (1-based) in which a column left, 0 if it never iterated:
    // with every column gone, the reference's residual field names the first
    // column that entered the last iteration (src/ops_lin_sol.c:406-410)
    int left_at[kPcgMaxCols];
    int nactive;
    int niter;
};

// Grid barrier state of the persistent solve kernel (zeroed before each
// launch) and counters that accumulate over launches.
struct PcgSync {
    unsigned long long arrive;   // block arrivals at barriers, over the launch
    unsigned long long release;  // number of the last barrier released
    unsigned long long t_spmm;   // globaltimer at the start of the SpMM phase
    int error;                   // a barrier wait ran out of time
    int pad;
};
struct PcgStats {
    double kernel_bytes;         // algorithmic bytes of the whole solves
    double spmm_bytes;           // algorithmic bytes of their SpMM phases
    unsigned long long spmm_ns;  // summed SpMM phase time (device clock)
    unsigned long long iters;    // summed iterations
    unsigned long long launches;
    int error;                   // sticky: some launch's barrier timed out
    int pad;
};

struct PcgWork {
    int kmax = 0;
    DevBuf<double> part;
    DevBuf<PcgScalars> sc;
    DevBuf<PcgSync> sync;
    DevBuf<PcgStats> stats;
    PinnedBuf<PcgScalars> h_sc;
    PinnedBuf<PcgStats> h_stats;
    // whole-kernel timing (event pairs) and algorithmic bytes of the solves
    std::vector<cudaEvent_t> ev;
    size_t ev_used = 0;
    int launches = 0;
    void reserve(int n, int kmax);
    void timing_reset(cudaStream_t st);
    // synchronises; fills the totals below and throws if a barrier timed out
    void collect(cudaStream_t st);
    double kernel_ms = 0.0, spmm_ms = 0.0, kernel_bytes = 0.0, spmm_bytes = 0.0;
    long long total_iters = 0;
    ~PcgWork();
};

// Solve S x = b column-wise (S on the SELL pattern `pat` with values sval)
// starting from x (or from 0 when x_zero, in which case x need not be
// initialised).  B, X, R, P, W are slice-blocked n x kp blocks
// (pcg_block_elems; padding rows and columns of B and X zero).  One persistent launch runs the
// whole iteration; the iteration count and any error stay on the device
// (PcgWork::collect, or pcg_last_iters after a synchronisation).
template <typename T>
void block_pcg_rows(PcgWork &wk, const SellPattern &pat, const T *sval, const T *B, T *X, T *R,
                    T *P, T *W, int kp, int k, int max_iter, double rate, double tol, bool rel_tol,
                    bool x_zero, cudaStream_t st);
// Iterations of the last solve (synchronises the stream).  A barrier wait
// that ran out in that solve throws GCGE_ERR_CUDA (and is cleared, so the
// work area's next solve starts clean).
int pcg_last_iters(PcgWork &wk, cudaStream_t st);

// Failure-detection test of the grid barrier (this thread's launches only):
// a short wait bound, and the grid's last block leaving before its first
// barrier so that the others' waits run out.  Inactive by default.
struct PcgBarrierTest {
    bool active = false;
    unsigned long long timeout_ns = 0;
    int withhold_last = 0;
};
extern thread_local PcgBarrierTest t_pcg_barrier_test;

// Elements of a slice-blocked n x kp block (rows padded to a multiple of 32).
inline size_t pcg_block_elems(int n, int kp) { return (size_t)((n + 31) / 32) * 32 * kp; }

// Column-major (ld) <-> slice-blocked (kp) block conversions (pcg.cu).
template <typename S, typename T>
void col_to_rows(int n, int k, int kp, const S *X, int ldx, T *Y, cudaStream_t st);
template <typename T, typename D>
void rows_to_col(int n, int k, int kp, const T *X, D *Y, int ldy, bool add, cudaStream_t st);

}  // namespace gcge
