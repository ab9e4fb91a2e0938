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
    int nactive;
    int niter;
};

struct PcgWork {
    int kmax = 0;
    DevBuf<double> part;
    DevBuf<PcgScalars> sc;
    PinnedBuf<PcgScalars> h_sc;
    // per-launch timing of the SpMM inside the iterations (event pairs)
    std::vector<cudaEvent_t> ev;
    size_t ev_used = 0;
    double spmm_bytes = 0.0;
    int spmm_launches = 0;
    void reserve(int n, int kmax, int spmm_nblocks);
    void timing_reset();
    double timing_collect_ms();  // synchronises, sums the recorded intervals
    ~PcgWork();
};

// Solve S x = b column-wise (S on the SELL pattern `pat` with values sval)
// starting from x.  B, X, R, P, W are row-interleaved n x kp blocks (row i at
// i*kp, padding columns zero).  Returns the number of iterations run.
template <typename T>
int block_pcg_rows(PcgWork &wk, const SellPattern &pat, const T *sval, const T *B, T *X, T *R,
                   T *P, T *W, int kp, int k, int max_iter, double rate, double tol, bool rel_tol,
                   cudaStream_t st);

// Column-major (ld) <-> row-interleaved (kp) block conversions.
template <typename S, typename T>
void col_to_rows(int n, int k, int kp, const S *X, int ldx, T *Y, cudaStream_t st);
template <typename T, typename D>
void rows_to_col(int n, int k, int kp, const T *X, D *Y, int ldy, bool add, cudaStream_t st);

}  // namespace gcge
