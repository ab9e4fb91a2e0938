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
// starting from x; R, P, W are n x k work blocks with leading dimension ld.
// Returns the number of iterations run (<= max_iter).
template <typename T>
int block_pcg(PcgWork &wk, const SellPattern &pat, const T *sval, const T *B, int ldb, T *X,
              int ldx, T *R, T *P, T *W, int ld, int k, int max_iter, double rate, double tol,
              bool rel_tol, cudaStream_t st);

}  // namespace gcge
