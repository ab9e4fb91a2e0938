// Dense symmetric eigensolver of the Rayleigh-Ritz step (eig.cu).
#pragma once
#include "common.cuh"

namespace gcge {

struct EigWork {
    int cap = 0;
    int max_rounds = 0;
    DevBuf<double> G, W, S, C, X, X2, lam, delta, gscr;
    DevBuf<float4> log;  // rotation log: (c, s, p, q as int bits) per pair and round
    DevBuf<unsigned char> ozb;  // right-operand digit planes of the emulated products
    DevBuf<int> info;
    PinnedBuf<double> h_S, h_C, h_lam, h_info;
    double last_delta = 0, last_orth = 0;
    int last_rounds = 0, last_sweeps = 0, last_steps = 0;
    void reserve(int smax);
};

size_t jacobi_smem_bytes(int s);
int jacobi_max_dim();

// Eigenpairs of a small symmetric n x n matrix G on the host (column-major):
// ascending eigenvalues w, orthonormal eigenvectors in the columns of V
// (column-major n x n).  FP64 cyclic Jacobi; an exactly zero row of G gives an
// exactly zero eigenvalue.
void host_eigh(int n, const double *G, double *w, double *V);

// Eigenpairs of the symmetric s x s matrix M (device, leading dim ld):
// ascending eigenvalues to eval_host, orthonormal eigenvectors to Z
// (device, ldz).  refine_steps Ogita-Aishima steps follow the FP32 Jacobi;
// with `emulated` their s x s products run on the FP64-accurate digit-plane
// tensor-core kernels instead of the FP64 units.
int sym_eig(EigWork &wk, int s, const double *M, int ld, double *eval_host, double *Z, int ldz,
            int refine_steps, cudaStream_t st, bool emulated = false);

}  // namespace gcge
