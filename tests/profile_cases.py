"""Single-kernel cases for profiling, at the shapes of the benchmark solve
(n = 262144 rows, the 64^3 generalized problem: nev_max + 2 bs = 200 basis
columns, blocks of bs = 20).

    python tests/profile_cases.py gram      # Q^T P, Q n x 180, P n x 20
    python tests/profile_cases.py lincomb   # X C, X n x 180, C 180 x 20
    python tests/profile_cases.py both
    python tests/profile_cases.py pcg       # FP32 block PCG, 20 columns, 30 steps
    python tests/profile_cases.py eig       # dense eigensolver, s = 200
    python tests/profile_cases.py pcgsmall  # FP32 block PCG, 2D n = 4160 (cluster form)
    python tests/profile_cases.py pcg128    # FP32 block PCG, 128^3 variable coefficient, 40 columns

Each case runs the FP64-accurate digit-plane product once after one warm-up
call, through the same C-ABI entry points the parity tests use
(GCGE_DenseGram / GCGE_DenseLinComb), and checks the result against the FP64
kernel's.  Under ncu, select the product kernel with -k regex:k_oz_gemm.

The pcg case runs the persistent FP32 block PCG of the W step (30 CG steps,
no early stop) on the shifted generalized 64^3 operator A + sigma B through
GCGE_BlockPCG, once after one warm-up call, and checks that the residual
dropped; select it with -k regex:k_block_pcg.

The pcgsmall case runs the same solve on a batch-sized operator (anisotropic
2D 64 x 65, diagonal B, n = 4160, 130 slices), which the library runs in the
kernel's cluster form (one thread-block cluster, hardware barrier).

The eig case runs the dense eigensolver of the Rayleigh-Ritz step
(GCGE_DenseEig) on a 200 x 200 matrix shaped like a late GCG projection (a
diagonal block of 160 Ritz values with double eigenvalues, coupled weakly to a
dense 40 x 40 block) and checks it against numpy; the FP32 Jacobi kernel is
k_jacobi32_cluster.
"""
from __future__ import annotations

import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import gcge_gb300 as G  # noqa: E402

N, M, W = 262144, 180, 20


def _data(seed):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((N, M)), rng.standard_normal((N, W))


def gram():
    Q, P = _data(1)
    G.dense_gram(Q, P, emulated=True)
    C = G.dense_gram(Q, P, emulated=True)
    ref = G.dense_gram(Q, P, emulated=False)
    err = float(np.max(np.abs(C - ref)) / np.max(np.abs(Q).T @ np.abs(P)))
    print(f"gram n={N} m={M} w={W}: max |emulated - fp64| / max(|Q|^T |P|) = {err:.2e}")
    return err < 1e-14


def lincomb():
    X, _ = _data(2)
    C = np.random.default_rng(3).standard_normal((M, W))
    Y0 = np.zeros((N, W))
    G.dense_lincomb(X, C, Y0, emulated=True)
    Y = G.dense_lincomb(X, C, Y0, emulated=True)
    ref = G.dense_lincomb(X, C, Y0, emulated=False)
    err = float(np.max(np.abs(Y - ref)) / np.max(np.abs(X) @ np.abs(C)))
    print(f"lincomb n={N} k={M} m={W}: max |emulated - fp64| / max(|X| |C|) = {err:.2e}")
    return err < 1e-14


def pcg():
    from gcge_gb300 import problems as Pr
    A, B = Pr.laplace3d(64), Pr.mass3d(64)
    b = np.random.default_rng(4).standard_normal((A.n, W))
    x0 = np.zeros_like(b)
    sigma = 10.0
    G.block_pcg(A, B, sigma, b, x0, max_iter=30, rate=1e-30, tol=1e-30, fp32=True)
    x, it = G.block_pcg(A, B, sigma, b, x0, max_iter=30, rate=1e-30, tol=1e-30, fp32=True)
    S = A.to_scipy() + sigma * B.to_scipy()
    red = float(np.max(np.linalg.norm(b - S @ x, axis=0) / np.linalg.norm(b, axis=0)))
    print(f"pcg n={A.n} k={W} steps={it}: max relative residual {red:.2e}")
    return it == 30 and red < 0.5


def pcg128():
    """The W-step PCG of the benchmark solve's shape: the variable-coefficient
    128^3 operator with its lumped diagonal mass, 40 right-hand sides, 30
    FP32 steps without early stop (k_block_pcg<float, 40>)."""
    from gcge_gb300 import problems as Pr
    A, B = Pr.vardiff3d(128)
    b = np.random.default_rng(4).standard_normal((A.n, 40))
    x0 = np.zeros_like(b)
    sigma = 1.0
    G.block_pcg(A, B, sigma, b, x0, max_iter=30, rate=1e-30, tol=1e-30, fp32=True)
    x, it = G.block_pcg(A, B, sigma, b, x0, max_iter=30, rate=1e-30, tol=1e-30, fp32=True)
    S = A.to_scipy() + sigma * B.to_scipy()
    red = float(np.max(np.linalg.norm(b - S @ x, axis=0) / np.linalg.norm(b, axis=0)))
    print(f"pcg n={A.n} k=40 steps={it}: max relative residual {red:.2e}")
    return it == 30 and red < 1.0


def pcgsmall():
    from gcge_gb300 import problems as Pr
    A = Pr.aniso2d(64, 65, 2.31)
    B = Pr.diag_matrix(0.5 + 1.5 * Pr.splitmix_uniform(7, A.n, 0))
    b = np.random.default_rng(4).standard_normal((A.n, W))
    x0 = np.zeros_like(b)
    sigma = 0.01
    G.block_pcg(A, B, sigma, b, x0, max_iter=30, rate=1e-30, tol=1e-30, fp32=True)
    x, it = G.block_pcg(A, B, sigma, b, x0, max_iter=30, rate=1e-30, tol=1e-30, fp32=True)
    S = A.to_scipy() + sigma * B.to_scipy()
    red = float(np.max(np.linalg.norm(b - S @ x, axis=0) / np.linalg.norm(b, axis=0)))
    print(f"pcg n={A.n} k={W} steps={it}: max relative residual {red:.2e}")
    return it == 30 and red < 0.5


def eig():
    rng = np.random.default_rng(5)
    d = np.sort(rng.uniform(1.0, 100.0, 160))
    d[10:13] = d[10]
    M = np.zeros((200, 200))
    M[:160, :160] = np.diag(d)
    Cw = 1e-3 * rng.standard_normal((160, 40))
    M[:160, 160:] = Cw
    M[160:, :160] = Cw.T
    Wm = rng.standard_normal((40, 40))
    M[160:, 160:] = 150.0 + 10.0 * (Wm + Wm.T)
    G.dense_eig(M)
    ev, Z = G.dense_eig(M)
    ref = np.linalg.eigvalsh(M)
    err = float(np.max(np.abs(ev - ref)) / np.abs(ref).max())
    res = float(np.abs(M @ Z - Z * ev).max() / np.abs(ref).max())
    print(f"eig s=200: eigenvalue error {err:.1e}, residual {res:.1e}")
    return err < 1e-13 and res < 1e-12


# long-dimension product shapes of the mixed solves: (kind, n, m, w)
PROD_SHAPES = [("gram", 262144, 180, 20), ("lincomb", 262144, 180, 20),
               ("gram", 2097152, 360, 40), ("lincomb", 2097152, 360, 40),
               ("gram", 2097152, 400, 40), ("lincomb", 2097152, 400, 320),
               ("gram", 2097152, 320, 40), ("gram", 2097152, 40, 40),
               ("lincomb", 2097152, 400, 200), ("lincomb", 2097152, 80, 40)]


def prodbench():
    """CUDA-event time of each product shape, digit kernels and FP64 kernels,
    with its algorithmic bytes (8 n (m + w) for a Gram, 8 n (m + 2 w) for a
    linear combination) over the measured HBM peak."""
    import json
    try:
        with open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                               "MEASURED_PEAKS.json")) as f:
            peak = float(json.load(f)["hbm_gbs"])
    except Exception:
        peak = 6800.0
    for kind, n, m, w in PROD_SHAPES:
        emu = G.bench_dense_product(kind, n, m, w, emulated=True, reps=5)
        f64 = G.bench_dense_product(kind, n, m, w, emulated=False, reps=2)
        byts = 8.0 * n * (m + w) if kind == "gram" else 8.0 * n * (m + 2 * w)
        print(f"{kind} n={n} m={m} w={w}: digits {emu:.3f} ms ({byts / emu / 1e6:.0f} GB/s, "
              f"{byts / emu / 1e6 / peak:.3f} of HBM), fp64 {f64:.3f} ms", flush=True)
    return True


def tcgram():
    """One Gram product of the tensor-core digit kernel at n = 524288, 360 x 40
    (Q 1.5 GB, larger than L2), after one warm-up call: the shape of the 128^3
    B-orthogonalisation at a quarter of its length, for a profiler capture of
    k_tc_digits (second launch)."""
    ms = G.bench_dense_product("gram", 524288, 360, 40, emulated=True, reps=1)
    print(f"gram n=524288 m=360 w=40: digits {ms:.3f} ms")
    return True


def main(argv):
    what = argv[1] if len(argv) > 1 else "both"
    ok = True
    if what == "prodbench":
        ok &= prodbench()
    if what == "tcgram":
        ok &= tcgram()
    if what in ("gram", "both"):
        ok &= gram()
    if what in ("lincomb", "both"):
        ok &= lincomb()
    if what == "pcg":
        ok &= pcg()
    if what == "eig":
        ok &= eig()
    if what == "pcgsmall":
        ok &= pcgsmall()
    if what == "pcg128":
        ok &= pcg128()
    return 0 if ok else 1


if __name__ == "__main__":
    sys.exit(main(sys.argv))
