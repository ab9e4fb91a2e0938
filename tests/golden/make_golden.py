"""Generate the golden fixtures from the reference GCGE CPU path.

Runs the reference's own C sources (compiled by oracle/ref/Makefile into
oracle/_ref/libgcge_ref.so) on seeded problems from gcge_gb300.problems and
stores eigenvalues, converged counts and iteration counts (golden.json) plus
the leading eigenvectors of the small cases (golden_vectors.npz, FP64) and of
the cases at the benchmarked sizes (golden_vectors_large.npz: the leading
columns up to a cluster boundary, stored in FP32, which resolves subspace
angles far below the 1e-6 rad the tests ask for).

    make -C oracle/ref && OPENBLAS_NUM_THREADS=1 python tests/golden/make_golden.py
    OPENBLAS_NUM_THREADS=1 python tests/golden/make_golden.py vardiff3d_12_nev200   # one case

The reference tree must be present; the fixtures it writes are what the
tests use everywhere else (including on machines without the reference).
"""
from __future__ import annotations

import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from gcge_gb300 import problems as P  # noqa: E402
from oracle import ref_lib  # noqa: E402


def cases():
    """name -> (builder, nev, bs, nev_init, nev_max, options, keep_vectors).

    keep_vectors: True stores all nev eigenvectors in FP64; an integer m stores
    the leading columns (at most m, ending at a cluster boundary) in FP32."""
    rule = P.gcge_block_rule
    out = {}
    out["laplace2d_24x24_nev8"] = (lambda: (P.laplace2d(24, 24), None), 8, 4, 12, 20, {}, True)
    out["laplace2d_24x24_noshift"] = (lambda: (P.laplace2d(24, 24), None), 8, 4, 12, 20,
                                      {"auto_shift": 0}, True)
    out["laplace2d_20x20_abstol"] = (lambda: (P.laplace2d(20, 20), None), 6, 6, 12, 12,
                                     {"tol": (1e-7, 1e300)}, True)
    out["laplace2d_128x128_nev20_bs20"] = (lambda: (P.laplace2d(128, 128), None), 20, 20, 40, 40,
                                           {}, False)
    bs, ni, nm = rule(20)
    out["laplace2d_128x128_nev20_rule"] = (lambda: (P.laplace2d(128, 128), None), 20, bs, ni, nm,
                                           {}, False)
    bs, ni, nm = rule(100)
    out["laplace3d_mass_16"] = (lambda: (P.laplace3d(16), P.mass3d(16)), 100, bs, ni, nm, {}, False)
    out["laplace3d_mass_24"] = (lambda: (P.laplace3d(24), P.mass3d(24)), 100, bs, ni, nm, {}, False)
    bs, ni, nm = rule(20)
    out["vardiff3d_12"] = (lambda: P.vardiff3d(12, seed=3), 20, bs, ni, nm, {}, True)
    # the block rule of the 128^3 variable-coefficient workload (nev 200: bs 40,
    # nevInit 120, nevMax 320; projected dimensions up to 400)
    bs, ni, nm = rule(200)
    out["vardiff3d_12_nev200"] = (lambda: P.vardiff3d(12, seed=3), 200, bs, ni, nm, {}, False)
    bs, ni, nm = rule(16)
    out["aniso2d_40x30_eps10_diagB"] = (
        lambda: (P.aniso2d(40, 30, 10.0), P.diag_matrix(0.5 + 1.5 * P.splitmix_uniform(11, 1200, 0))),
        16, bs, ni, nm, {}, True)
    bs, ni, nm = rule(12)
    out["rgg_2000_deg10"] = (lambda: (P.rgg_laplacian(2000, 10.0, seed=5), None), 12, bs, ni, nm, {},
                             True)
    # the benchmarked workloads at full size (64^3 stiffness + Kronecker mass,
    # nev 100) and reduced (32^3), and the 128^3 variable-coefficient operator's
    # generator with the nev-200 block rule at 32^3
    bs, ni, nm = rule(100)
    out["laplace3d_mass_32"] = (lambda: (P.laplace3d(32), P.mass3d(32)), 100, bs, ni, nm, {}, 40)
    out["laplace3d_mass_64"] = (lambda: (P.laplace3d(64), P.mass3d(64)), 100, bs, ni, nm, {},
                                False)
    bs, ni, nm = rule(200)
    out["vardiff3d_32_nev200"] = (lambda: P.vardiff3d(32, seed=3), 200, bs, ni, nm, {}, 48)
    return out


def leading_cluster_cut(ev, m, rel_gap=1e-6):
    """The largest j <= m such that eigenvalues j-1 and j are not in one cluster."""
    j = m
    while j > 1 and abs(ev[j] - ev[j - 1]) <= rel_gap * abs(ev[j]):
        j -= 1
    return j


def main(only=None):
    """All cases, or only the named ones (merged into the existing fixtures)."""
    if not ref_lib.available():
        raise SystemExit("oracle/_ref/libgcge_ref.so missing: run make -C oracle/ref")
    out, vecs, large = {}, {}, {}
    if only:
        with open(os.path.join(HERE, "golden.json")) as f:
            out = json.load(f)
        with np.load(os.path.join(HERE, "golden_vectors.npz")) as z:
            vecs = {k: z[k] for k in z.files}
    large_path = os.path.join(HERE, "golden_vectors_large.npz")
    if os.path.exists(large_path):
        with np.load(large_path) as z:
            large = {k: z[k] for k in z.files}
    for name, (builder, nev, bs, ni, nm, opt, keep) in cases().items():
        if only and name not in only:
            continue
        A, B = builder()
        X0 = P.initial_block(A.n, ni, seed=1)
        tol = opt.get("tol", (1e300, 1e-8))
        shift = opt.get("auto_shift", 1)
        t = time.time()
        ev, evec, nc, it, sec = ref_lib.ref_solve(A, B, X0, nev, bs, ni, nm, tol=tol, max_iter=500,
                                                  gap_min=1e-5, auto_shift=shift)
        print(f"{name}: n={A.n} nconv={nc} niter={it} {time.time() - t:.1f}s", flush=True)
        out[name] = dict(n=A.n, nnz_a=A.nnz, nnz_b=None if B is None else B.nnz, nev=nev,
                         block_size=bs, nev_init=ni, nev_max=nm, tol=list(tol), auto_shift=shift,
                         gap_min=1e-5, max_iter=500, x0_seed=1, nconv=nc, niter=it,
                         eval=[float(v) for v in ev], ref_seconds=sec)
        if keep is True:
            vecs[name] = evec[:, :nev].copy()
        elif keep:
            m = leading_cluster_cut(ev, int(keep))
            large[name] = evec[:, :m].astype(np.float32)
        with open(os.path.join(HERE, "golden.json"), "w") as f:
            json.dump(out, f, indent=1)
        np.savez_compressed(os.path.join(HERE, "golden_vectors.npz"), **vecs)
        np.savez_compressed(large_path, **large)


if __name__ == "__main__":
    main(sys.argv[1:] or None)
