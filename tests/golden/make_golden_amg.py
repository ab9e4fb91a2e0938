"""Generate the block AMG fixtures from the reference GCGE CPU path.

The reference's BlockAMG (MultiLinearSolverSetup_BlockAMG and the V-cycle it
installs, src/ops_lin_sol.c:466-715) runs from its own C sources compiled
into oracle/_ref/libgcge_ref.so (oracle/ref/Makefile) on the app_ccs backend.
No backend of the reference fills ops->MultiVecFromItoJ, which the V-cycle
calls to move residuals and corrections between levels, so the driver
(oracle/ref/ref_driver.c, ref_block_amg) supplies one that multiplies by P_l^T
and P_l with app_ccs's own MatDotMultiVec.  The hierarchies are
problems.multigrid_2d (linear interpolation, Galerkin coarse operators).

    make -C oracle/ref && OPENBLAS_NUM_THREADS=1 python tests/golden/make_golden_amg.py

Writes golden_amg.json (parameters and the solver's residual field) and
golden_amg.npz (the solutions x) beside this file.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from gcge_gb300 import problems as P  # noqa: E402


def cases():
    """name -> dict(grid, levels, k, seed, x0_random, max_iter, rate, tol, tol_type).

    fixed: rate 0 and tol 0, so every smoothing solve runs its full iteration
    cap and the result is a fixed polynomial in b (no stopping decisions);
    abs / rel: the stopping rules of the level solves and of the cycles;
    wide: 48 columns (more than one 40-column block of the GPU solve)."""
    return {
        "lap2d_63_L3_fixed": dict(grid=63, levels=3, k=4, seed=11, x0_random=False,
                                  max_iter=[2, 3, 3, 3, 3, 20], rate=[0.0] * 3, tol=[0.0] * 3,
                                  tol_type="abs"),
        "lap2d_63_L3_abs": dict(grid=63, levels=3, k=4, seed=11, x0_random=False,
                                max_iter=[30, 2, 2, 2, 2, 30], rate=[1e-2] * 3,
                                tol=[1e-9, 1e-12, 1e-12], tol_type="abs"),
        "lap2d_127_L4_rel": dict(grid=127, levels=4, k=8, seed=12, x0_random=True,
                                 max_iter=[30, 2, 2, 2, 2, 2, 2, 40], rate=[1e-2] * 4,
                                 tol=[1e-10] * 4, tol_type="rel"),
        "lap2d_31_L2_wide": dict(grid=31, levels=2, k=48, seed=13, x0_random=False,
                                 max_iter=[3, 2, 2, 25], rate=[0.0] * 2, tol=[0.0] * 2,
                                 tol_type="abs"),
    }


def inputs(c):
    """The hierarchy, b and x0 of a case (seeded; identical on every machine)."""
    A, T = P.multigrid_2d(c["grid"], c["grid"], c["levels"])
    n, k = A[0].n, c["k"]
    b = (P.splitmix_uniform(c["seed"], n * k, 0) - 0.5).reshape((n, k), order="F")
    if c["x0_random"]:
        x0 = (P.splitmix_uniform(c["seed"], n * k, 1) - 0.5).reshape((n, k), order="F")
    else:
        x0 = np.zeros((n, k), order="F")
    return A, T, np.asfortranarray(b), np.asfortranarray(x0)


def main():
    from oracle import ref_lib
    if not ref_lib.available():
        raise SystemExit("oracle/_ref/libgcge_ref.so is missing: make -C oracle/ref")
    meta, arrays = {}, {}
    for name, c in cases().items():
        A, T, b, x0 = inputs(c)
        x, res = ref_lib.ref_block_amg(A, T, b, x0, c["max_iter"], c["rate"], c["tol"],
                                       c["tol_type"])
        meta[name] = dict(c, n=[a.n for a in A], residual=res)
        arrays[name] = x
        print(name, [a.n for a in A], "residual", res)
    with open(os.path.join(HERE, "golden_amg.json"), "w") as f:
        json.dump(meta, f, indent=1)
    np.savez_compressed(os.path.join(HERE, "golden_amg.npz"), **arrays)


if __name__ == "__main__":
    main()
