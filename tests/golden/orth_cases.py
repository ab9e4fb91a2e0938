"""Inputs of the MultiVecOrth fixtures (binary and modified Gram-Schmidt).

Every input is built from exact operations (SplitMix64 uniforms, Hadamard or
unit-vector prefixes, sums and products of those, correctly rounded square
roots), so the same bits come out on any machine: the fixtures store only the
reference's outputs.

A case is (start, ncols, block_size, B kind, layout, edits) on N rows: the
prefix [0, start) is B-orthonormal, the block [start, start + ncols) is
uniform in [-1/32, 1/32) with the layout's edits:
  "plain"  - no edits (Hadamard prefix),
  "zero"   - the listed columns zero (dropped by every method),
  "dep"    - unit-vector prefix, the listed columns 2 e_0 - e_1: the projection
             against the prefix leaves them exactly zero, so they drop,
  "near"   - the block copies the prefix's columns plus a ~1e-9 perturbation.
Columns that are dependent only up to rounding are left out on purpose: the
reference's drop decision for them compares rounding-level quantities with
the zero tolerance and is not reproducible across summation orders.
"""
from __future__ import annotations

import numpy as np

N = 128

# name -> (start, ncols, block_size, B kind, layout, edits)
CASES = {
    "mleaf_plain": (0, 12, -1, None, "plain", ()),
    "mleaf_prefix_diagB_zero": (8, 10, -1, "diag", "zero", (2, 7)),
    "mleaf_near_prefix": (6, 6, 2, None, "near", ()),
    "mleaf_prefix_dep": (4, 9, -1, "diag", "dep", (0, 5)),
    "evp_plain": (0, 20, -1, None, "plain", ()),
    "evp_prefix_diagB_dep": (6, 32, 4, "diag", "dep", (3, 11, 30)),
    "evp_wide_massB_zero": (0, 64, -1, "mass", "zero", (9, 40, 63)),
    "evp_prefix_zero": (16, 24, 100, None, "zero", (0, 23)),
}


def uniform(seed: int, n: int, k: int) -> np.ndarray:
    from gcge_gb300.problems import splitmix_uniform
    return (2.0 * splitmix_uniform(seed, n * k) - 1.0).reshape((n, k), order="F")


def b_matrix(kind, start=0, n=N):
    """None, a diagonal B (exactly 1 on the first `start` rows), or a
    tridiagonal mass-like B (CSRMatrix)."""
    from gcge_gb300 import problems as P
    if kind is None:
        return None
    if kind == "diag":
        d = 0.5 + P.splitmix_uniform(77, n)
        d[:start] = 1.0
        return P.diag_matrix(d)
    if kind == "mass":
        import scipy.sparse as sp
        m = sp.diags([np.full(n - 1, 1.0), np.full(n, 4.0), np.full(n - 1, 1.0)], [-1, 0, 1]) / 6.0
        return P._from_scipy(m.tocsr())
    raise ValueError(kind)


def build(name: str):
    """(x (N x (start + ncols), column-major), start, end, block_size, B)."""
    from scipy.linalg import hadamard
    start, ncols, bs, bkind, layout, edits = CASES[name]
    assert bkind != "mass" or start == 0
    B = b_matrix(bkind, start if layout == "dep" else 0)
    x = np.zeros((N, start + ncols), order="F")
    if start and layout == "dep":
        x[:start, :start] = np.eye(start)
    elif start:
        h = hadamard(N).astype(np.float64)[:, 1:start + 1] / np.sqrt(float(N))
        if B is not None:   # diagonal B: prefix columns h / sqrt(d)
            h = h / np.sqrt(B.data)[:, None]
        x[:, :start] = h
    # block columns of B-norm about 0.2, so that the Gram matrices of the
    # eigen-decomposition leaves stay near unit scale: their zero eigenvalues
    # then come out well inside the zero tolerance
    blk = uniform(hash_seed(name), N, ncols) * 2.0 ** -5
    if layout == "zero":
        for j in edits:
            blk[:, j] = 0.0
    elif layout == "dep":
        for j in edits:
            blk[:, j] = 2.0 * x[:, 0] - x[:, 1]
    elif layout == "near":
        for j in range(ncols):
            blk[:, j] = x[:, j % start] + 3.2e-8 * blk[:, j]
    x[:, start:] = blk
    return x, start, start + ncols, bs, B


def hash_seed(name: str) -> int:
    h = 1469598103934665603 & 0xFFFFFFFF
    for ch in name.encode():
        h = ((h ^ ch) * 16777619) & 0xFFFFFFFF
    return h
