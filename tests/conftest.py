import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN_DIR = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden():
    with open(os.path.join(GOLDEN_DIR, "golden.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def golden_vectors():
    return dict(np.load(os.path.join(GOLDEN_DIR, "golden_vectors.npz")))


@pytest.fixture(scope="session")
def golden_vectors_large():
    """Leading eigenvectors (FP32) of the fixtures at the benchmarked sizes."""
    return dict(np.load(os.path.join(GOLDEN_DIR, "golden_vectors_large.npz")))


@pytest.fixture(scope="session")
def golden_orth():
    with open(os.path.join(GOLDEN_DIR, "golden_orth.json")) as f:
        meta = json.load(f)
    meta["arrays"] = dict(np.load(os.path.join(GOLDEN_DIR, "golden_orth.npz")))
    return meta


def orth_case(name):
    """Inputs of an orthogonalisation fixture (tests/golden/orth_cases.py)."""
    if GOLDEN_DIR not in sys.path:
        sys.path.insert(0, GOLDEN_DIR)
    import orth_cases
    return orth_cases.build(name)


def orth_solve_case(name):
    """The generator call of each bgs / ComputeW12 solve fixture (make_golden_orth.py)."""
    if GOLDEN_DIR not in sys.path:
        sys.path.insert(0, GOLDEN_DIR)
    from make_golden_orth import solve_cases
    return solve_cases()[name][0]()


def b_projector(X, B):
    """X X^T B: the B-orthogonal projector onto span(X) for B-orthonormal X."""
    return X @ (X if B is None else B @ X).T


def build_case(name):
    """The generator call of each golden case (mirrors tests/golden/make_golden.py)."""
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    from make_golden import cases
    builder = cases()[name][0]
    return builder()


@pytest.fixture(scope="session")
def gpu_lib():
    import gcge_gb300 as G
    G.load()
    return G


def cluster_subspace_angle(evals, V1, V2, B=None, rel_gap=1e-6):
    """Largest principal angle (radians) between V1 and V2 over clusters of
    nearly equal eigenvalues (subspaces are compared cluster by cluster, so
    degenerate eigenvalues do not need matching eigenvectors).  Columns are
    B-orthonormal; the angle is measured in the B inner product."""
    k = V1.shape[1]
    worst = 0.0
    i = 0
    BV2 = V2 if B is None else B @ V2
    while i < k:
        j = i + 1
        while j < k and abs(evals[j] - evals[j - 1]) <= rel_gap * abs(evals[j]):
            j += 1
        if j == k and i > 0 and j - i > 0:
            pass
        C = V1[:, i:j].T @ BV2[:, i:j]
        s = np.linalg.svd(C, compute_uv=False)
        worst = max(worst, float(np.arccos(np.clip(s.min(), -1.0, 1.0))))
        i = j
    return worst


def cluster_subspace_sine(evals, V1, V2, B=None, rel_gap=1e-6):
    """Largest sine of the principal angles between span(V1) and span(V2) over
    clusters of nearly equal eigenvalues, in the B inner product.  V1 is
    B-orthonormal; each cluster block of V2 is B-orthonormalised first (V2 may
    be stored in FP32), and the sine is the norm of the part of that block
    outside span(V1) - stable for small angles, where arccos of a cosine near 1
    is not."""
    k = V1.shape[1]
    V2 = np.asarray(V2, dtype=np.float64)
    worst = 0.0
    i = 0
    while i < k:
        j = i + 1
        while j < k and abs(evals[j] - evals[j - 1]) <= rel_gap * abs(evals[j]):
            j += 1
        Q = V2[:, i:j]
        BQ = Q if B is None else B @ Q
        L = np.linalg.cholesky(Q.T @ BQ)
        Q = np.linalg.solve(L, Q.T).T
        BQ = np.linalg.solve(L, BQ.T).T
        V = V1[:, i:j]
        R = Q - V @ (V.T @ BQ)
        BR = R if B is None else B @ R
        s = float(np.sqrt(max(0.0, np.linalg.eigvalsh(R.T @ BR).max())))
        worst = max(worst, s)
        i = j
    return worst
