"""The SpMM column-split autotuner (gcge_gb300/csrc/spmm.cu): whichever split
it picks, SpMM results are bitwise those of the fixed 40-column launches (each
column's sum runs over the same entries in the same order), the choice is one
of the candidates, and a GCG solve with tuning on matches the reference's
eigenvalues as the untuned solve does."""
import numpy as np
import pytest

from conftest import build_case
from gcge_gb300 import problems as P

pytestmark = pytest.mark.gpu


@pytest.fixture()
def tuning(gpu_lib):
    gpu_lib.set_spmm_tuning(-1)
    yield gpu_lib
    gpu_lib.set_spmm_tuning(-1)


@pytest.mark.parametrize("k", [40, 33, 17, 9])
def test_tuned_split_is_bitwise_the_fixed_one(tuning, k):
    G = tuning
    A, _ = P.vardiff3d(14)
    rng = np.random.default_rng(k)
    X = rng.standard_normal((A.n, k))
    ops = G.CudaOps()
    try:
        h = ops.mat(A)
        x = ops.multivec(h, k, X)
        y0 = ops.multivec(h, k)
        y1 = ops.multivec(h, k)
        ops.mat_dot(h, x, y0, (0, 0), (k, k))
        fixed = ops.download(y0, 0, k)
        G.set_spmm_tuning(1)
        ops.mat_dot(h, x, y1, (0, 0), (k, k))      # tunes, then multiplies
        tuned = ops.download(y1, 0, k)
        ops.mat_dot(h, x, y1, (0, 0), (k, k))      # the kept choice
        again = ops.download(y1, 0, k)
    finally:
        ops.close()
    assert np.array_equal(tuned, fixed)
    assert np.array_equal(again, fixed)
    np.testing.assert_allclose(fixed, A.to_scipy() @ X, rtol=0, atol=1e-11)


@pytest.mark.parametrize("fp32", [False, True])
def test_tuner_times_every_candidate(tuning, fp32):
    G = tuning
    A = P.laplace3d(40)
    chunk, ms = G.spmm_tune(A, 40, fp32)
    cands = G.spmm_tune_candidates(40)
    assert cands == [40, 20, 14, 8]
    assert sorted(ms) == sorted(cands)
    assert chunk in cands
    assert all(t > 0 for t in ms.values())
    # the chosen split is within 2% of the fastest or faster than the wider ones
    assert ms[chunk] <= min(ms.values()) / 0.98 + 1e-9
    ms_fixed, _ = G.bench_spmm(A, 40, fp32, reps=5)
    assert ms_fixed > 0


def test_solve_with_tuning_matches_reference(tuning, golden):
    G = tuning
    case = "vardiff3d_12_nev200"          # blocks of 40 columns
    g = golden[case]
    A, B = build_case(case)
    X0 = P.initial_block(A.n, g["nev_init"], seed=g["x0_seed"])
    kw = dict(X0=X0, tol=tuple(g["tol"]), max_iter=g["max_iter"], gap_min=g["gap_min"],
              auto_shift=g["auto_shift"])
    args = (A, B, g["nev"], g["block_size"], g["nev_init"], g["nev_max"])
    r0 = G.solve(*args, **kw)
    G.set_spmm_tuning(1)
    r1 = G.solve(*args, **kw)
    nev = g["nev"]
    ref = np.array(g["eval"][:nev])
    assert r1.status == G.GCGE_OK and r1.nconv >= nev
    rel = np.abs(r1.eval[:nev] - ref) / np.abs(ref)
    assert rel.max() < 1e-10, rel.max()
    np.testing.assert_allclose(r1.eval[:nev], r0.eval[:nev], rtol=1e-12, atol=0)
