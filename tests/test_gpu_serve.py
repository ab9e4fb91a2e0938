"""Many solves on one GPU (serve.cu): batched independent problems of uneven n
and nev, and requests arriving while others run.  Each result must equal the
same problem solved alone (up to rounding of the shared PCG grid) and the
dense generalized eigensolver's; the memory budget must serialise admission
when it is too small for two solves at once."""
import time

import numpy as np
import pytest

from gcge_gb300 import problems as P

pytestmark = pytest.mark.gpu


def small_batch(count, seed):
    return P.batch_problems(count=count, seed=seed, nx_range=(20, 40), nev_range=(6, 14))


def job_for(G, c, precision=None):
    return G.Job(c["A"], c["B"], c["nev"], c["block_size"], c["nev_init"], c["nev_max"],
                 X0=P.initial_block(c["A"].n, c["nev_init"], seed=1),
                 precision=G.PREC_MIXED if precision is None else precision)


def alone(G, c, precision=None):
    return G.solve(c["A"], c["B"], c["nev"], c["block_size"], c["nev_init"], c["nev_max"],
                   X0=P.initial_block(c["A"].n, c["nev_init"], seed=1),
                   precision=G.PREC_MIXED if precision is None else precision, want_evec=False)


def test_batch_matches_single_solves_and_dense_reference(gpu_lib):
    G = gpu_lib
    probs = small_batch(8, seed=21)
    jobs = [job_for(G, c, G.PREC_MIXED if i % 2 == 0 else G.PREC_FP64) for i, c in enumerate(probs)]
    res = G.solve_batch(jobs, workers=4)
    import scipy.linalg as sl
    for i, (c, r) in enumerate(zip(probs, res)):
        nev = c["nev"]
        assert r.status == G.GCGE_OK and r.nconv >= nev, (c["name"], r.status, r.nconv)
        ref = alone(G, c, G.PREC_MIXED if i % 2 == 0 else G.PREC_FP64)
        np.testing.assert_allclose(r.eval[:nev], ref.eval[:nev], rtol=1e-10, atol=0)
        if i < 3:
            w = sl.eigh(c["A"].to_scipy().toarray(), c["B"].to_scipy().toarray(),
                        eigvals_only=True, subset_by_index=[0, nev - 1])
            np.testing.assert_allclose(r.eval[:nev], w, rtol=1e-9, atol=0)


def test_server_staggered_arrivals_match_alone(gpu_lib):
    G = gpu_lib
    probs = small_batch(6, seed=22)
    with G.Server(workers=3) as srv:
        jobs = []
        for c in probs:
            jobs.append(srv.submit(job_for(G, c)))
            time.sleep(0.01)
        results = [srv.wait(j) for j in jobs]
    for c, j, r in zip(probs, jobs, results):
        nev = c["nev"]
        assert r.status == G.GCGE_OK and r.nconv >= nev
        q = j.req
        assert q.t_submit <= q.t_start <= q.t_end and j.latency > 0
        np.testing.assert_allclose(r.eval[:nev], alone(G, c).eval[:nev], rtol=1e-10, atol=0)


def test_server_budget_serialises_admission(gpu_lib):
    G = gpu_lib
    probs = small_batch(4, seed=23)
    with G.Server(workers=3, budget_bytes=1) as srv:   # nothing fits beside another solve
        jobs = [srv.submit(job_for(G, c)) for c in probs]
        for j in jobs:
            assert srv.wait(j).status == G.GCGE_OK
    spans = sorted((j.req.t_start, j.req.t_end) for j in jobs)
    for (s0, e0), (s1, e1) in zip(spans, spans[1:]):
        assert s1 >= e0 - 1e-3, spans   # one at a time
