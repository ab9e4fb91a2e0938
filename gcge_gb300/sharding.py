"""Assignment of independent solves to ranks (one GPU per rank).

The batched problems and serving requests are independent units, so several
GPUs share them with no collective on the data path: every rank solves its own
subset and only the timing and the counts are reduced.  Units are assigned by
their estimated device footprint, which also tracks their work per outer
iteration (both scale with n times the basis width), largest first to the
least-loaded rank (the longest-processing-time rule), ties to the lower rank,
so every rank computes the same assignment from the same list.
"""
from __future__ import annotations


def footprint_bytes(n: int, nnz_a: int, nnz_b: int, nev_max: int, block_size: int) -> int:
    """Estimated device bytes of one solve: the basis V = [X P W]
    (n x (nev_max + 2 bs)), the Ritz vectors (n x nev_max), the A x / B x
    blocks and right-hand sides of ComputeW (~4 n x bs), five slice-blocked
    block-PCG vectors (FP64 and FP32), the matrices in SELL-32 (value and
    index per entry, with the union pattern of A and B) and the projected
    problem's dense state."""
    cols = nev_max + 2 * block_size
    s = cols
    vec = 8 * n * (cols + nev_max + 4 * block_size) + 5 * (8 + 4) * n * block_size
    mat = 12 * (nnz_a + nnz_b) * 2 + 12 * (nnz_a + nnz_b + n)
    dense = 8 * 8 * s * s
    return int(vec + mat + dense)


def problem_footprint(c: dict) -> int:
    """footprint_bytes of a problem dict of gcge_gb300.problems (A, B, nev_max, block_size)."""
    A, B = c["A"], c["B"]
    return footprint_bytes(A.n, A.nnz, 0 if B is None else B.nnz, c["nev_max"], c["block_size"])


def shard_by_footprint(weights, world: int):
    """Indices of the units assigned to each of `world` ranks, each rank's
    list in increasing index order (so arrival order is kept)."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(weights)), key=lambda i: (-weights[i], i))
    load = [0] * world
    out = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda j: (load[j], j))
        out[r].append(i)
        load[r] += weights[i]
    return [sorted(x) for x in out]
