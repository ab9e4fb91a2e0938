"""The multi-process path of bench.py on CPU: two ranks over gloo at
127.0.0.1.  A single problem does not shard (each GPU runs its own replica of
the solve); the batched problems and serving requests are sharded across the
ranks by device footprint with no collective on the data path, so the only
collectives are the benchmark's barrier, its max/sum over ranks and the
gathering of latencies, which these tests exercise without a GPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(WORLD_SIZE=str(world), RANK=str(rank), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist()
    try:
        d.barrier()
        # rank r reports a step time of r + 1 and r + 1 units of work
        q.put((rank, d.max(float(rank + 1)), d.sum(float(rank + 1))))
        d.barrier()
    finally:
        d.pg.destroy_process_group()


def test_bench_collectives_two_ranks_gloo():
    pytest.importorskip("torch")
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert sorted(results) == [(0, 2.0, 3.0), (1, 2.0, 3.0)]


def test_bench_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    os.environ.pop("WORLD_SIZE", None)
    d = bench.Dist()
    assert d.pg is None and d.max(3.5) == 3.5 and d.sum(2.0) == 2.0
    d.barrier()


def test_reference_arm_times_complete_solves():
    """The CPU reference arm: one JSON line with impl "reference", measured on
    complete solves of the bounded sample (here 2 processes at 12^3), the
    headline workload's config, no host-device bytes; exit status 0."""
    import json
    import subprocess
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                          "--steps", "1", "--warmup", "0", "--cores", "2", "--cpu-grid", "12"],
                         capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    rec = json.loads(lines[0])
    assert rec["impl"] == "reference" and rec["value"] > 0 and rec["steps"] == 1
    assert rec["config"]["workload"].startswith("vardiff3d_7pt_128^3")
    assert rec["config"]["n"] == 128 ** 3 and rec["config"]["nnz_A"] == 14581760
    cb = rec["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] == 2 and "12^3" in cb["sample"]
    assert rec["e2e"]["h2d_bytes_per_step"] == 0 and rec["e2e"]["value"] == rec["value"]


def test_shard_by_footprint_single_process():
    sys.path.insert(0, ROOT)
    from gcge_gb300.sharding import shard_by_footprint
    w = [5, 1, 9, 9, 2, 7, 3, 3, 8]
    for world in (1, 2, 3, 4, 16):
        parts = shard_by_footprint(w, world)
        assert len(parts) == world
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(w)))
        loads = [sum(w[i] for i in p) for p in parts]
        if world <= len(w):
            assert max(loads) - min(loads) <= max(w)
    assert shard_by_footprint([], 3) == [[], [], []]


def _shard_rank(rank, world, port, q):
    os.environ.update(WORLD_SIZE=str(world), RANK=str(rank), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    from gcge_gb300 import problems as P
    from gcge_gb300.sharding import problem_footprint, shard_by_footprint
    d = bench.Dist()
    try:
        probs = P.batch_problems(count=48, seed=4)
        mine = shard_by_footprint([problem_footprint(c) for c in probs], d.world)[d.rank]
        # stand-in for the solves: each rank "converges" nev pairs per problem
        pairs = sum(probs[i]["nev"] for i in mine)
        everyone = d.gather(mine)
        q.put((rank, everyone, d.sum(float(pairs)), sum(c["nev"] for c in probs),
               d.max(float(len(mine)))))
        d.barrier()
    finally:
        d.pg.destroy_process_group()


def test_batch_sharding_two_ranks_gloo():
    """Every batched problem is assigned to exactly one of the two ranks, both
    ranks compute the same assignment, and the summed pairs equal the whole
    batch's."""
    pytest.importorskip("torch")
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_shard_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = sorted([q.get(timeout=300) for _ in procs], key=lambda x: x[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, g0, s0, tot0, m0), (r1, g1, s1, tot1, m1) = results
    assert g0 == g1
    flat = sorted(g0[0] + g0[1])
    assert flat == list(range(48))
    assert s0 == s1 == float(tot0) == float(tot1)
    assert m0 == m1 == float(max(len(g0[0]), len(g0[1])))
