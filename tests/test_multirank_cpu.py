"""The multi-process path of bench.py on CPU: two ranks over gloo at
127.0.0.1.  A single problem does not shard (each GPU runs its own replica of
the solve), so the only collectives are the benchmark's barrier and its
max/sum over ranks, which these tests exercise without a GPU."""
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


def test_reference_arm_reports_large_workload_unavailable():
    """The CPU reference arm is not sampled on the 128^3 workload: one JSON
    line with impl "reference" and the reason, exit status 0."""
    import json
    import subprocess
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                          "--workload", "vardiff3d"], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    rec = json.loads(lines[0])
    assert rec["impl"] == "reference" and "unavailable" in rec
