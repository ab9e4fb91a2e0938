#!/usr/bin/env python
"""Benchmark of the GB300 GCG eigensolver.

Headline workload (the mixed-precision configuration the metric is quoted
on): 3D variable-coefficient diffusion on a 128^3 grid, n = 2097152, 7-point
stencil with log-normal cell coefficients (mu 0, sigma 1) and harmonic-mean
face coefficients, B = diagonal lumped mass h^3 (1 + 0.1 U[0,1]); the nev = 200
smallest pairs with the reference front end's block rule (bs 40, nevInit 120,
nevMax 320, so the basis V is 400 columns, 6.7 GB), convergence
||A x - lambda B x|| <= 1e-8 |lambda|.  All data are generated and seeded
(gcge_gb300/problems.py); no dataset is involved.

One step = one complete GCG solve.  Metric: converged requested eigenpairs
per second.  `value` is the mixed-precision solver (FP32 block-PCG inner
solve, everything else FP64) with inputs resident in HBM, timed with CUDA
events on the library stream; `fp64_value` is the plain FP64 GPU GCG on the
same inputs with the largest relative eigenvalue difference between the two;
`e2e` is the same metric through GCGE_Solve from host CCS arrays in pinned
memory (matrix upload, device-side format build, solve, eigenvalue and
eigenvector download into pinned memory).  Extra keys: the generalized 64^3
stiffness + Kronecker-mass problem (nev 100) measured the same way, the
batched anisotropic-2D problems and a Poisson-arrival serving run.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`--impl reference` times the CPU restatement of the reference GCG
(oracle/gcg_oracle.py; the reference's C sources do not reach the GPU host)
on complete solves of a bounded sample of the headline workload: the same
generator and block rule at 16^3, one single-threaded solve per host core at
once, value = converged pairs / wall time.

N > 1 (torchrun): every rank solves its own replica of the single problem on
its own GPU ("replicas only": one problem is not split across GPUs), and the
batched problems and serving requests are sharded across the ranks by device
footprint; value = all ranks' pairs / max time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "converged eigenpairs/s @1e-8 resid: mixed vs FP64 GCG, 1 GB300; p50/p99 latency"
UNIT = "eigenpairs/s"
PEAK_FALLBACK_GBS = 6800.0
# bounded CPU sample of the headline workload: the same generator and block
# rule on a 16^3 grid (a complete single-threaded solve takes ~8 s)
CPU_SAMPLE_GRID = 16


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cores", type=int, default=0,
                    help="host cores of the CPU reference arm (0 = all)")
    ap.add_argument("--cpu-grid", type=int, default=CPU_SAMPLE_GRID,
                    help="grid of the CPU sample (k^3 unknowns)")
    ap.add_argument("--size", type=int, default=0,
                    help="grid size k of the single-problem workload (0: 128 for vardiff3d, "
                         "64 for laplace3d_mass)")
    ap.add_argument("--workload", choices=["vardiff3d", "laplace3d_mass"], default="vardiff3d",
                    help="the headline line: vardiff3d (128^3 variable coefficients, nev 200) or "
                         "laplace3d_mass (64^3 stiffness + Kronecker mass, nev 100)")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the second single-problem line and the batched / serving lines")
    ap.add_argument("--extra-steps", type=int, default=10,
                    help="mixed solves of the 64^3 extra line (FP64: half)")
    ap.add_argument("--batch-count", type=int, default=512)
    ap.add_argument("--workers", type=int, default=8)
    ap.add_argument("--serve-count", type=int, default=48)
    ap.add_argument("--serve-rate", type=float, default=8.0)
    ap.add_argument("--serve-max-n", type=int, default=300_000)
    ap.add_argument("--solve-once", choices=["mixed", "fp64"], default=None,
                    help="prepare the workload and run one solve (for profiler captures)")
    return ap.parse_args()


# ------------------------------------------------------------------ dist
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo", init_method="env://")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v: float) -> float:
        if not self.pg:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def sum(self, v: float) -> float:
        if not self.pg:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.SUM)
        return float(t.item())

    def gather(self, obj):
        """obj of every rank, in rank order."""
        if not self.pg:
            return [obj]
        out = [None] * self.world
        self.pg.all_gather_object(out, obj)
        return out

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# ------------------------------------------------------------------ clocks
class Clocks:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------------ helpers
def measured_peak_gbs():
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return PEAK_FALLBACK_GBS, "fallback"


def ncu_traffic_per_launch(name):
    """DRAM bytes per block-PCG kernel launch from a committed ncu summary."""
    p = os.path.join(HERE, "profiles", name)
    try:
        with open(p) as f:
            return float(json.load(f)["dram_bytes_per_launch"])
    except Exception:
        return None


def percentile(xs, q):
    xs = sorted(xs)
    if not xs:
        return None
    k = (len(xs) - 1) * q / 100.0
    lo, hi = int(k), min(len(xs) - 1, int(k) + 1)
    return xs[lo] + (xs[hi] - xs[lo]) * (k - lo)


def workload(name, size, build=True):
    """(problem dict or None, X0 or None, config description) of a
    single-problem workload; build=False gives the description alone."""
    from gcge_gb300 import problems as P
    if name == "vardiff3d":
        k = size or 128
        bs, ni, nm = P.gcge_block_rule(200)
        desc = dict(workload=f"vardiff3d_7pt_{k}^3 (log-normal kappa, harmonic faces) + lumped "
                             f"diagonal mass, nev=200",
                    n=k ** 3, nnz_A=7 * k ** 3 - 6 * k ** 2, nev=200, block_size=bs,
                    nev_init=ni, nev_max=nm, tol="rel 1e-8",
                    x0="library seeded uniform fill (nevGiven = 0)",
                    l2="working set (V alone 6.7 GB at 128^3) larger than the 129 MB L2")
        return (P.config3(k) if build else None), None, desc
    k = size or 64
    bs, ni, nm = P.gcge_block_rule(100)
    desc = dict(workload=f"laplace3d_7pt_{k}^3 + kron consistent mass (generalized), nev=100",
                n=k ** 3, nnz_A=7 * k ** 3 - 6 * k ** 2, nnz_B=(3 * k - 2) ** 3, nev=100,
                block_size=bs, nev_init=ni, nev_max=nm, tol="rel 1e-8",
                x0=f"seeded Gaussian n x {ni} (seed 1)",
                l2="working set (V 419 MB + matrices 106 MB at 64^3) larger than the 129 MB L2")
    if not build:
        return None, None, desc
    c = P.config2(k)
    return c, P.initial_block(c["A"].n, c["nev_init"], seed=1), desc


# ------------------------------------------------------------------ CPU arm
_CPU_CASES = {}


def _cpu_prepare(grid):
    """Import the oracle and build the sample problem in this pool process."""
    from gcge_gb300 import problems as P
    import oracle.gcg_oracle  # noqa: F401
    if grid not in _CPU_CASES:
        c = P.config3(grid)
        _CPU_CASES[grid] = (c, c["A"].to_scipy(), c["B"].to_scipy(),
                            P.initial_block(c["A"].n, c["nev_init"], seed=1))
    return os.getpid()


def _cpu_solve(grid):
    """One complete FP64 GCG solve of the CPU restatement (single-threaded
    BLAS: the pool's processes start with OPENBLAS_NUM_THREADS=1) on the
    headline generator at grid^3; returns (pairs, iterations, seconds)."""
    from oracle.gcg_oracle import gcg_solve
    _cpu_prepare(grid)
    c, A, B, X0 = _CPU_CASES[grid]
    t = time.perf_counter()
    r = gcg_solve(A, B, X0, c["nev"], c["block_size"], c["nev_init"], c["nev_max"])
    return min(r.nconv, c["nev"]), r.niter, time.perf_counter() - t


def cpu_sample_runs(grid, cores, steps, warmup):
    """`steps` timed rounds (after `warmup` untimed ones) of `cores` concurrent
    complete solves, one per process; returns (pairs, wall seconds, per-solve
    seconds, iterations) over the timed rounds."""
    import multiprocessing as mp
    os.environ["OPENBLAS_NUM_THREADS"] = "1"
    os.environ["OMP_NUM_THREADS"] = "1"
    ctx = mp.get_context("spawn")
    pairs, wall, per, iters = 0, 0.0, [], []
    with ctx.Pool(processes=cores) as pool:
        pool.map(_cpu_prepare, [grid] * cores, chunksize=1)  # imports, problem build
        for _ in range(warmup):
            pool.map(_cpu_solve, [grid] * cores, chunksize=1)
        for _ in range(steps):
            t0 = time.perf_counter()
            out = pool.map(_cpu_solve, [grid] * cores, chunksize=1)
            wall += time.perf_counter() - t0
            pairs += sum(o[0] for o in out)
            per += [o[2] for o in out]
            iters += [o[1] for o in out]
    return pairs, wall, per, iters



def cpu_sample_desc(grid, cores, per, iters):
    from gcge_gb300 import problems as P
    bs, ni, nm = P.gcge_block_rule(200)
    return (f"complete FP64 solves of the numpy/scipy restatement of the reference GCG "
            f"(oracle/gcg_oracle.py; the reference's C sources do not reach this host) on the "
            f"headline generator at {grid}^3 (n = {grid ** 3}, nev 200, bs {bs}, nevInit {ni}, "
            f"nevMax {nm}, tol rel 1e-8): {cores} single-threaded solves at once, one per "
            f"host core; {statistics.mean(per):.2f} s and {statistics.mean(iters):.0f} "
            f"iterations per solve")


def run_reference(args, d: Dist):
    """The reference arm: rank 0 alone times the CPU restatement on complete
    solves of the bounded sample; other ranks exit without work."""
    if d.rank != 0:
        return
    cores = args.cores or os.cpu_count() or 1
    pairs, wall, per, iters = cpu_sample_runs(args.cpu_grid, cores, args.steps, args.warmup)
    value = pairs / wall
    _, _, desc = workload(args.workload, args.size, build=False)
    sample = cpu_sample_desc(args.cpu_grid, cores, per, iters)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": wall / args.steps * 1000,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (generated, seeded)", "impl": "reference", "config": desc,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def cpu_baseline_line(args):
    """One complete single-threaded solve of the CPU sample in a child process
    (BLAS threads are fixed at start-up)."""
    env = dict(os.environ, OPENBLAS_NUM_THREADS="1", OMP_NUM_THREADS="1")
    cmd = [sys.executable, os.path.abspath(__file__), "--impl", "reference", "--steps", "1",
           "--warmup", "0", "--cores", "1", "--cpu-grid", str(args.cpu_grid)]
    try:
        out = subprocess.run(cmd, env=env, capture_output=True, text=True, timeout=900).stdout
        ref = json.loads([ln for ln in out.splitlines() if ln.startswith("{")][-1])
        return dict(ref["cpu_baseline"])
    except Exception as e:  # reported, not fatal
        return {"value": None, "unit": UNIT, "cores": 1, "kind": "port", "sample": f"failed: {e}"}


# ------------------------------------------------------------------ GPU arm
def measure_single(G, d: Dist, name, size, steps, warmup, fp64_steps, e2e_steps, clocks=None):
    """One single-problem workload: mixed solves timed with CUDA events (inputs
    resident in HBM), FP64 solves the same way, GCGE_Solve end to end from
    pinned host arrays, and the accuracy of the mixed solve."""
    import numpy as np
    from gcge_gb300 import problems as PP
    c, X0, desc = workload(name, size)
    A, B, nev = c["A"], c["B"], c["nev"]
    kw = dict(nev=nev, block_size=c["block_size"], nev_init=c["nev_init"], nev_max=c["nev_max"],
              max_iter=2000, X0=X0)

    def timed(prep, k):
        infos, pairs, r = [], 0, None
        d.barrier()
        with G.DeviceTimer() as tm:
            for _ in range(k):
                r = prep.solve()  # returns after the solve's last device work
                infos.append(r.info)
                pairs += min(r.nconv, nev) if r.status == G.GCGE_OK else 0
        return d.max(tm.ms / 1000.0), d.sum(pairs), infos, r

    prep = G.Prepared(A, B, precision=G.PREC_MIXED, **kw)
    for _ in range(warmup):
        prep.solve()
    if clocks:
        clocks.start()
    t_mixed, pairs_mixed, infos, r = timed(prep, steps)
    clk = clocks.stop() if clocks else None
    ev_mixed = r.eval[:nev].copy()
    prep.close()
    prep64 = G.Prepared(A, B, precision=G.PREC_FP64, **kw)
    t_fp64, pairs_fp64, infos64, r64 = timed(prep64, fp64_steps)
    prep64.close()
    value = pairs_mixed / t_mixed
    fp64_value = pairs_fp64 / t_fp64
    eig_err = float(np.max(np.abs(ev_mixed - r64.eval[:nev]) / np.abs(r64.eval[:nev])))

    # end to end through GCGE_Solve: every step uploads the CCS arrays (and the
    # initial block) from pinned host memory, builds the formats on the
    # device, solves, and reads eigenvalues and all nev_max eigenvectors back
    # into pinned host memory
    pA = PP.CSRMatrix(A.n, G.pinned_copy(A.indptr.astype(np.int32)),
                      G.pinned_copy(A.indices.astype(np.int32)), G.pinned_copy(A.data))
    pB = PP.CSRMatrix(B.n, G.pinned_copy(B.indptr.astype(np.int32)),
                      G.pinned_copy(B.indices.astype(np.int32)), G.pinned_copy(B.data))
    kw_e2e = dict(kw)
    if X0 is not None:
        kw_e2e["X0"] = G.pinned_copy(np.asfortranarray(X0), order="F")
    ev_out = G.pinned_empty(c["nev_max"])
    evec_out = G.pinned_empty((A.n, c["nev_max"]), order="F")
    d.barrier()
    t0 = time.perf_counter()
    e2e_pairs = 0
    for _ in range(e2e_steps):
        re = G.solve(pA, pB, precision=G.PREC_MIXED, evec_out=evec_out, eval_out=ev_out, **kw_e2e)
        e2e_pairs += min(re.nconv, nev) if re.status == G.GCGE_OK else 0
    t_e2e = d.max(time.perf_counter() - t0)
    e2e_value = d.sum(e2e_pairs) / t_e2e
    h2d = (A.indptr.nbytes + A.indices.nbytes + A.data.nbytes + B.indptr.nbytes
           + B.indices.nbytes + B.data.nbytes + (X0.nbytes if X0 is not None else 0))
    d2h = 8 * c["nev_max"] * (1 + A.n)
    # relative residuals ||A x - lambda B x|| / |lambda| of the returned pairs
    # (host sparse products on the e2e solve's eigenvectors, outside the timing)
    Xe = np.asarray(evec_out)[:, :nev]
    lam = np.asarray(ev_out)[:nev]
    Rr = A.to_scipy() @ Xe - (B.to_scipy() @ Xe) * lam
    max_res = float(np.max(np.linalg.norm(Rr, axis=0) / np.abs(lam)))

    def total(key, xs):
        return sum(i[key] for i in xs)
    pcg_ms, pcg_bytes = total("pcg_kernel_ms", infos), total("pcg_kernel_bytes", infos)
    pcg_launches = total("pcg_kernel_launches", infos)
    spmm_ms, spmm_bytes = total("pcg_spmm_ms", infos), total("pcg_spmm_bytes", infos)
    spmm_phases = total("pcg_spmm_launches", infos)
    peak, peak_kind = measured_peak_gbs()
    achieved = pcg_bytes / (pcg_ms / 1000.0) / 1e9 if pcg_ms > 0 else None
    spmm_achieved = spmm_bytes / (spmm_ms / 1000.0) / 1e9 if spmm_ms > 0 else None
    kp = 40 if c["block_size"] > 32 else (20 if c["block_size"] > 16 else 16)
    lat = [1000.0 * i["seconds"] for i in infos]
    traffic_file = ("block_pcg_fp32_vardiff3d_128_k40.json" if name == "vardiff3d"
                    else "block_pcg_fp32_laplace3d_mass_64.json")
    out = {
        "value": value, "ms_per_step": t_mixed / steps * 1000.0, "config": desc,
        "fp64_value": fp64_value, "mixed_over_fp64": value / fp64_value if fp64_value else None,
        "fp64_ms_per_step": t_fp64 / fp64_steps * 1000.0, "fp64_steps": fp64_steps,
        "eigenvalue_rel_error_vs_fp64": eig_err, "max_rel_residual": max_res,
        "niter": [i["niter"] for i in infos], "nconv": [i["nconv"] for i in infos],
        "fp64_niter": [i["niter"] for i in infos64],
        "phase_ms_last_step": infos[-1]["phase_ms"], "phase_ms_fp64": infos64[-1]["phase_ms"],
        "gpu_launches": total("kernel_launches", infos),
        "escalated_solves": sum(i.get("precision_escalation_iter", 0) > 0 for i in infos),
        "latency_ms": {"p50": percentile(lat, 50), "p99": percentile(lat, 99),
                       "solves": len(lat), "what": "one mixed solve, inputs resident in HBM"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "steps": e2e_steps},
        "roofline": {"kernel": f"k_block_pcg<float,{kp}> (persistent block PCG of the W step: "
                               f"p update, SpMM on the union pattern of A and B, x/r update)",
                     "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None, "peak_kind": peak_kind,
                     "traffic": ncu_traffic_per_launch(traffic_file),
                     "bytes_per_launch": pcg_bytes / max(1, pcg_launches),
                     "ms_per_launch": pcg_ms / max(1, pcg_launches), "launches": pcg_launches,
                     "spmm_phase": {"achieved": spmm_achieved,
                                    "frac": (spmm_achieved / peak) if spmm_achieved else None,
                                    "bytes_per_phase": spmm_bytes / max(1, spmm_phases),
                                    "ms_per_phase": spmm_ms / max(1, spmm_phases),
                                    "phases": spmm_phases}},
        "clocks": clk,
    }
    return out


def run_batch_lines(G, args, d: Dist):
    """Many solves per GPU through the request server: the batched workload
    (the 512 problems of the anisotropic-2D generator) in mixed and FP64
    precision, and a Poisson stream of serving requests in both precisions.
    With several ranks the problems and requests are sharded across them by
    device footprint (gcge_gb300.sharding); value = all pairs / slowest rank."""
    from gcge_gb300 import problems as P
    from gcge_gb300.sharding import problem_footprint, shard_by_footprint

    def job(c, prec):
        return G.Job(c["A"], c["B"], c["nev"], c["block_size"], c["nev_init"], c["nev_max"],
                     X0=P.initial_block(c["A"].n, c["nev_init"], seed=1),
                     tol=c.get("tol", (1e300, 1e-8)), precision=prec)

    def pairs_of(cs, results):
        return sum(min(r.nconv, c["nev"]) for c, r in zip(cs, results) if r.status == G.GCGE_OK)

    probs = P.batch_problems(count=args.batch_count, seed=4)
    mine = [probs[i] for i in shard_by_footprint([problem_footprint(c) for c in probs],
                                                 d.world)[d.rank]]
    G.solve_batch([job(c, G.PREC_MIXED) for c in mine[:args.workers]], workers=args.workers)
    out = {}
    for name, prec in (("mixed", G.PREC_MIXED), ("fp64", G.PREC_FP64)):
        jobs = [job(c, prec) for c in mine]
        d.barrier()
        t0 = time.perf_counter()
        res = G.solve_batch(jobs, workers=args.workers)
        dt = d.max(time.perf_counter() - t0)
        out[name] = {"eigenpairs_per_s": d.sum(pairs_of(mine, res)) / dt, "seconds": dt,
                     "ok": int(d.sum(sum(r.status == G.GCGE_OK for r in res))),
                     "problems": int(d.sum(len(mine)))}
    lines = {"batch": {
        "workload": f"the {len(probs)} anisotropic 2D problems (nx, ny in 40..220, anisotropy "
                    "1..100, diagonal B, nev 8..64, tol 1e-8), seeded",
        "workers_per_gpu": args.workers, "mixed": out["mixed"], "fp64": out["fp64"],
        "mixed_over_fp64": out["mixed"]["eigenpairs_per_s"] / out["fp64"]["eigenpairs_per_s"]}}

    reqs = P.serving_requests(args.serve_count, seed=5, rate=args.serve_rate,
                              max_n=args.serve_max_n)
    mine_idx = shard_by_footprint([problem_footprint(c) for c in reqs], d.world)[d.rank]
    mreqs = [reqs[i] for i in mine_idx]
    serve = {}
    for name, prec in (("mixed", G.PREC_MIXED), ("fp64", G.PREC_FP64)):
        jobs = [job(c, prec) for c in mreqs]
        d.barrier()
        with G.Server(workers=args.workers) as srv:
            t0 = time.perf_counter()
            for c, j in zip(mreqs, jobs):
                delay = t0 + c["arrival"] - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
                srv.submit(j)
            res = [srv.wait(j) for j in jobs]
            span = d.max(time.perf_counter() - t0)
        lat = [x for part in d.gather([j.latency for j in jobs]) for x in part]
        not_ok = [[c["name"], c["nev"], r.status, r.nconv, r.niter]
                  for c, r in zip(mreqs, res) if r.status != G.GCGE_OK]
        serve[name] = {"eigenpairs_per_s": d.sum(pairs_of(mreqs, res)) / span, "seconds": span,
                       "ok": int(d.sum(sum(r.status == G.GCGE_OK for r in res))),
                       "not_ok": [x for part in d.gather(not_ok) for x in part],
                       "latency_ms": {"p50": 1000.0 * percentile(lat, 50),
                                      "p99": 1000.0 * percentile(lat, 99)}}
    lines["serve"] = {
        "workload": f"{len(reqs)} Poisson-arrival requests at {args.serve_rate}/s: 2D/3D "
                    f"Laplacians, shifted RGG Laplacians, variable-coefficient 3D diffusion, "
                    f"n <= {args.serve_max_n}, nev 10..100, tol 1e-6..1e-10, B = I or lumped mass",
        "workers_per_gpu": args.workers, "mixed": serve["mixed"], "fp64": serve["fp64"],
        "mixed_over_fp64": serve["mixed"]["eigenpairs_per_s"] / serve["fp64"]["eigenpairs_per_s"],
        "latency_what": "arrival (submit) to results on the host"}
    return lines


def run_ours(args, d: Dist):
    os.environ.setdefault("CUDA_VISIBLE_DEVICES", str(d.local))
    import gcge_gb300 as G
    G.load(build_if_missing=True)
    head = args.workload
    big = head == "vardiff3d"
    fp64_steps = 1 if big else max(1, args.steps // 2)
    e2e_steps = max(1, args.steps // 10) if big else max(1, args.steps // 2)
    m = measure_single(G, d, head, args.size, args.steps, args.warmup, fp64_steps, e2e_steps,
                       clocks=Clocks(d.local))
    line = {"metric": METRIC, "value": m.pop("value"), "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": m.pop("ms_per_step"),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64 outer / f32 inner PCG (mixed)", "data": "synthetic (generated, seeded)"}
    cfg = m.pop("config")
    cfg.update(precision="mixed", parallelism=f"replicas x{d.world}")
    line["config"] = cfg
    line.update(m)
    if not args.no_extra:
        other = "laplace3d_mass" if big else "vardiff3d"
        if other == "laplace3d_mass":
            k2 = max(1, args.extra_steps)
            x = measure_single(G, d, other, 0, k2, 3, max(1, k2 // 2), max(1, k2 // 2))
            x.pop("clocks", None)
            line["laplace3d_mass_64"] = x
        line.update(run_batch_lines(G, args, d))
    if d.rank == 0 and d.world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_line(args)
    if d.rank == 0:
        print(json.dumps(line), flush=True)


def solve_once(args):
    import gcge_gb300 as G
    G.load(build_if_missing=True)
    c, X0, _ = workload(args.workload, args.size)
    prep = G.Prepared(c["A"], c["B"], c["nev"], c["block_size"], c["nev_init"], c["nev_max"], X0=X0,
                      max_iter=2000,
                      precision=G.PREC_MIXED if args.solve_once == "mixed" else G.PREC_FP64)
    r = prep.solve()
    prep.close()
    print(json.dumps({"nconv": r.nconv, "niter": r.niter, "status": r.status,
                      "kernel_launches": r.info["kernel_launches"],
                      "phase_ms": r.info["phase_ms"]}))
    return 0 if r.status == G.GCGE_OK else 1


def main():
    args = parse()
    if args.solve_once:
        sys.exit(solve_once(args))
    d = Dist()
    try:
        if args.impl == "reference":
            run_reference(args, d)
        else:
            run_ours(args, d)
    finally:
        d.close()


if __name__ == "__main__":
    main()
