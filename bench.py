#!/usr/bin/env python
"""Benchmark of the GB300 GCG eigensolver on the generalized 3D workload.

Workload (the generalized problem the headline metric is quoted on): A = (1/h^2)
7-point Dirichlet Laplacian on a 64^3 grid (h = 1/65), B = M x M x M with the
1D consistent mass M = h tridiag(1/6, 4/6, 1/6) (27 nonzeros per row),
n = 262144; the nev = 100 smallest pairs, block size 20, nevInit 60,
nevMax 160 (the reference front end's block rule), convergence
||A x - lambda B x|| <= 1e-8 |lambda|, seeded Gaussian initial block.  All
data are generated (problems.py); no dataset is involved.

One step = one complete GCG solve.  Metric: converged requested eigenpairs per
second (nev / solve time).  `value` is the mixed-precision solver (FP32
block-PCG inner solve, everything else FP64) with inputs resident in HBM,
timed with CUDA events on the library stream; `fp64_value` is the plain FP64
GPU GCG on the same inputs; `e2e` is the same metric through GCGE_Solve from
host CCS arrays in pinned memory (matrix upload, device-side format build,
solve, eigenvalue and eigenvector download into pinned memory).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

N > 1 (torchrun): every rank solves its own replica on its own GPU (a single
problem is not split across GPUs); value = all ranks' pairs / max time.
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
WORKLOAD = dict(workload="laplace3d_7pt_64^3 + kron consistent mass (generalized), nev=100",
                n=262144, nnz_A=1810432, nnz_B=6859000, nev=100, block_size=20, nev_init=60,
                nev_max=160, tol="rel 1e-8", x0="seeded Gaussian n x 60 (seed 1)",
                l2="working set (V 419 MB + matrices 106 MB) larger than the 129 MB L2")
PEAK_FALLBACK_GBS = 6800.0
# Iterations the full solve needs at this workload: measured with the GPU
# FP64 path (54, same algorithm and initial block); the reference CPU arm and
# the CPU baseline time a bounded number of outer iterations and scale by it.
FULL_SOLVE_ITERS = 54


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-iters", type=int, default=2,
                    help="outer iterations of the CPU sample (baseline / reference arm)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--threads", type=int, default=0,
                    help="host threads of the CPU reference arm (0 = all)")
    ap.add_argument("--size", type=int, default=64, help="grid size k (k^3 unknowns)")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched and serving lines")
    ap.add_argument("--batch-count", type=int, default=64)
    ap.add_argument("--workers", type=int, default=8)
    ap.add_argument("--serve-count", type=int, default=24)
    ap.add_argument("--serve-rate", type=float, default=8.0)
    ap.add_argument("--serve-max-n", type=int, default=100_000)
    ap.add_argument("--solve-once", choices=["mixed", "fp64"], default=None,
                    help="prepare the workload and run one solve (for profiler captures)")
    ap.add_argument("--workload", choices=["laplace3d_mass", "vardiff3d"],
                    default="laplace3d_mass",
                    help="vardiff3d: the 128^3 variable-coefficient problem, nev 200 (about "
                         "four minutes at the default steps); its line reports the mixed solve, "
                         "the FP64 solve and the eigenvalue error between them")
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


def ncu_traffic_per_launch():
    """DRAM bytes per block-PCG kernel launch from the committed ncu summary, if any."""
    p = os.path.join(HERE, "profiles", "block_pcg_fp32_laplace3d_mass_64.json")
    try:
        with open(p) as f:
            return float(json.load(f)["dram_bytes_per_launch"])
    except Exception:
        return None


def build_workload(k):
    from gcge_gb300 import problems as P
    c = P.config2(k)
    X0 = P.initial_block(c["A"].n, c["nev_init"], seed=1)
    return c, X0


def cpu_sample(c, X0, iters, threads):
    """The CPU oracle (numpy restatement of the reference GCG) on the same
    workload for `iters` outer iterations.  Returns the estimated seconds of a
    full solve: set-up (InitializeX, first Rayleigh-Ritz) + FULL_SOLVE_ITERS x
    the mean measured outer-iteration time, and the sampled seconds."""
    from oracle.gcg_oracle import GCGOracle, GCGParams
    p = GCGParams(nev_init=c["nev_init"], nev_max=c["nev_max"], block_size=c["block_size"],
                  num_iter_max=iters)
    o = GCGOracle(c["A"].to_scipy(), c["B"].to_scipy(), p)
    r = o.solve(X0, c["nev"])
    m = r.marks
    setup = m[1] - m[0]
    per_iter = (m[-1] - m[1]) / max(1, len(m) - 2)
    return setup + FULL_SOLVE_ITERS * per_iter, m[-1] - m[0]


# ------------------------------------------------------------------ arms
def run_reference(args, d: Dist):
    if d.rank != 0:
        return
    if args.workload == "vardiff3d":
        print(json.dumps({"impl": "reference", "unavailable": "the CPU restatement is not sampled "
                          "at n = 2097152 with nev 200 (6.7 GB per basis); the default workload's "
                          "reference line is the CPU comparison"}), flush=True)
        return
    threads = args.threads or os.cpu_count() or 1
    c, X0 = build_workload(args.size)
    cw, X0w = build_workload(12)
    for _ in range(args.warmup):
        cpu_sample(cw, X0w, 1, threads)
    runs = [cpu_sample(c, X0, args.cpu_iters, threads) for _ in range(args.steps)]
    per_solve = statistics.mean(r[0] for r in runs)
    sampled = statistics.mean(r[1] for r in runs)
    value = c["nev"] / per_solve
    sample = (f"numpy/scipy restatement of the reference GCG (oracle/gcg_oracle.py; the reference's "
              f"own C build is not available on this host): set-up + {args.cpu_iters} outer "
              f"iterations of this workload ({sampled:.1f} s sampled per step), extrapolated to "
              f"set-up + {FULL_SOLVE_ITERS} iterations")
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_solve * 1000,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference", "config": WORKLOAD,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, d: Dist):
    os.environ.setdefault("CUDA_VISIBLE_DEVICES", str(d.local))
    import numpy as np
    import gcge_gb300 as G
    G.load(build_if_missing=True)
    c, X0 = build_workload(args.size)
    A, B, nev = c["A"], c["B"], c["nev"]
    kw = dict(nev=nev, block_size=c["block_size"], nev_init=c["nev_init"], nev_max=c["nev_max"],
              X0=X0)
    prep_mixed = G.Prepared(A, B, precision=G.PREC_MIXED, **kw)
    prep_fp64 = G.Prepared(A, B, precision=G.PREC_FP64, **kw)

    last_eval = {}

    def timed(prep, steps):
        infos, pairs = [], 0
        d.barrier()
        with G.DeviceTimer() as tm:
            for _ in range(steps):
                r = prep.solve()  # returns after the solve's last device work
                infos.append(r.info)
                pairs += min(r.nconv, nev) if r.status == G.GCGE_OK else 0
        last_eval[id(prep)] = r.eval[:nev].copy()
        return tm.ms / 1000.0, pairs, infos

    def percentile(xs, q):
        xs = sorted(xs)
        k = (len(xs) - 1) * q / 100.0
        lo, hi = int(np.floor(k)), int(np.ceil(k))
        return xs[lo] + (xs[hi] - xs[lo]) * (k - lo)

    for _ in range(args.warmup):
        prep_mixed.solve()
    prep_fp64.solve()
    clocks = Clocks(d.local)
    clocks.start()
    t_mixed, pairs_mixed, infos = timed(prep_mixed, args.steps)
    clk = clocks.stop()
    t_fp64, pairs_fp64, infos64 = timed(prep_fp64, max(1, args.steps // 2))
    t_mixed_max = d.max(t_mixed)
    value = d.sum(pairs_mixed) / t_mixed_max
    fp64_value = d.sum(pairs_fp64) / d.max(t_fp64)

    # end to end through GCGE_Solve: every step uploads the CCS arrays and the
    # initial block from pinned host memory, builds the formats, solves, and
    # reads eigenvalues and eigenvectors back into pinned host memory
    from gcge_gb300 import problems as PP
    pA = PP.CSRMatrix(A.n, G.pinned_copy(A.indptr.astype(np.int32)),
                      G.pinned_copy(A.indices.astype(np.int32)), G.pinned_copy(A.data))
    pB = PP.CSRMatrix(B.n, G.pinned_copy(B.indptr.astype(np.int32)),
                      G.pinned_copy(B.indices.astype(np.int32)), G.pinned_copy(B.data))
    kw_e2e = dict(kw)
    kw_e2e["X0"] = G.pinned_copy(np.asfortranarray(X0), order="F")
    ev_out = G.pinned_empty(c["nev_max"])
    evec_out = G.pinned_empty((A.n, c["nev_max"]), order="F")
    e2e_steps = max(1, args.steps // 2)
    d.barrier()
    t0 = time.perf_counter()
    e2e_pairs = 0
    for _ in range(e2e_steps):
        r = G.solve(pA, pB, precision=G.PREC_MIXED, evec_out=evec_out, eval_out=ev_out, **kw_e2e)
        e2e_pairs += min(r.nconv, nev) if r.status == G.GCGE_OK else 0
    t_e2e = d.max(time.perf_counter() - t0)
    # accuracy of the mixed solve: eigenvalues against the FP64 solve, and the
    # relative residuals ||A x - lambda B x|| / |lambda| of the returned pairs
    # (host sparse products on the e2e solve's eigenvectors, outside the timing)
    ev_m, ev_f = last_eval[id(prep_mixed)], last_eval[id(prep_fp64)]
    eig_err = float(np.max(np.abs(ev_m - ev_f) / np.abs(ev_f)))
    Xe = np.asarray(evec_out)[:, :nev]
    lam = np.asarray(ev_out)[:nev]
    Rr = A.to_scipy() @ Xe - (B.to_scipy() @ Xe) * lam
    max_res = float(np.max(np.linalg.norm(Rr, axis=0) / np.abs(lam)))
    # per-solve latency of the mixed solve (host clock around each solve,
    # which returns after its device work)
    lat = [1000.0 * i["seconds"] for i in infos]
    e2e_value = d.sum(e2e_pairs) / t_e2e
    h2d = (A.indptr.nbytes + A.indices.nbytes + A.data.nbytes + B.indptr.nbytes + B.indices.nbytes
           + B.data.nbytes + X0.nbytes)
    d2h = 8 * c["nev_max"] * (1 + A.n)

    # many solves on this GPU (batched problems, serving); rank 0 of a 1-GPU run
    batch = run_batch_lines(G, args) if (not args.no_batch and d.world == 1) else None

    spmm_ms = sum(i["pcg_spmm_ms"] for i in infos)
    spmm_bytes = sum(i["pcg_spmm_bytes"] for i in infos)
    spmm_phases = sum(i["pcg_spmm_launches"] for i in infos)
    pcg_ms = sum(i["pcg_kernel_ms"] for i in infos)
    pcg_bytes = sum(i["pcg_kernel_bytes"] for i in infos)
    pcg_launches = sum(i["pcg_kernel_launches"] for i in infos)
    peak, peak_kind = measured_peak_gbs()
    achieved = pcg_bytes / (pcg_ms / 1000.0) / 1e9 if pcg_ms > 0 else None
    spmm_achieved = spmm_bytes / (spmm_ms / 1000.0) / 1e9 if spmm_ms > 0 else None
    traffic = ncu_traffic_per_launch()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_mixed_max / args.steps * 1000.0,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64 outer / f32 inner PCG (mixed)", "data": "synthetic (generated, seeded)",
        "config": dict(WORKLOAD, precision="mixed", parallelism=f"replicas x{d.world}"),
        "fp64_value": fp64_value, "mixed_over_fp64": value / fp64_value if fp64_value else None,
        "fp64_ms_per_step": t_fp64 / max(1, args.steps // 2) * 1000.0,
        "eigenvalue_rel_error_vs_fp64": eig_err,
        "max_rel_residual": max_res,
        "niter": [i["niter"] for i in infos], "nconv": [i["nconv"] for i in infos],
        "phase_ms_last_step": infos[-1]["phase_ms"], "phase_ms_fp64": infos64[-1]["phase_ms"],
        "gpu_launches": sum(i["kernel_launches"] for i in infos),
        "escalated_solves": sum(i.get("precision_escalation_iter", 0) > 0 for i in infos),
        "latency_ms": {"p50": percentile(lat, 50), "p99": percentile(lat, 99), "solves": len(lat),
                       "what": "one mixed solve, inputs resident in HBM"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "steps": e2e_steps},
        "roofline": {"kernel": "k_block_pcg<float,20> (persistent block PCG of the W step: "
                               "p update, SpMM on the union pattern of A and B, x/r update)",
                     "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None, "peak_kind": peak_kind,
                     "traffic": traffic,
                     "bytes_per_launch": pcg_bytes / max(1, pcg_launches),
                     "ms_per_launch": pcg_ms / max(1, pcg_launches), "launches": pcg_launches,
                     "spmm_phase": {"achieved": spmm_achieved,
                                    "frac": (spmm_achieved / peak) if spmm_achieved else None,
                                    "bytes_per_phase": spmm_bytes / max(1, spmm_phases),
                                    "ms_per_phase": spmm_ms / max(1, spmm_phases),
                                    "phases": spmm_phases}},
        "clocks": clk,
    }
    if batch:
        line.update(batch)
    prep_mixed.close()
    prep_fp64.close()
    if d.rank == 0 and d.world == 1 and not args.no_cpu_baseline:
        # single-threaded CPU oracle in a child process (BLAS threads fixed at start-up)
        env = dict(os.environ, OPENBLAS_NUM_THREADS="1", OMP_NUM_THREADS="1")
        cmd = [sys.executable, os.path.abspath(__file__), "--impl", "reference", "--steps", "1",
               "--warmup", "0", "--threads", "1", "--cpu-iters", str(args.cpu_iters),
               "--size", str(args.size)]
        try:
            out = subprocess.run(cmd, env=env, capture_output=True, text=True, timeout=900).stdout
            ref = json.loads([ln for ln in out.splitlines() if ln.startswith("{")][-1])
            line["cpu_baseline"] = dict(ref["cpu_baseline"])
        except Exception as e:  # reported, not fatal
            line["cpu_baseline"] = {"value": None, "unit": UNIT, "cores": 1, "kind": "port",
                                    "sample": f"failed: {e}"}
    if d.rank == 0:
        print(json.dumps(line), flush=True)


def _percentiles(xs):
    xs = sorted(xs)

    def q(p):
        k = (len(xs) - 1) * p / 100.0
        lo, hi = int(k), min(len(xs) - 1, int(k) + 1)
        return xs[lo] + (xs[hi] - xs[lo]) * (k - lo)
    return {"p50": 1000.0 * q(50), "p99": 1000.0 * q(99)}


def run_batch_lines(G, args):
    """Many solves on the one GPU through the request server: the batched
    workload (first `--batch-count` problems of the 512-problem generator) in
    mixed and FP64 precision, and a Poisson stream of serving requests."""
    from gcge_gb300 import problems as P

    def job(c, prec):
        return G.Job(c["A"], c["B"], c["nev"], c["block_size"], c["nev_init"], c["nev_max"],
                     X0=P.initial_block(c["A"].n, c["nev_init"], seed=1),
                     tol=c.get("tol", (1e300, 1e-8)), precision=prec)

    def pairs_of(cs, results):
        return sum(min(r.nconv, c["nev"]) for c, r in zip(cs, results) if r.status == G.GCGE_OK)

    probs = P.batch_problems(count=args.batch_count, seed=4)
    G.solve_batch([job(c, G.PREC_MIXED) for c in probs[:args.workers]], workers=args.workers)
    out = {}
    for name, prec in (("mixed", G.PREC_MIXED), ("fp64", G.PREC_FP64)):
        jobs = [job(c, prec) for c in probs]
        t0 = time.perf_counter()
        res = G.solve_batch(jobs, workers=args.workers)
        dt = time.perf_counter() - t0
        out[name] = {"eigenpairs_per_s": pairs_of(probs, res) / dt, "seconds": dt,
                     "ok": sum(r.status == G.GCGE_OK for r in res)}
    batch = {"batch": {
        "workload": f"first {len(probs)} of the 512 anisotropic 2D problems (nx, ny in 40..220, "
                    "anisotropy 1..100, diagonal B, nev 8..64, tol 1e-8), seeded",
        "workers": args.workers, "mixed": out["mixed"], "fp64": out["fp64"],
        "mixed_over_fp64": out["mixed"]["eigenpairs_per_s"] / out["fp64"]["eigenpairs_per_s"]}}

    reqs = P.serving_requests(args.serve_count, seed=5, rate=args.serve_rate, max_n=args.serve_max_n)
    jobs = [job(c, G.PREC_MIXED) for c in reqs]
    with G.Server(workers=args.workers) as srv:
        t0 = time.perf_counter()
        for c, j in zip(reqs, jobs):
            delay = t0 + c["arrival"] - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            srv.submit(j)
        res = [srv.wait(j) for j in jobs]
        span = time.perf_counter() - t0
    batch["serve"] = {
        "workload": f"{len(reqs)} Poisson-arrival requests at {args.serve_rate}/s: 2D/3D Laplacians, "
                    f"shifted RGG Laplacians, variable-coefficient 3D diffusion, n <= "
                    f"{args.serve_max_n}, nev 10..100, tol 1e-6..1e-10, B = I or lumped mass",
        "workers": args.workers, "eigenpairs_per_s": pairs_of(reqs, res) / span, "seconds": span,
        "ok": sum(r.status == G.GCGE_OK for r in res),
        "not_ok": [[c["name"], c["nev"], r.status, r.nconv, r.niter]
                   for c, r in zip(reqs, res) if r.status != G.GCGE_OK],
        "latency_ms": _percentiles([j.latency for j in jobs]),
        "latency_what": "arrival (submit) to results on the host"}
    return batch


def run_vardiff(args, d: Dist):
    """The mixed-precision workload of the 128^3 variable-coefficient diffusion
    problem (n = 2097152, 7-point, diagonal lumped B, nev 200, bs 40, nevInit
    120, nevMax 320, so projected dimensions up to 400): mixed solves timed
    like the default workload, one FP64 solve, and the largest relative
    eigenvalue difference between them.  The initial basis is the library's
    seeded random fill (nevGiven = 0), so nothing of size n x nev is generated
    on the host."""
    os.environ.setdefault("CUDA_VISIBLE_DEVICES", str(d.local))
    import numpy as np
    import gcge_gb300 as G
    from gcge_gb300 import problems as PP
    G.load(build_if_missing=True)
    k = args.size if args.size != 64 else 128
    c = PP.config3(k)
    A, B, nev = c["A"], c["B"], c["nev"]
    kw = dict(nev=nev, block_size=c["block_size"], nev_init=c["nev_init"], nev_max=c["nev_max"],
              max_iter=2000)
    prep_mixed = G.Prepared(A, B, precision=G.PREC_MIXED, **kw)
    for _ in range(args.warmup):
        prep_mixed.solve()
    clocks = Clocks(d.local)
    clocks.start()
    d.barrier()
    infos, pairs = [], 0
    with G.DeviceTimer() as tm:
        for _ in range(args.steps):
            r = prep_mixed.solve()
            infos.append(r.info)
            pairs += min(r.nconv, nev) if r.status == G.GCGE_OK else 0
    clk = clocks.stop()
    ev_mixed = r.eval[:nev].copy()
    t_mixed = d.max(tm.ms / 1000.0)
    prep_mixed.close()
    prep_fp64 = G.Prepared(A, B, precision=G.PREC_FP64, **kw)
    with G.DeviceTimer() as tm64:
        r64 = prep_fp64.solve()
    prep_fp64.close()
    t_fp64 = d.max(tm64.ms / 1000.0)
    value = d.sum(pairs) / t_mixed
    fp64_value = d.sum(min(r64.nconv, nev) if r64.status == G.GCGE_OK else 0) / t_fp64
    ev64 = r64.eval[:nev]
    err = float(np.max(np.abs(ev_mixed - ev64) / np.abs(ev64)))
    # end to end: GCGE_Solve from page-locked host arrays, eigenvalues and
    # eigenvectors back into page-locked memory
    pA = PP.CSRMatrix(A.n, G.pinned_copy(A.indptr.astype(np.int32)),
                      G.pinned_copy(A.indices.astype(np.int32)), G.pinned_copy(A.data))
    pB = PP.CSRMatrix(B.n, G.pinned_copy(B.indptr.astype(np.int32)),
                      G.pinned_copy(B.indices.astype(np.int32)), G.pinned_copy(B.data))
    ev_out = G.pinned_empty(c["nev_max"])
    evec_out = G.pinned_empty((A.n, c["nev_max"]), order="F")
    d.barrier()
    t0 = time.perf_counter()
    re = G.solve(pA, pB, precision=G.PREC_MIXED, evec_out=evec_out, eval_out=ev_out, **kw)
    t_e2e = d.max(time.perf_counter() - t0)
    e2e_pairs = min(re.nconv, nev) if re.status == G.GCGE_OK else 0
    Xe = np.asarray(evec_out)[:, :nev]
    lam = np.asarray(ev_out)[:nev]
    Rr = A.to_scipy() @ Xe - (B.to_scipy() @ Xe) * lam
    max_res = float(np.max(np.linalg.norm(Rr, axis=0) / np.abs(lam)))
    pcg_ms = sum(i["pcg_kernel_ms"] for i in infos)
    pcg_bytes = sum(i["pcg_kernel_bytes"] for i in infos)
    pcg_launches = sum(i["pcg_kernel_launches"] for i in infos)
    peak, peak_kind = measured_peak_gbs()
    achieved = pcg_bytes / (pcg_ms / 1000.0) / 1e9 if pcg_ms > 0 else None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_mixed / args.steps * 1000.0,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64 outer / f32 inner PCG (mixed)", "data": "synthetic (generated, seeded)",
        "config": dict(workload=f"vardiff3d_7pt_{k}^3 (log-normal kappa, harmonic faces) + "
                                f"lumped diagonal mass, nev={nev}",
                       n=A.n, nnz_A=A.nnz, nev=nev, block_size=c["block_size"],
                       nev_init=c["nev_init"], nev_max=c["nev_max"], tol="rel 1e-8",
                       x0="library seeded uniform fill (nevGiven = 0)",
                       l2="working set (V alone 6.7 GB) larger than the 129 MB L2",
                       precision="mixed", parallelism=f"replicas x{d.world}"),
        "fp64_value": fp64_value, "mixed_over_fp64": value / fp64_value if fp64_value else None,
        "fp64_ms_per_step": t_fp64 * 1000.0,
        "eigenvalue_rel_error_vs_fp64": err,
        "max_rel_residual": max_res,
        "niter": [i["niter"] for i in infos], "nconv": [i["nconv"] for i in infos],
        "fp64_niter": r64.niter, "fp64_nconv": r64.nconv,
        "phase_ms_last_step": infos[-1]["phase_ms"], "phase_ms_fp64": r64.info["phase_ms"],
        "gpu_launches": sum(i["kernel_launches"] for i in infos),
        "escalated_solves": sum(i.get("precision_escalation_iter", 0) > 0 for i in infos),
        "e2e": {"value": e2e_pairs / t_e2e, "unit": UNIT,
                "h2d_bytes_per_step": int(A.indptr.nbytes + A.indices.nbytes + A.data.nbytes
                                          + B.indptr.nbytes + B.indices.nbytes + B.data.nbytes),
                "d2h_bytes_per_step": int(8 * c["nev_max"] * (1 + A.n)), "steps": 1},
        "roofline": {"kernel": "k_block_pcg<float,40> (persistent block PCG of the W step)",
                     "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None, "peak_kind": peak_kind,
                     "traffic": None,
                     "bytes_per_launch": pcg_bytes / max(1, pcg_launches),
                     "ms_per_launch": pcg_ms / max(1, pcg_launches), "launches": pcg_launches},
        "cpu_baseline": {"value": None, "unit": UNIT, "cores": 1, "kind": "port",
                         "sample": "not sampled at this size (the numpy restatement would hold "
                                   "6.7 GB per basis); see the default workload's line"},
        "clocks": clk,
    }
    if d.rank == 0:
        print(json.dumps(line), flush=True)


def solve_once(args):
    import gcge_gb300 as G
    G.load(build_if_missing=True)
    c, X0 = build_workload(args.size)
    prep = G.Prepared(c["A"], c["B"], c["nev"], c["block_size"], c["nev_init"], c["nev_max"], X0=X0,
                      precision=G.PREC_MIXED if args.solve_once == "mixed" else G.PREC_FP64)
    r = prep.solve()
    prep.close()
    print(json.dumps({"nconv": r.nconv, "niter": r.niter, "status": r.status,
                      "kernel_launches": r.info["kernel_launches"]}))
    return 0 if r.status == G.GCGE_OK else 1


def main():
    args = parse()
    if args.solve_once:
        sys.exit(solve_once(args))
    if args.impl == "reference":
        threads = args.threads or os.cpu_count() or 1
        os.environ["OPENBLAS_NUM_THREADS"] = str(threads)
        os.environ["OMP_NUM_THREADS"] = str(threads)
    d = Dist()
    try:
        if args.impl == "reference":
            run_reference(args, d)
        elif args.workload == "vardiff3d":
            run_vardiff(args, d)
        else:
            run_ours(args, d)
    finally:
        d.close()


if __name__ == "__main__":
    main()
