"""Benchmark: converged eigenpairs/s of the Krylov-Schur path on one GB300 (replicas on N GPUs).

Default workload (one "step" = one complete EPSSolve): 3-D 7-point Laplacian 128^3 (n = 2,097,152,
nnz = 14,581,760, FP64 CSR), EPS_HEP, nev = 50 largest algebraic, ncv = 128, tol = 1e-10, start vector
uniform[-1,1] (splitmix64, seed 2).  The basis alone is 2.2 GB, far larger than the 129 MB L2, so no flush is needed
between steps.

  value      nev converged eigenpairs per solve / device time of EPSSolve (CUDA events on the solver's stream),
             matrix resident in HBM since EPSSetUp (the start vector's 16.8 MB upload is inside EPSSolve).
             Arithmetic: IEEE FP64 storage (--arith f64, the default); Gram-Schmidt products exact on the integer
             pipes, each result rounded once (--gs auto: the library's default for this size; --gs fma for FP64 FMA)
  parity     after the timed solves, on the host: every converged eigenvalue against the closed-form spectrum
             (set-based over distinct values), ||Ax - lam x|| / (||A||_inf |lam|) with scipy.sparse on the CSR
             arrays, ||X^T X - I|| in numpy, from the eigenvectors EPSGetEigenpair returns; exit code 3 if a bound fails
  pair       the same workload in FP32-pair arithmetic (narrower than FP64), reported beside the headline
  e2e        the same metric through the public C-ABI from host buffers: MatCreateSeqAIJWithArrays + EPSSetUp (CSR
             host->device) + EPSSolve + EPSGetEigenpair for all nev (eigenvectors device->host), host wall clock
  roofline   the dominant kernel class of one profiled solve: algorithmic bytes / summed CUDA-event time
  cpu_baseline  the oracle (CPU restatement of SLEPc's Krylov-Schur) on the host cores for a bounded time, scaled
             by Krylov steps to the full solve

  python bench.py [--gpus N --steps K --warmup W] [--impl reference] [--workload lap3d128|lap2d100|convdiff1000]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "lap3d128": dict(desc="3-D 7-point Laplacian 128^3 (n=2097152, nnz=14581760, FP64 CSR), EPS_HEP, nev=50 "
                          "largest algebraic, ncv=128, tol=1e-10, start vector uniform[-1,1] seed 2",
                     gen=lambda mg: mg.laplacian_3d(128), exact=lambda mg: mg.laplacian_eigenvalues([128] * 3),
                     hermitian=True, which="LR", nev=50, ncv=128, tol=1e-10, seed=2),
    "lap2d100": dict(desc="2-D 5-point Laplacian 100x100 (n=10000, nnz=49600), EPS_HEP, nev=10 largest magnitude, "
                          "ncv=32, tol=1e-8, start vector seed 1",
                     gen=lambda mg: mg.laplacian_2d(100), exact=lambda mg: mg.laplacian_eigenvalues([100, 100]),
                     hermitian=True, which="LM", nev=10, ncv=32, tol=1e-8, seed=1),
    "lap3d64": dict(desc="3-D 7-point Laplacian 64^3 (n=262144, nnz=1810432), EPS_HEP, nev=50 largest algebraic, "
                         "ncv=128, tol=1e-10, start vector seed 2 (the 128^3 solve's shape at 1/8 size, for profiling)",
                    gen=lambda mg: mg.laplacian_3d(64), exact=lambda mg: mg.laplacian_eigenvalues([64] * 3),
                    hermitian=True, which="LR", nev=50, ncv=128, tol=1e-10, seed=2),
    "chunglu4m": dict(desc="Chung-Lu power-law graph n=4194304, mean degree 32, gamma 2.1, max degree 1e5 (seed 4), "
                           "weights U(0,1] (seed 5), normalised adjacency D^-1/2 A D^-1/2 (nnz 125,195,026), EPS_HEP, "
                           "nev=16 largest algebraic, ncv=48, tol=1e-10, start vector seed 4",
                      gen=lambda mg: mg.chung_lu(4194304), hermitian=True, which="LR", nev=16, ncv=48, tol=1e-10,
                      seed=4),
    "convdiff1000": dict(desc="2-D upwind convection-diffusion 1000x1000 (n=1e6), Peclet 10, EPS_NHEP, nev=20 "
                              "largest real, ncv=64, tol=1e-10, start vector seed 3",
                         gen=lambda mg: mg.convection_diffusion_2d(1000, 10.0),
                         exact=lambda mg: mg.convdiff_eigenvalues(1000, 10.0), hermitian=False, which="LR", nev=20,
                         ncv=64, tol=1e-10, seed=3),
}
BATCH = dict(desc="4096 independent EPS_HEP problems, n_i = round(exp(U[ln 1000, ln 65536])) (splitmix64 seed 6+i), "
                  "2-D 5-point Laplacian on an r x c grid (r = floor(sqrt n_i), c = ceil(n_i/r)) plus diag(U[0,1]) "
                  "(seed 6+i), nev=8 largest magnitude, ncv=24, tol=1e-10, start vector seed 6+i",
             count=4096, nev=8, ncv=24, tol=1e-10, which="LM")
METRIC = "converged eigenpairs/s at tol 1e-10 (plain Krylov-Schur, one solve per step)"
UNIT = "eigenpairs/s"


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi sampling of SM clock and throttle reasons during the timed region."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                                          "-i", str(self.index), "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        mhz = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(mhz) if mhz else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def committed_traffic(workload):
    """DRAM traffic / algorithmic bytes per kernel class from the committed ncu captures, if recorded."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get(workload)
    return None


def full_size_steps(workload):
    """Krylov steps of the complete reference-algorithm solve (oracle/full_size_runs.py), 0 if not recorded."""
    p = os.path.join(ROOT, "oracle", "full_size_runs.json")
    if os.path.exists(p):
        rec = json.load(open(p)).get(workload, {})
        here = rec.get("hosts", {}).get(os.uname().machine, {})  # the count of a solve on this kind of host
        return int(here.get("steps", rec.get("steps", 0)))
    return 0


def full_solves(workload, nev):
    """Complete oracle solves of the workload timed once per host (oracle/full_size_runs.json): eigenpairs/s of
    each, to set beside the bounded samples."""
    p = os.path.join(ROOT, "oracle", "full_size_runs.json")
    if not os.path.exists(p):
        return {}
    rec = json.load(open(p)).get(workload, {})
    runs = dict(rec.get("hosts", {}))
    if rec.get("seconds"):
        runs.setdefault(rec.get("host", "x86_64"), {k: rec[k] for k in ("seconds", "threads", "steps", "its")
                                                    if k in rec})
    return {h: dict(r, value=nev / r["seconds"]) for h, r in runs.items() if r.get("seconds")}


def cpu_baseline(csr, wl, steps_full, budget_s=20.0, nthreads=0):
    """Oracle (CPU restatement of the reference) on all host cores (or nthreads) for a bounded time; eigenpairs/s
    extrapolated by the number of Krylov steps of the full solve."""
    import oracle
    from slepc_gb300 import matgen

    oracle.build()
    cores = nthreads or os.cpu_count() or 1
    n = len(csr[0]) - 1
    t = time.time()
    r = oracle.solve(*csr, hermitian=wl["hermitian"], which=wl["which"], nev=wl["nev"], ncv=wl["ncv"], tol=wl["tol"],
                     v0=matgen.start_vector(n, wl["seed"]), nthreads=cores, vectors=False, time_budget=budget_s)
    el = time.time() - t
    finished = r.reason in (1, -1, -2)
    if finished:
        value = wl["nev"] / el
        sample = f"complete solve ({r.nsteps} Krylov steps, {r.its} restarts) in {el:.1f} s"
    else:
        per_step = el / max(r.nsteps, 1)
        est = per_step * steps_full
        value = wl["nev"] / est
        sample = (f"first {r.nsteps} Krylov steps ({r.its} restarts, {el:.1f} s) of the same solve, scaled to the "
                  f"full solve's {steps_full} steps")
    return {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample,
            "host": os.uname().machine}


def run_reference(args, wl):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from slepc_gb300 import matgen

    csr = wl["gen"](matgen)
    steps_full = full_size_steps(args.workload)
    budget = 20.0 if args.workload == "lap3d128" else 10.0
    vals = []
    for i in range(args.warmup + args.steps):
        b = cpu_baseline(csr, wl, steps_full or 5000, budget_s=budget if i >= args.warmup else 3.0)
        if i >= args.warmup:
            vals.append(b)
    v = statistics.median([b["value"] for b in vals])
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * wl["nev"] / v,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": wl["desc"], "impl": "oracle port of SLEPc 3.22 Krylov-Schur (CGS+IFNEEDED, "
                                                      "host DS), OpenMP over rows"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": vals[-1]["cores"], "kind": "port",
                             "sample": vals[-1]["sample"]},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    full = full_solves(args.workload, wl["nev"])
    if full:
        # the complete solve, timed once per host, beside the sampled value (the sample's early steps have fewer
        # basis columns than the average step, so the sample overstates the reference's speed)
        line["full_solve"] = full
        here = full.get(os.uname().machine)
        if here:
            line["sample_over_full"] = v / here["value"]
    print(json.dumps(line), flush=True)


def batch_instances(matgen, count):
    """The batched workload's matrices (CSR) and start-vector seeds."""
    out = []
    for i in range(count):
        u = matgen.uniform_01(6 + i, 1)[0]
        n = int(round(np.exp(np.log(1000.0) + u * (np.log(65536.0) - np.log(1000.0)))))
        out.append((matgen.laplacian_2d_randdiag(n, 6 + i), 6 + i))
    return out


def run_batch(args):
    """Batched form: all problems in one EPSGB300SolveBatch per step, beside the one-problem-per-launch EPSSolve
    path on a stratified sample of the same problems."""
    import slepc_gb300 as sg
    from slepc_gb300 import matgen
    from slepc_gb300.replicas import Replicas
    import ctypes

    sg.build()
    rep = Replicas()
    ctypes.CDLL("libcudart.so").cudaSetDevice(rep.local)
    count = args.batch_count or BATCH["count"]
    t = time.time()
    # replicas: each rank solves a round-robin share of the independent problems (no data-path collective)
    inst = rep.shard(batch_instances(matgen, count))
    gen_s = time.time() - t
    nsum = sum(len(c[0]) - 1 for c, _ in inst)

    def make(csr, seed, A=None):
        A = A or sg.Mat(*csr)
        e = sg.EPS().create()
        e.setOperators(A)
        e.setProblemType(sg.EPS.ProblemType.HEP)
        e.setDimensions(BATCH["nev"], BATCH["ncv"])
        e.setTolerances(BATCH["tol"])
        e.setWhichEigenpairs(BATCH["which"])
        e.setInitialSpace(matgen.start_vector(len(csr[0]) - 1, seed))
        if args.arith == "f32":
            e.setArithmetic("f32")  # the FP32-storage variant
        e._A = A
        return e

    if args.profile_solve:
        # the ncu launch-list case: one batched solve with the default tuning table
        eps = [make(c, sd) for c, sd in inst]
        for e in eps:
            e.setUp()
        sg.solve_batch(eps)
        print(json.dumps({"profile_solve": "batch", "instances": count,
                          "converged": sum(1 for e in eps if e.getConvergedReason() == 1)}), flush=True)
        return
    t = time.time()
    tuning = sg.batch_tune(1, 7) if not args.no_tune else sg.batch_get_tuning()
    tune_s = time.time() - t
    t = time.time()
    eps = [make(c, sd) for c, sd in inst]
    for e in eps:
        e.setUp()
    setup_s = time.time() - t
    for _ in range(args.warmup):
        sg.solve_batch(eps)
    clocks = ClockSampler(rep.local)
    rep.barrier()
    clocks.start()
    times, conv = [], []
    for _ in range(args.steps):
        t = time.perf_counter()
        sg.solve_batch(eps)
        times.append(time.perf_counter() - t)
        conv.append(sum(BATCH["nev"] for e in eps if e.getConvergedReason() == 1 and e.getConverged() >= BATCH["nev"]))
    rep.barrier()
    clk = clocks.stop()
    # whole job: every rank's converged eigenpairs over the slowest rank's time
    value = rep.sum(sum(conv)) / rep.max(sum(times))
    its = [e.getIterationNumber() for e in eps]
    launches = eps[0].getStats()["kernel_launches"] * args.steps

    # the plain path: EPSSolve one problem at a time, on every (count/sample)-th problem in order of size
    count_local = len(inst)
    order = sorted(range(count_local), key=lambda i: len(inst[i][0][0]))
    sample = order[:: max(1, count_local // max(1, args.batch_plain_sample // rep.world))]
    plain_eps = [eps[i] for i in sample]
    for e in plain_eps[:3]:
        e.solve()
    t = time.perf_counter()
    pconv = 0
    for e in plain_eps:
        e.solve()
        pconv += BATCH["nev"] if (e.getConvergedReason() == 1 and e.getConverged() >= BATCH["nev"]) else 0
    plain_s = time.perf_counter() - t
    plain_value = pconv / plain_s

    # e2e: matrices from host CSR, setup, batched solve, every eigenpair back to the host
    e2e = None
    if not args.no_e2e:
        t = time.perf_counter()
        eps2 = [make(c, sd) for c, sd in inst]
        sg.solve_batch(eps2)
        d2h = 0
        for e in eps2:
            x = np.empty(e._A.m)
            for i in range(BATCH["nev"]):
                e.getEigenpair(i, x)
            d2h += BATCH["nev"] * (x.nbytes + 16)
        e2e_s = time.perf_counter() - t
        h2d = sum(c[0].nbytes + c[1].nbytes + c[2].nbytes + 8 * (len(c[0]) - 1) for c, _ in inst)
        e2e = {"value": sum(BATCH["nev"] for e in eps2 if e.getConvergedReason() == 1) / e2e_s, "unit": UNIT,
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h}
        for e in eps2:
            e.destroy()
    if rep.rank != 0:
        rep.close()
        return
    line = {"metric": METRIC.replace("plain Krylov-Schur", "batched Krylov-Schur"), "value": value, "unit": UNIT,
            "n_gpus": rep.world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * sum(times) / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": BATCH["desc"].replace("4096", str(count)), "instances": count, "sum_n": nsum,
                       "arith": args.arith, "parallelism": f"replicas x{rep.world} (problems sharded round-robin)",
                       "l2": "inputs larger than L2 (bases 13 GB)",
                       "restarts_per_instance": {"min": min(its), "median": float(np.median(its)), "max": max(its)},
                       "generate_s": round(gen_s, 1), "setup_s": round(setup_s, 1),
                       "tuning": {"tiles_per_virtual_block_by_bucket": tuning, "tune_s": round(tune_s, 1)}},
            "plain": {"value": plain_value, "unit": UNIT, "sample": f"{len(plain_eps)} of {count} problems "
                      "(every k-th by size), EPSSolve one at a time", "seconds": plain_s},
            "speedup_vs_plain": value / plain_value, "e2e": e2e, "clocks": clk, "gpu_launches": launches}
    print(json.dumps(line), flush=True)
    rep.close()


SERVED = dict(desc="served stream: Poisson arrivals at each rate for the window; per request n = exp(U[ln 2e3, ln 2e6]); "
                   "70% EPS_HEP Laplacian + diag(U[0,1]) (3-D m^3 when n > 2e5, else 2-D near-square), 30% EPS_NHEP "
                   "upwind convection-diffusion N^2 with Pe ~ U[1,50]; nev ~ U{4..32}, ncv = max(2 nev + 8, 24), "
                   "tol = 1e-10, largest real; every request's matrix generated for it on arrival (no shared pool); "
                   "seed 7")


def served_request(matgen, i, seed=7):
    """Request i of the stream: (kind, n, Pe, nev, ncv, start seed), from its own splitmix64 draws."""
    u = matgen.uniform_01(seed * 1000003 + i, 5)
    n = float(np.exp(np.log(2e3) + u[0] * (np.log(2e6) - np.log(2e3))))
    nev = 4 + min(28, int(u[2] * 29))
    ncv = max(2 * nev + 8, 24)
    if u[1] < 0.7:
        kind = "hep3" if n > 2e5 else "hep2"
        pe = 0.0
    else:
        kind = "nhep"
        pe = 1.0 + 49.0 * float(u[3])
    return kind, int(round(n)), pe, nev, ncv, 1000 + i


def served_matrix(matgen, kind, n, pe, i):
    if kind == "hep3":
        m = max(2, int(round(n ** (1.0 / 3.0))))
        return matgen.laplacian_3d_randdiag(m, 7 + i)
    if kind == "hep2":
        return matgen.laplacian_2d_randdiag(n, 7 + i)
    N = max(2, int(round(np.sqrt(n))))
    return matgen.convection_diffusion_2d(N, pe)


def run_served(args):
    """Served form at the stated arrival rates: for each rate, Poisson arrivals for one window, every request's
    matrix generated when it arrives and submitted to EPSGB300Server (continuous batching, HBM-budget admission),
    then a bounded drain.  Latency runs from the scheduled arrival to the result, so generator lag and queueing
    count.  A request that arrives while max_queue requests are unfinished is refused at the door and counted as
    dropped."""
    import slepc_gb300 as sg
    from slepc_gb300 import matgen
    import ctypes

    sg.build()
    ctypes.CDLL("libcudart.so").cudaSetDevice(0)
    rates = [float(r) for r in args.served_rates.split(",")]
    W, drain, budget = args.served_window, args.served_drain, args.served_budget_gb * 1e9
    max_queue = args.served_max_queue
    clocks = ClockSampler(0)
    clocks.start()
    per_rate = []
    base = 0
    # finished requests are released on a thread of their own: freeing device memory waits for the device to go
    # idle, which would stall the arrival loop behind the solves in flight (the client hands results off)
    import queue
    grave = queue.Queue()

    def release():
        while True:
            e = grave.get()
            if e is None:
                return
            A = getattr(e, "_A", None)
            e.destroy()
            if A is not None:
                A.destroy()

    releaser = threading.Thread(target=release, daemon=True)
    releaser.start()
    for rate in rates:
        srv = sg.Server(budget, max_requests=4096, max_ncv=72)
        rng = np.random.default_rng(7 + int(rate))
        arrivals = np.cumsum(rng.exponential(1.0 / rate, size=int(rate * W * 1.5) + 16))
        arrivals = arrivals[arrivals < W]
        live = []          # (request, eps, scheduled arrival, submit time)
        finished = []      # (request, latency s, converged)
        dropped = 0
        lock = threading.Lock()
        t0 = time.perf_counter()

        def reap(block_until=None):
            """Collect finished requests without blocking (or until a deadline)."""
            nonlocal live
            keep = []
            for r, e, arr, sub in live:
                try:
                    done = srv.wait(e, 0.0 if block_until is None else max(0.0, block_until - time.perf_counter()))
                except sg.SlepcError:
                    done = True
                if done:
                    st = e.getStats()
                    ok = e.getConvergedReason() == 1 and e.getConverged() >= r[3]
                    finished.append((r, (sub - t0 - arr) + st["solve_seconds"], ok))
                    grave.put(e)
                else:
                    keep.append((r, e, arr, sub))
            live = keep

        gen_s = 0.0
        for k, arr in enumerate(arrivals):
            r = served_request(matgen, base + k)
            now = time.perf_counter() - t0
            if now > W:
                dropped += len(arrivals) - k  # arrivals the generator could not reach within the window
                break
            reap()
            if len(live) >= max_queue:
                dropped += 1
                continue
            g0 = time.perf_counter()
            csr = served_matrix(matgen, r[0], r[1], r[2], base + k)
            A = sg.Mat(*csr)
            e = sg.EPS().create()
            e.setOperators(A)
            e.setProblemType(sg.EPS.ProblemType.NHEP if r[0] == "nhep" else sg.EPS.ProblemType.HEP)
            e.setDimensions(r[3], r[4])
            e.setTolerances(1e-10)
            e.setWhichEigenpairs("LR")
            e.setInitialSpace(matgen.start_vector(A.m, r[5]))
            e._A = A
            gen_s += time.perf_counter() - g0
            wait = t0 + arr - time.perf_counter()
            if wait > 0:
                time.sleep(wait)
            srv.submit(e)
            live.append((r, e, arr, time.perf_counter()))
        base += len(arrivals)
        end = t0 + W + drain
        while live and time.perf_counter() < end:
            reap(block_until=min(end, time.perf_counter() + 0.5))
        incomplete = len(live)
        srv.cancel()
        for r, e, arr, sub in live:
            try:
                srv.wait(e)
            except sg.SlepcError:
                pass
        st = srv.stats()
        srv.destroy()
        for r, e, arr, sub in live:
            grave.put(e)
        live = []
        lat = sorted(x[1] for x in finished if x[2])
        conv = sum(x[0][3] for x in finished if x[2])
        per_rate.append({"rate_per_s": rate, "offered": int(len(arrivals)), "submitted": int(len(arrivals) - dropped),
                         "dropped_at_door": int(dropped), "completed": len(lat), "incomplete_after_drain": incomplete,
                         "p50_ms": 1000.0 * float(np.percentile(lat, 50)) if lat else None,
                         "p99_ms": 1000.0 * float(np.percentile(lat, 99)) if lat else None,
                         "eigenpairs_per_s": conv / (W + drain), "peak_admitted_bytes": st["peak_bytes"],
                         "max_live": st["max_live"], "host_generate_s": round(gen_s, 1)})
        print(json.dumps({"served_rate": per_rate[-1]}), file=sys.stderr, flush=True)
    grave.put(None)
    releaser.join()
    clk = clocks.stop()
    best = max(per_rate, key=lambda x: x["eigenpairs_per_s"])
    line = {"metric": METRIC.replace("plain Krylov-Schur, one solve per step", "served Krylov-Schur stream"),
            "value": best["eigenpairs_per_s"], "unit": UNIT, "n_gpus": 1, "steps": len(rates), "warmup": 0,
            "ms_per_step": 1000.0 * (W + drain), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "pair", "data": "synthetic",
            "config": {"workload": SERVED["desc"], "window_s": W, "drain_s": drain, "hbm_budget_gb": args.served_budget_gb,
                       "max_queue": max_queue, "arith": "pair (the batched engine's arithmetic)"},
            "rates": per_rate, "clocks": clk}
    print(json.dumps(line), flush=True)


def run_batch_reference(args):
    """The reference algorithm (the oracle port of SLEPc's Krylov-Schur) on the host cores, one problem after
    another as the reference would solve them, over a stratified sample of the batched workload."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import oracle
    from slepc_gb300 import matgen

    oracle.build()
    count = args.batch_count or BATCH["count"]
    inst = batch_instances(matgen, count)
    order = sorted(range(count), key=lambda i: len(inst[i][0][0]))
    sample = order[:: max(1, count // 64)]
    cores = os.cpu_count() or 1
    vals = []
    for k in range(args.warmup + args.steps):
        t = time.time()
        conv = 0
        for i in (sample[:4] if k < args.warmup else sample):
            csr, seed = inst[i]
            r = oracle.solve(*csr, hermitian=True, which=BATCH["which"], nev=BATCH["nev"], ncv=BATCH["ncv"],
                             tol=BATCH["tol"], v0=matgen.start_vector(len(csr[0]) - 1, seed), nthreads=cores,
                             vectors=False)
            conv += BATCH["nev"] if (r.reason == 1 and r.nconv >= BATCH["nev"]) else 0
        if k >= args.warmup:
            vals.append(conv / (time.time() - t))
    v = statistics.median(vals)
    line = {"impl": "reference", "metric": METRIC.replace("plain Krylov-Schur", "batched Krylov-Schur"), "value": v,
            "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * BATCH["nev"] * len(sample) / v, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": BATCH["desc"].replace("4096", str(count)),
                       "impl": "oracle port of SLEPc 3.22 Krylov-Schur, one problem at a time, OpenMP over rows"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{len(sample)} of {count} problems (every k-th by size), complete solves"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="lap3d128", choices=list(WORKLOADS) + ["batch4096", "served"])
    ap.add_argument("--served-rates", default="50,100,200,500,1000,2000",
                    help="Poisson arrival rates (requests/s) of the served runs, one window each")
    ap.add_argument("--served-drain", type=float, default=30.0, help="seconds of drain after each window")
    ap.add_argument("--served-max-queue", type=int, default=256,
                    help="unfinished requests the host holds before refusing arrivals at the door")
    ap.add_argument("--served-budget-gb", type=float, default=200.0, help="HBM budget of the server")
    ap.add_argument("--served-window", type=float, default=60.0, help="seconds of each served measurement")
    ap.add_argument("--batch-count", type=int, default=0, help="problems in the batched workload (default 4096)")
    ap.add_argument("--batch-plain-sample", type=int, default=256,
                    help="problems of the batched workload timed through the one-problem-per-launch path")
    ap.add_argument("--arith", default="f64", choices=["pair", "f64", "f32"],
                    help="f64: IEEE FP64 storage (the headline); pair: FP32-pair arithmetic (reported beside "
                         "it); f32: the precision form")
    ap.add_argument("--restart", default="tensor", choices=["tensor", "pair", "mma_sync", "tcgen05"],
                    help="kernel of the thick restart (EPSGB300SetRestartMethod)")
    ap.add_argument("--gs", default="auto", choices=["auto", "tensor", "fma", "integer"],
                    help="Gram-Schmidt of the f64 arithmetic: the library's default (exact integer products, FP64 FMA "
                         "where segments replay from graphs), exact products on the integer pipes, FP64 FMA, or exact "
                         "products on the tensor cores")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-parity", action="store_true", help="skip the host-side parity block")
    ap.add_argument("--no-pair", action="store_true", help="skip the pair-arithmetic line beside the FP64 one")
    ap.add_argument("--no-tune", action="store_true", help="batched workload: keep the default tuning table")
    ap.add_argument("--profile-case", action="store_true",
                    help="run exactly one solve limited to 2 restarts and exit (the ncu capture case)")
    ap.add_argument("--profile-solve", action="store_true",
                    help="run exactly one complete solve and exit (the ncu launch-list case: same work as a step)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.workload == "served":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the served stream has no CPU counterpart here; "
                              "the reference arm is measured on the single-problem and batched workloads"}))
            return
        run_served(args)
        return
    if args.workload == "batch4096":
        if args.impl == "reference":
            run_batch_reference(args)
            return
        run_batch(args)
        return
    wl = WORKLOADS[args.workload]
    if args.impl == "reference":
        run_reference(args, wl)
        return
    run_plain(args, wl)


# FP64 FMA throughput of this GPU (DFMA microbenchmark: 1.20 TFLOP/s).  A Gram-Schmidt half does two FMAs per 8-byte
# basis entry (0.5 flop/byte), so IEEE FP64 Gram-Schmidt is bounded at 1.20e12 * 2 = 2.4 TB/s, below the HBM rate.
DFMA_TFLOPS = 1.20
GS_LABEL = {"integer": "Gram-Schmidt products exact on the integer pipes (54-bit fixed point, exact integer sums, "
                       "one rounding per result)",
            "fma": "Gram-Schmidt in IEEE FP64 FMA",
            "tensor": "Gram-Schmidt products exact on the tensor cores (Ozaki slices)"}
ARITH_LABEL = {"f64": "IEEE FP64 storage, FP64 arithmetic elsewhere",
               "pair": "FP32-pair storage and arithmetic (hi+lo floats, 47-bit significand, ~2^-46 per product)",
               "f32": "FP32 storage, pair accumulation, FP64-class refinement sweep"}


def eigenpairs(eps, n, count):
    """The first `count` converged eigenpairs through EPSGetEigenpair (real parts; vectors as returned)."""
    lams = np.zeros(count)
    imag = np.zeros(count)
    X = np.empty((n, count))
    x = np.empty(n)
    for i in range(count):
        lam = eps.getEigenpair(i, x)
        lams[i] = lam.real if isinstance(lam, complex) else lam
        imag[i] = lam.imag if isinstance(lam, complex) else 0.0
        X[:, i] = x
    return lams, imag, X


def parity_of(eps, csr, wl, n):
    """Host-side parity of the solve left in `eps`: eigenvalues against the closed-form spectrum (set-based),
    residuals with scipy.sparse on the caller's CSR and ||X^T X - I|| in numpy (slepc_gb300.verify)."""
    from slepc_gb300 import matgen, verify

    nconv = eps.getConverged()
    lams, imag, X = eigenpairs(eps, n, nconv)
    real = imag == 0.0
    exact = wl["exact"](matgen) if wl.get("exact") else None
    if exact is not None:
        p = verify.parity_block(csr, lams[real], X[:, real], exact, wl["which"], wl["nev"], wl["tol"],
                                hermitian=wl["hermitian"])
    else:
        r_a, r_l = verify.residuals(csr, lams[real], X[:, real])
        p = {"checked": "residuals and orthogonality (no closed form)", "converged": int(nconv),
             "max_rel_residual": float(r_a.max()), "max_residual_over_lambda": float(r_l.max()),
             "orth_err": verify.orthogonality(X) if wl["hermitian"] else None, "tol": wl["tol"]}
        p["ok"] = bool(p["max_rel_residual"] <= wl["tol"] and (p["orth_err"] is None or p["orth_err"] <= 1e-12))
    p["complex_pairs"] = int(np.sum(~real))
    del X
    return p


def run_plain(args, wl):
    import ctypes

    import slepc_gb300 as sg
    from slepc_gb300 import matgen
    from slepc_gb300.replicas import Replicas

    sg.build()
    rep = Replicas()
    rank, world, local = rep.rank, rep.world, rep.local
    ctypes.CDLL("libcudart.so").cudaSetDevice(local)

    csr = wl["gen"](matgen)
    n = len(csr[0]) - 1
    nnz = len(csr[1])
    v0 = matgen.start_vector(n, wl["seed"])

    def make_eps(A, arith):
        eps = sg.EPS().create()
        eps.setOperators(A)
        eps.setProblemType(sg.EPS.ProblemType.HEP if wl["hermitian"] else sg.EPS.ProblemType.NHEP)
        eps.setDimensions(wl["nev"], wl["ncv"])
        eps.setTolerances(wl["tol"])
        eps.setWhichEigenpairs(wl["which"])
        eps.setArithmetic(arith)
        eps.setRestartMethod(args.restart)
        if arith == "f64":
            eps.setGSMethod(args.gs)
        eps.setInitialSpace(v0)
        return eps

    barrier = rep.barrier
    max_over_ranks = rep.max

    A = sg.Mat(*csr)
    eps = make_eps(A, args.arith)
    if args.profile_case:
        eps.setTolerances(wl["tol"], 2)
        eps.setUp()
        eps.solve()
        print(json.dumps({"profile_case": args.workload, "stats": eps.getStats()}), flush=True)
        return
    if args.profile_solve:
        eps.setUp()
        eps.setProfiling(True)
        eps.solve()
        prof = eps.getProfile()
        print(json.dumps({"profile_solve": args.workload, "arith": args.arith, "gs": args.gs, "restart": args.restart,
                          "stats": eps.getStats(), "per_class_ms": {k: round(v[0], 3) for k, v in prof.items()}}),
              flush=True)
        return

    def timed(e, steps, warmup, clocks=None):
        """warmup untimed solves, then `steps` solves: device time (CUDA events on the solver's stream), wall
        latency, launches, converged counts."""
        e.setUp()
        for _ in range(warmup):
            e.solve()
        barrier()
        if clocks:
            clocks.start()
        r = {"dev_ms": [], "lat": [], "launches": 0, "nconv": [], "steps": [], "restarts": []}
        for _ in range(steps):
            e.solve()
            st = e.getStats()
            r["dev_ms"].append(st["solve_device_ms"])
            r["lat"].append(st["solve_seconds"] * 1000.0)
            r["launches"] += st["kernel_launches"]
            r["nconv"].append(e.getConverged())
            r["steps"].append(st["krylov_steps"])
            r["restarts"].append(st["restarts"])
        barrier()
        r["clk"] = clocks.stop() if clocks else None
        r["total_ms"] = max_over_ranks(sum(r["dev_ms"]))
        assert min(r["nconv"]) >= wl["nev"], f"solve did not converge ({r['nconv']})"
        r["value"] = world * steps * wl["nev"] / (r["total_ms"] / 1000.0)
        return r

    def roofline_of(e, arith):
        """One profiled solve: per kernel class device time and algorithmic bytes; the dominant class's rate."""
        e.setProfiling(True)
        e.solve()
        prof = e.getProfile()
        e.setProfiling(False)
        exact_gs = bool(e.getStats()["gs_exact"])
        peak, peak_kind = measured_peaks()
        top = max(("gs_dot", "gs_update", "spmv", "restart"), key=lambda k: prof[k][0])
        ms_k, by_k, nl_k = prof[top]
        achieved = by_k / (ms_k / 1000.0) / 1e9 if ms_k > 0 else None
        tkey = args.workload + ("" if arith == "pair" else "_" + arith) + ("_integer" if exact_gs else "")
        tr = (committed_traffic(tkey) or committed_traffic(tkey.replace("_integer", "")) or {}).get(top)
        traffic = tr * by_k / nl_k if (tr and nl_k) else None  # DRAM bytes per launch: ncu ratio x algorithmic
        roof = {"bound": "hbm", "kernel": top, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak if achieved else None, "peak_source": peak_kind,
                "traffic": traffic, "algorithmic_bytes_per_launch": by_k / nl_k if nl_k else None,
                "launches": nl_k,
                "per_class_ms": {k: round(v[0], 3) for k, v in prof.items()},
                "per_class_GBps": {k: (round(v[1] / (v[0] / 1000.0) / 1e9, 1) if v[0] > 0 else None)
                                   for k, v in prof.items()}}
        krylov_ms = sum(prof[k][0] for k in ("spmv", "gs_dot", "gs_update"))
        krylov_bytes = sum(prof[k][1] for k in ("spmv", "gs_dot", "gs_update"))
        roof["krylov_step_GBps"] = round(krylov_bytes / (krylov_ms / 1000.0) / 1e9, 1) if krylov_ms > 0 else None
        roof["krylov_step_frac"] = round(roof["krylov_step_GBps"] / peak, 4) if krylov_ms > 0 else None
        roof["solve_bytes"] = sum(v[1] for v in prof.values())
        if arith == "f64" and not exact_gs:
            # the FP64 pipe bounds FMA Gram-Schmidt before HBM does: 2 DFMA per 8-byte entry
            bound = DFMA_TFLOPS * 1e12 * 2.0 / 1e9
            roof["fp64_fma_bound"] = {
                "dfma_tflops": DFMA_TFLOPS, "gs_flop_per_byte": 0.5, "bound_GBps": bound,
                "gs_dot_frac": (roof["per_class_GBps"]["gs_dot"] or 0.0) / bound,
                "gs_update_frac": (roof["per_class_GBps"]["gs_update"] or 0.0) / bound}
        return roof

    clocks = ClockSampler(local)
    main_run = timed(eps, args.steps, args.warmup, clocks)
    par = parity_of(eps, csr, wl, n) if (rank == 0 and not args.no_parity) else None

    # e2e: public API from host buffers, per step: CSR + start vector host->device, solve, eigenpairs device->host
    e2e = None
    if not args.no_e2e:
        e2e_times = []
        h2d = csr[0].nbytes + csr[1].nbytes + csr[2].nbytes + v0.nbytes
        d2h = wl["nev"] * (n * 8 + 16)
        for _ in range(args.steps):
            barrier()
            t = time.perf_counter()
            Ae = sg.Mat(*csr)
            e = make_eps(Ae, args.arith)
            e.solve()
            x = np.empty(n)
            for i in range(wl["nev"]):
                e.getEigenpair(i, x)
            e.destroy()
            Ae.destroy()
            barrier()
            e2e_times.append(time.perf_counter() - t)
        e2e_t = max_over_ranks(sum(e2e_times))
        e2e = {"value": world * args.steps * wl["nev"] / e2e_t, "unit": UNIT, "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h}

    roofline = roofline_of(eps, args.arith)
    stats = eps.getStats()
    gs_used = args.gs if args.gs != "auto" else ("integer" if stats["gs_exact"] else "fma")

    # the pair arithmetic beside the headline, labelled as what it is (narrower than IEEE FP64)
    pair = None
    if args.arith != "pair" and not args.no_pair and args.workload in ("lap3d128", "lap3d64", "lap2d100"):
        ep = make_eps(A, "pair")
        pr = timed(ep, max(1, min(args.steps, 2)), 1)
        pair = {"value": pr["value"], "unit": UNIT, "arith": "pair", "dtype": ARITH_LABEL["pair"],
                "ms_per_step": pr["total_ms"] / len(pr["dev_ms"]), "steps": len(pr["dev_ms"]),
                "krylov_steps_per_solve": pr["steps"][-1], "restarts_per_solve": pr["restarts"][-1],
                "nconv": pr["nconv"][-1]}
        rp = roofline_of(ep, "pair")
        pair["roofline"] = {k: rp[k] for k in ("kernel", "achieved", "peak", "frac", "per_class_ms",
                                               "per_class_GBps", "krylov_step_frac")}
        if rank == 0 and not args.no_parity:
            pair["parity"] = parity_of(ep, csr, wl, n)
        ep.destroy()

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(csr, wl, full_size_steps(args.workload) or main_run["steps"][-1])
        one = cpu_baseline(csr, wl, full_size_steps(args.workload) or main_run["steps"][-1], budget_s=10.0,
                           nthreads=1)
        cpu["one_thread"] = {"value": one["value"], "cores": 1, "sample": one["sample"]}

    if rank == 0:
        lat_sorted = sorted(main_run["lat"])
        line = {"metric": METRIC, "value": main_run["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": main_run["total_ms"] / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.arith == "f64" else args.arith,
                "data": "synthetic",
                "config": {"workload": wl["desc"], "n": n, "nnz": nnz, "arith": args.arith,
                           "arith_detail": ARITH_LABEL[args.arith] + ("; " + GS_LABEL[gs_used]
                                                                      if args.arith == "f64" else ""),
                           "gs": gs_used if args.arith == "f64" else None, "restart": args.restart,
                           "parallelism": f"replicas x{world}", "l2": "inputs larger than L2 (basis 2.2 GB)"
                           if args.workload == "lap3d128" else "small inputs",
                           "krylov_steps_per_solve": main_run["steps"][-1],
                           "restarts_per_solve": main_run["restarts"][-1],
                           "precision_phase_steps": stats["precision_steps"], "nconv": main_run["nconv"][-1]},
                "latency_ms": {"p50": float(np.percentile(lat_sorted, 50)),
                               "p99": float(np.percentile(lat_sorted, 99))},
                "parity": par, "e2e": e2e, "roofline": roofline, "pair": pair, "cpu_baseline": cpu,
                "clocks": main_run["clk"], "gpu_launches": main_run["launches"]}
        print(json.dumps(line), flush=True)
        if par is not None and not par["ok"]:
            print(f"parity check failed: {par}", file=sys.stderr, flush=True)
            rep.close()
            sys.exit(3)
    rep.close()


if __name__ == "__main__":
    main()
