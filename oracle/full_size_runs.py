"""Full-size oracle solves of the benchmark workloads: Krylov steps and restarts of the reference algorithm.

The reference arm of bench.py times the oracle on a bounded sample (the first Krylov steps of the same solve) and
scales the time by the number of Krylov steps the complete solve needs; this script measures that number once, by
running the complete solve, and records it in full_size_runs.json beside this file.  The oracle is the CPU
restatement of SLEPc 3.22's Krylov-Schur (CGS with IFNEEDED refinement, FP64 LAPACK-style projected solvers), so
the counts are those of the reference algorithm on the same matrix and start vector.

  python oracle/full_size_runs.py lap3d128 [lap3d64 convdiff1000 ...] [--threads T] [--out FILE]

--out writes the records to another file (a run on another host, merged into full_size_runs.json under the
workload's "hosts" entry by hand).
"""
import argparse
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))


def main():
    import bench
    import oracle
    from slepc_gb300 import matgen

    ap = argparse.ArgumentParser()
    ap.add_argument("workloads", nargs="+")
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--out", default=os.path.join(HERE, "full_size_runs.json"))
    args = ap.parse_args()
    oracle.build()
    path = args.out
    out = json.load(open(path)) if os.path.exists(path) else {}
    for name in args.workloads:
        wl = bench.WORKLOADS[name]
        csr = wl["gen"](matgen)
        n = len(csr[0]) - 1
        t = time.time()
        r = oracle.solve(*csr, hermitian=wl["hermitian"], which=wl["which"], nev=wl["nev"], ncv=wl["ncv"],
                         tol=wl["tol"], v0=matgen.start_vector(n, wl["seed"]), nthreads=args.threads, vectors=False)
        out[name] = {"n": n, "nconv": int(r.nconv), "its": int(r.its), "steps": int(r.nsteps),
                     "passes": int(r.npasses), "reason": int(r.reason), "seconds": round(time.time() - t, 1),
                     "threads": args.threads, "host": os.uname().machine,
                     "eigr": [float(x) for x in r.eigr[:wl["nev"]]]}
        print(name, json.dumps({k: v for k, v in out[name].items() if k != "eigr"}), flush=True)
        json.dump(out, open(path, "w"), indent=1)


if __name__ == "__main__":
    main()
