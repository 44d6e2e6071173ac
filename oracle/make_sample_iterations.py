"""Iteration counts of the oracle's FP64 Jacobi-PCG on every system of the
seeded serving-stream sample (the default workload of bench.py), written to
oracle/serving_sample_iterations.json.

The CPU reference arm of bench.py cannot run the sample's largest requests to
completion within its time bound (a 1.3M-unknown LSCM system needs ~10^5
iterations); it times a fixed number of iterations of those systems on the
host cores and scales the per-iteration time to the counts recorded here,
which this script obtains by running the same oracle to completion.

Usage: python oracle/make_sample_iterations.py [--requests 12] [--seed 20261203]
"""
import argparse
import json
import sys
import time
from pathlib import Path

HERE = Path(__file__).resolve().parent
# the script's own folder would shadow the `oracle` package with oracle.py
sys.path = [p for p in sys.path if Path(p or ".").resolve() != HERE]
sys.path.insert(0, str(HERE.parent))

from graphitethree_gb300 import systems  # noqa: E402
from oracle import oracle  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--requests", type=int, default=12)
    ap.add_argument("--seed", type=int, default=20261203)
    ap.add_argument("--rate", type=float, default=1000.0)
    ap.add_argument("--eps", type=float, default=1e-10)
    ap.add_argument("--out", default=str(HERE / "serving_sample_iterations.json"))
    a = ap.parse_args()
    reqs, objs = systems.serving_sample(a.requests, a.seed, a.rate)
    out = {"requests": a.requests, "seed": a.seed, "rate": a.rate, "eps": a.eps,
           "threads": oracle.max_threads(), "systems": []}
    for i, (kind, o) in enumerate(objs):
        t0 = time.perf_counter()
        rp, ci, va, rhs = oracle.assemble_rowstream(o if kind == "rows" else o.to_rows())
        its, sts = [], []
        for s in range(rhs.shape[0]):
            _, st, it, _ = oracle.pcg(rp, ci, va, rhs[s], eps=a.eps)
            its.append(it)
            sts.append(st)
        rec = {"request": i, "kind": reqs[i].kind, "unknowns": int(rp.shape[0] - 1), "nnz": int(rp[-1]),
               "iterations": its, "status": sts, "seconds_here": round(time.perf_counter() - t0, 2)}
        out["systems"].append(rec)
        print(json.dumps(rec), flush=True)
    Path(a.out).write_text(json.dumps(out, indent=1) + "\n")


if __name__ == "__main__":
    main()
