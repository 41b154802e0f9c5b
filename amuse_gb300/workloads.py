"""Workload runners for the benchmark configurations other than the headline
one (which is bench.py).  Each prints one JSON line.

  python -m amuse_gb300.workloads batch   [--nsys 4096] [--exact-sample 256]
      Config 4: nsys few-body systems, n ~ U[3, 64], Plummer with virial
      radius 1e-3, eps = 0, to 10 crossing times, smallN's scheme
      (g6x_batch_run) after the autotuner; systems/s, p50/p99 per-system
      GPU time, the bit-identical (exact) mode on a sample, and the oracle's
      smallN restatement on the host cores for the same sample.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def run_batch(args):
    import amuse_gb300 as ag
    from amuse_gb300 import ic
    import oracle
    oracle.build_port()
    ns, m, x, v, tcr = ic.encounter_batch(args.nsys, 3, 64, r_vir=1e-3, seed=args.seed)
    t_end = 10 * tcr
    off = np.concatenate([[0], np.cumsum(ns)])
    g6 = ag.G6X(0)
    out = {"workload": f"{args.nsys} few-body systems, n~U[3,64], Plummer r_vir=1e-3, eps=0, "
                       f"t_end=10 t_cross={t_end:.4g}, eta={args.eta}, smallN scheme "
                       f"(n_iter=2, Kepler criterion), FP64, step cap {args.max_steps}/system"}

    # 1. parity: exact mode on the first systems, truncated at a step budget,
    #    against the oracle (smallN restated) on the host
    k = min(args.exact_sample, args.nsys)
    sub = slice(0, off[k])
    re = g6.batch_run(ns[:k], t_end, m[sub], x[sub], v[sub], eta=args.eta,
                      max_steps=args.exact_steps, exact=True)
    same = True
    for s in range(k):
        a, b = off[s], off[s + 1]
        px, pv, tf, st = oracle.smalln(m[a:b], x[a:b], v[a:b], args.eta, t_end,
                                       max_steps=args.exact_steps)
        same &= bool(np.array_equal(re["pos"][a:b], px) and np.array_equal(re["vel"][a:b], pv)
                     and re["steps"][s] == st)
    out["parity"] = {"systems": k, "step_budget": args.exact_steps,
                     "exact_mode_bit_identical_to_oracle": same}
    print(json.dumps(out), flush=True)

    # 2. autotune on 512 systems for 0.5% of the end time
    kt = min(args.nsys, 512)
    tune = g6.batch_tune(ns[:kt], t_end, m[:off[kt]], x[:off[kt]], v[:off[kt]], eta=args.eta,
                         frac=0.005)
    out["autotune"] = tune
    print(json.dumps(out), flush=True)

    # 3. GPU vs host cores on the same sample of systems (same step cap)
    kc = min(args.cpu_sample, args.nsys)
    sc = slice(0, off[kc])
    rg = g6.batch_run(ns[:kc], t_end, m[sc], x[sc], v[sc], eta=args.eta,
                      max_steps=args.max_steps)
    if not args.no_cpu:
        threads = os.cpu_count() or 1

        def one(s):
            a, b = off[s], off[s + 1]
            return oracle.smalln(m[a:b], x[a:b], v[a:b], args.eta, t_end,
                                 max_steps=args.max_steps)

        t1 = time.perf_counter()
        with cf.ThreadPoolExecutor(threads) as ex:
            list(ex.map(one, range(kc)))
        cdt = time.perf_counter() - t1
        out["sample_gpu_vs_cpu"] = {
            "systems": kc, "gpu_systems_per_s": kc / (rg["elapsed_ms"] / 1e3),
            "cpu_systems_per_s": kc / cdt, "cpu_cores": threads, "cpu_kind": "port",
            "gpu_mode": "fast"}
        print(json.dumps(out), flush=True)

    # 4. the full batch
    t0 = time.perf_counter()
    r = g6.batch_run(ns, t_end, m, x, v, eta=args.eta, max_steps=args.max_steps)
    wall = time.perf_counter() - t0
    done = r["status"] == 0
    out.update({
        "systems_per_s": args.nsys / (r["elapsed_ms"] / 1e3),
        "completed_systems_per_s": int(done.sum()) / (r["elapsed_ms"] / 1e3),
        "elapsed_ms_gpu": r["elapsed_ms"], "wall_s_incl_copies": wall,
        "per_system_ms": {"p50": float(np.percentile(r["wall_ms"], 50)),
                          "p99": float(np.percentile(r["wall_ms"], 99)),
                          "max": float(r["wall_ms"].max())},
        "steps": {"total": int(r["steps"].sum()), "p50": float(np.percentile(r["steps"], 50)),
                  "p90": float(np.percentile(r["steps"], 90)),
                  "p99": float(np.percentile(r["steps"], 99)), "max": int(r["steps"].max())},
        "completed": int(done.sum()), "capped": int((r["status"] == 1).sum()),
    })
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="cmd", required=True)
    b = sub.add_parser("batch")
    b.add_argument("--nsys", type=int, default=4096)
    b.add_argument("--seed", type=int, default=1)
    b.add_argument("--eta", type=float, default=0.14)
    b.add_argument("--max-steps", type=int, default=250_000)
    b.add_argument("--exact-sample", type=int, default=32)
    b.add_argument("--exact-steps", type=int, default=5_000)
    b.add_argument("--cpu-sample", type=int, default=64)
    b.add_argument("--no-cpu", action="store_true")
    a = ap.parse_args()
    if a.cmd == "batch":
        run_batch(a)


if __name__ == "__main__":
    main()
