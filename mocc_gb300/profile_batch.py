"""One batched branch-case run (or one single solve) for profilers.

    python -m mocc_gb300.profile_batch [--cases 256] [--bundles-per-unit 1]
    python -m mocc_gb300.profile_batch --single assembly17 [--precision 1]

Runs the seeded branch-case batch (lattices uniform over 1x1/3x3/7x7/17x17
pins, perturbed cross sections) once to capture the graph, then once more
inside an NVTX range named ``mocgpu_timed`` so that a profiler can restrict
itself to the second run (with --single: one solve of that workload through
MoCSweeper + EigenSolver, warmed up by a first solve), e.g.

    ncu --nvtx --nvtx-include "mocgpu_timed/" --metrics gpu__time_duration.sum \\
        --clock-control none --csv --log-file launches.csv \\
        python -m mocc_gb300.profile_batch --cases 256
"""
from __future__ import annotations

import argparse
import json
import time


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--cases", type=int, default=256)
    ap.add_argument("--bundles-per-unit", type=int, default=1)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--single", choices=["assembly17", "minicore"], default=None)
    ap.add_argument("--precision", type=int, default=1)
    a = ap.parse_args(argv)

    import torch

    import mocc_gb300 as m
    from mocc_gb300 import workloads as W

    if a.single:
        prec = "mixed" if a.precision else "fp64"
        xml, xsl = getattr(W, a.single)(precision=prec)
        P = m.Problem(xml, xsl)
        S = m.MoCSweeper(P, a.precision)
        E = m.EigenSolver(P, sweeper=S)
        E.solve()
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push("mocgpu_timed")
        t = time.perf_counter()
        r = E.solve()
        torch.cuda.synchronize()
        wall = time.perf_counter() - t
        torch.cuda.nvtx.range_pop()
        print(json.dumps({"single": a.single, "precision": a.precision, "wall_s": wall, "k": r["k"],
                          "iterations": r["iterations"], "converged": r["converged"]}))
        return 0 if r["converged"] else 1

    cases = W.branch_cases(a.cases, seed=a.seed)
    bases = {}
    for size, ng, xml, xsl in cases:
        if (size, ng) not in bases:
            bases[(size, ng)] = m.Problem(xml, xsl)
    E = m.BatchEngine(precision=1, capacity=max(1, a.cases), bundles_per_unit=a.bundles_per_unit)

    def batch():
        ids = [E.submit(bases[(s, ng)], xsl) for s, ng, xml, xsl in cases]
        E.run()
        return [E.take(i) for i in ids]

    batch()
    torch.cuda.synchronize()
    s0 = E.stats()
    torch.cuda.nvtx.range_push("mocgpu_timed")
    t = time.perf_counter()
    res = batch()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t
    torch.cuda.nvtx.range_pop()
    s1 = E.stats()
    ok = all(r["error"] == 0 and r["converged"] for r in res)
    print(json.dumps({"cases": a.cases, "wall_s": wall, "replay_ms": s1["replay_ms"] - s0["replay_ms"],
                      "replays": s1["graph_replays"] - s0["graph_replays"], "all_converged": ok}))
    return 0 if ok else 1


if __name__ == "__main__":
    raise SystemExit(main())
