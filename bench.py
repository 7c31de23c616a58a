"""Benchmark: k-eigenvalue MoC solves per second on one GB300.

Default workload: the 17x17 pin assembly (264 fuel + 25 guide-tube cells,
24 FSR/pin, 7 groups, 16 azimuths/octant, 3 polar, 0.03 cm spacing) solved
with the mixed-precision path (FP32 sweep, FP64 k/fission source/CMFD), CMFD
on, k_tol 1e-6, psi_tol 1e-5. One step = one full eigenvalue solve (flux
initialisation through convergence). Cross sections are the seeded synthetic
library (no benchmark data is used).

Printed JSON (one line, rank 0):
  value        solves/s with the traced problem resident in HBM
  e2e          solves/s through the C ABI from host buffers: sweeper creation
               (host->device upload of tracks, cross sections, geometry),
               the solve, and the device->host read of the pin powers
  roofline     the sweep kernel: algorithmic bytes per launch / CUDA-event
               duration, against the measured HBM copy bandwidth
  cpu_baseline the CPU oracle (FP64 OpenMP restatement of MOCC's sweep) on the
               same workload, all host threads
The segment stream of this workload (~23 MB) fits in L2; L2 is flushed
(256 MB write) before every timed solve.

--impl reference times the reference's CPU algorithm (the oracle port, since
MOCC itself cannot be built without its third-party dependencies) with all
host threads on the same workload: each step is one outer iteration, scaled to
solves/s by the outer-iteration count of a full solve.
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
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="assembly17", choices=["assembly17", "pin3x3", "minicore"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU oracle baseline")
    return ap.parse_args()


def workload(name):
    from mocc_gb300 import workloads as W
    if name == "assembly17":
        return W.assembly17(precision="mixed"), {"pins": "17x17 (264 fuel + 25 guide tube)", "groups": 7,
                                                   "azimuthal_per_octant": 16, "polar": 3, "spacing_cm": 0.03}
    if name == "pin3x3":
        return W.pin3x3(precision="mixed"), {"pins": "3x3", "groups": 7, "azimuthal_per_octant": 8, "polar": 3,
                                               "spacing_cm": 0.05}
    return W.minicore(precision="mixed"), {"pins": "68x68 (3x3 fuel assemblies + reflector row)", "groups": 7,
                                             "azimuthal_per_octant": 16, "polar": 3, "spacing_cm": 0.03}


def dist_init(args):
    rank, world = int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))
    if world > 1:
        import torch.distributed as dist
        backend = "gloo" if args.impl == "reference" else "nccl"
        dist.init_process_group(backend)
    return rank, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(v, world):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits", "-lms",
                                       "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait()
        self.f.flush()
        rows = [r.split(",") for r in Path(self.f.name).read_text().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm = [float(r[1]) for r in rows if len(r) > 8 and r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if len(r) > 8 and r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows if len(r) > 8 for n, v in zip(names, r[5:9]) if "Active" in v})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def run_reference(args, rank, world):
    if rank != 0:
        return
    import oracle
    import mocc_gb300 as m
    (xml, xsl), cfg = workload(args.workload)
    P = m.Problem(xml, xsl)
    O = oracle.OracleSolver(P)
    full = O.solve()  # outer-iteration count of a full solve (untimed)
    n_outer = full["iterations"]
    for _ in range(args.warmup):
        O.solve(max_outer=1)
    times = []
    for _ in range(args.steps):
        t = time.perf_counter()
        O.solve(max_outer=1)
        times.append(time.perf_counter() - t)
    t_outer = statistics.median(times)
    v = 1.0 / (t_outer * n_outer)
    line = {"impl": "reference", "metric": "solves/s", "value": v, "unit": "solves/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_outer,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.workload, **cfg},
            "cpu_baseline": {"value": v, "unit": "solves/s", "cores": O.threads, "kind": "port",
                             "sample": f"one outer iteration per step x {n_outer} outers per solve"},
            "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, rank, world):
    import numpy as np
    import torch

    import mocc_gb300 as m
    m.load_library()
    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    (xml, xsl), cfg = workload(args.workload)
    P = m.Problem(xml, xsl)
    S = m.MoCSweeper(P, 1)
    E = m.EigenSolver(P, sweeper=S)
    stream = torch.cuda.ExternalStream(S.stream())
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def solve_once():
        r = E.solve()
        assert r["converged"], r
        return r

    for _ in range(args.warmup):
        solve_once()
    barrier(world)
    torch.cuda.synchronize()
    clocks = Clocks()
    l0 = m.launch_count()
    ms_steps, results = [], []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        results.append(solve_once())
        e1.record(stream)
        e1.synchronize()
        ms_steps.append(e0.elapsed_time(e1))
    torch.cuda.synchronize()
    launches = m.launch_count() - l0
    barrier(world)
    clk = clocks.stop()
    total_ms = max_over_ranks(sum(ms_steps), world)
    value = world * args.steps / (total_ms / 1e3)
    r0 = results[-1]
    sgu = P.sizes["nseg"] * r0["sweeps"] / (statistics.median(ms_steps) / 1e3)

    # end to end through the C ABI from host buffers
    db, sweep_bytes = S.bytes()
    pins = None
    e2e_t = []
    for i in range(max(2, args.steps)):
        torch.cuda.synchronize()
        t = time.perf_counter()
        S2 = m.MoCSweeper(P, 1)
        r = m.EigenSolver(P, sweeper=S2).solve()
        pins = S2.pin_powers()
        S2.close()
        torch.cuda.synchronize()
        e2e_t.append(time.perf_counter() - t)
    e2e_v = world / max_over_ranks(statistics.median(e2e_t), world)
    h2d = db  # device arrays uploaded or initialised at creation
    d2h = pins.nbytes + 8 * 8

    # sweep-kernel roofline (CUDA events around the sweep launches only)
    reps = 20
    ms, nl = S.time_sweep(0, reps)
    per_launch_ms = ms / nl
    bytes_per_launch = sweep_bytes / (nl / reps)
    achieved = bytes_per_launch / (per_launch_ms / 1e3) / 1e9
    peak, peak_kind = measured_peaks()

    line = {"metric": "solves/s", "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": statistics.median(ms_steps), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": args.workload, **cfg, "precision": "FP32 sweep, FP64 k/fs/CMFD",
                       "l2": "flushed (256 MB write) before each timed solve", "replicas": world},
            "sgu_per_s": sgu, "outer_iterations": r0["iterations"], "sweeps_per_solve": r0["sweeps"],
            "k": r0["k"],
            "e2e": {"value": e2e_v, "unit": "solves/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": None, "kernel": "k_sweep", "bytes_per_launch": bytes_per_launch,
                         "ms_per_launch": per_launch_ms, "peak_source": peak_kind},
            "clocks": clk, "gpu_launches": int(launches)}
    if rank == 0 and not args.no_cpu:
        import oracle
        O = oracle.OracleSolver(P)
        t = time.perf_counter()
        ro = O.solve()
        tc = time.perf_counter() - t
        line["cpu_baseline"] = {"value": 1.0 / tc, "unit": "solves/s", "cores": O.threads, "kind": "port",
                                "sample": "one full FP64 solve of the same workload"}
        po = O.pin_powers()
        pg = S.pin_powers() if pins is None else pins
        mask = po > 0
        line["k_err_pcm"] = 1e5 * abs(r0["k"] - ro["k"]) / ro["k"]
        line["max_pin_err"] = float(np.max(np.abs(pg[mask] - po[mask]) / po[mask]))
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, world = dist_init(args)
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
