"""Benchmark: k-eigenvalue MoC solves per second on one GB300.

Default workload (``--workload branch256``): 256 independent branch-case
eigenvalue solves of uneven size, lattices drawn uniformly from {1x1, 3x3,
7x7, 17x17} pins (24 FSR/pin), each perturbing moderator Sigma_t/scattering
by U[0.9, 1.1] and fuel nu-Sigma_f by U[0.95, 1.05] of a seeded synthetic
7-group library; 8 azimuths/octant (32 over 2pi), 3 Tabuchi-Yamamoto polar
angles, 0.05 cm spacing, CMFD on the pin mesh, k_tol 1e-6, psi_tol 1e-5,
n_inner 5, reflective boundaries. FP32 sweep, FP64 k/fission source/CMFD.
One step = all 256 solves from flat-flux start to convergence through the
batch engine (continuous batching, one captured CUDA graph per outer
iteration, work-unit and segment-ring shapes chosen by the autotuner).

Printed JSON (one line, rank 0):
  value          solves/s: solves / device time of the graph replays (CUDA
                 events on the engine's stream), inputs resident in HBM
  e2e            solves/s through the public API from host buffers: submit
                 (cross-section parse + upload, state initialisation), the
                 solves, and the device->host read of k and pin powers
  plain          the plain single-solve GPU path (one EigenSolver per case,
                 same precision) over the same 256 cases, and the speed-up
  serving        a Poisson request stream at 50-2000 requests/s (lattice
                 sizes weighted 0.4/0.3/0.2/0.1, 7 or 23 groups, given as
                 MOCC input text): solves/s, p50/p99 latency overall and per
                 class with each request's phases (host, queue, run,
                 collect), host setup time per request
  accuracy       k error (pcm) and max fuel-pin power error of every one of
                 the 256 batched solves against the FP64 CPU oracle (which
                 traces each input itself); served results likewise, one per
                 (lattice size, group count) class
  roofline       the batched sweep kernel: algorithmic bytes of its launches /
                 their CUDA-event device time in a single-engine pass over
                 the same 256 solves, against the measured HBM copy
                 bandwidth (overall and for the launches with all 256
                 solves active)
  cpu_baseline   the CPU oracle (FP64 OpenMP restatement of MOCC) solving one
                 case of each size with all host threads
L2 is flushed (256 MB write) before every timed step; within a step the four
shared traced geometries (~35 MB of segment streams) stay in the 129 MB L2 by
design, while the per-solve state (~0.2 GB for 256 solves) does not fit.

--workload pin3x3 / assembly17 / minicore: one solve of that single lattice
per step (the 3x3 pin lattice, the 17x17 assembly at 0.03 cm, or the
68x68-pin mini-core with vacuum reflector faces), mixed precision timed, with the plain FP64 path's time and
its k / pin-power difference, the sweep kernel's roofline, and a full FP64
solve of the oracle with the accuracy of both paths.

--impl reference times the reference's CPU algorithm (the oracle port:
MOCC itself cannot be built without Blitz++, Eigen, pugixml and HDF5) with
all host threads on the same workload: each step solves one case of each
lattice size, reported as solves/s of that mixture. The oracle reads each
case's MOCC input text and traces it with its own restatement of MOCC's
tracer: this arm loads no part of the GPU library.

--profile-once: one untimed and one NVTX-marked run of the workload, for
profilers (see profile_once).
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

N_CASES = 256
SIZES = (1, 3, 7, 17)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="branch256", choices=["branch256", "pin3x3", "assembly17", "minicore"])
    ap.add_argument("--cases", type=int, default=N_CASES)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU oracle legs")
    ap.add_argument("--no-serve", action="store_true", help="skip the served request stream")
    ap.add_argument("--profile-once", action="store_true",
                    help="for profilers: one untimed run of the workload, then one more inside an NVTX range "
                         "named mocgpu_timed (branch256: one batch of --cases solves in one engine; assembly17 / "
                         "minicore: one solve); prints a JSON summary, no benchmark line")
    ap.add_argument("--bundles-per-unit", type=int, default=1, help="work-unit shape for --profile-once")
    ap.add_argument("--sweep-ring", type=int, default=0, help="segment-ring shape index for --profile-once")
    return ap.parse_args()


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

    NAMES = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]

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
        rows = [[c.strip() for c in r.split(",")] for r in Path(self.f.name).read_text().strip().splitlines()
                if r.strip()]
        os.unlink(self.f.name)
        rows = [r for r in rows if len(r) > 8]
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = sorted({n for r in rows for n, v in zip(self.NAMES, r[5:9]) if v == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def l2_copy_gbs():
    """Copy bandwidth of a buffer that stays in L2 (two 32 MB halves, read +
    write bytes, best of 20 batches of 50 copies, CUDA events): the ceiling
    of a kernel whose data is L2-resident."""
    import torch
    a = torch.empty(32 << 20, dtype=torch.uint8, device="cuda")
    b = torch.empty_like(a)
    b.copy_(a)
    best = 0.0
    for _ in range(20):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(50):
            b.copy_(a)
        e1.record()
        e1.synchronize()
        best = max(best, 2 * a.numel() * 50 / (e0.elapsed_time(e1) / 1e3) / 1e9)
    return best


def secondary_ceilings(achieved_gbs, sgu_per_s, clk):
    """The sweep against the two other ceilings of its path: the L2 copy
    bandwidth (its data is L2-resident on the branch workload) and the
    exponential throughput (6 ex2 per segment-group update, 16 per clock per
    SM nominal, at the SM clock sampled during the run)."""
    l2 = l2_copy_gbs()
    mhz = (clk or {}).get("sm_mhz") or 2070.0
    sfu = 16 * 152 * mhz * 1e6 / 6
    return {"l2_copy_gbs": l2, "frac_of_l2": achieved_gbs / l2 if achieved_gbs else None,
            "sfu_sgu_per_s": sfu, "frac_of_sfu": sgu_per_s / sfu if sgu_per_s else None,
            "how": "l2: copy of a 32 MB buffer (read + write bytes), best of 20 x 50, CUDA events; sfu: nominal"}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic(name="kb_sweep_fast_dram_branch256.md", key="traffic_bytes_per_launch"):
    """DRAM bytes of the sweep from a committed ncu summary (None if absent)."""
    p = ROOT / "profiles" / name
    if p.exists():
        for line in p.read_text().splitlines():
            if line.startswith(key + ":"):
                return float(line.split(":")[1])
    return None


def pcm(k, k_ref):
    return 1e5 * abs(k - k_ref) / k_ref


def max_pin_err(p, p_ref):
    import numpy as np
    p, p_ref = np.ravel(p), np.ravel(p_ref)
    mask = p_ref > 0
    return float(np.max(np.abs(p[mask] - p_ref[mask]) / p_ref[mask]))


def branch_workload(n_cases, seed=7):
    """256 seeded branch cases; one traced base problem per lattice size."""
    import mocc_gb300 as m
    from mocc_gb300 import workloads as W
    cases = W.branch_cases(n_cases, seed=seed)
    bases = {}
    for size, ng, xml, xsl in cases:
        if (size, ng) not in bases:
            bases[(size, ng)] = (m.Problem(xml, xsl), xml)
    reqs = [(bases[(size, ng)][0], xsl) for size, ng, xml, xsl in cases]
    return cases, bases, reqs


CONFIG = {"workload": "branch256: 256 eigenvalue solves, lattices uniform over 1x1/3x3/7x7/17x17 pins",
          "fsr_per_pin": 24, "groups": 7, "azimuthal": "32 over 2pi", "polar": "3 (Tabuchi-Yamamoto)",
          "spacing_cm": 0.05, "perturbation": "moderator x U[0.9,1.1], fuel nu-Sigma_f x U[0.95,1.05]",
          "cmfd": "pin mesh, BiCGSTAB", "tolerances": "k 1e-6, psi 1e-5", "n_inner": 5,
          "precision": "FP32 sweep, FP64 k/fission source/CMFD",
          "l2": "flushed (256 MB write) before each timed step; shared geometries (~35 MB) L2-resident within a step"}


def oracle_sample(cases, per_size=1):
    """(index, xml, xsl) of the first `per_size` cases of each lattice size."""
    out, seen = [], {}
    for i, (size, ng, xml, xsl) in enumerate(cases):
        if seen.get(size, 0) < per_size:
            seen[size] = seen.get(size, 0) + 1
            out.append((i, xml, xsl))
    return out


def run_reference(args, rank, world):
    """The reference's algorithm on the host cores: the FP64 oracle, which
    reads each case's MOCC input text and traces it with its own
    restatement of MOCC's tracer (no part of the GPU library is loaded).
    Each step solves one case of each lattice size (a bounded sample of the
    workload), reported as solves/s of that mixture."""
    if rank != 0:
        return
    import oracle
    from mocc_gb300 import workloads as W
    config = CONFIG
    what = ("each step: one full FP64 solve of one case of each lattice size (1x1, 3x3, 7x7, 17x17) of the 256, "
            "each traced by the oracle from its MOCC input text before the timed steps")
    if args.workload in SINGLE:
        # one full solve of the single lattice per step, as the GPU arm times
        xml, xsl = getattr(W, args.workload)(precision="mixed")
        solvers = [oracle.OracleSolver.from_xml(xml, xsl)]
        config = {"workload": SINGLE[args.workload], "segments": solvers[0].n_seg,
                  "l2": "flushed (256 MB write) before each timed solve"}
        what = "each step: one full FP64 solve, traced by the oracle from the MOCC input text before the timed steps"
    else:
        cases = W.branch_cases(args.cases, seed=7)
        solvers = [oracle.OracleSolver.from_xml(xml, xsl) for _, xml, xsl in oracle_sample(cases)]

    def step():
        for O in solvers:
            O.solve()

    for _ in range(args.warmup):
        step()
    times = []
    for _ in range(args.steps):
        t = time.perf_counter()
        step()
        times.append(time.perf_counter() - t)
    t_step = statistics.median(times)
    v = len(solvers) / t_step
    line = {"impl": "reference", "metric": "solves/s", "value": v, "unit": "solves/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config,
            "cpu_baseline": {"value": v, "unit": "solves/s", "cores": solvers[0].threads, "kind": "port",
                             "sample": what},
            "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_branch(args, rank, world):
    import numpy as np
    import torch

    import mocc_gb300 as m
    from mocc_gb300 import workloads as W
    from mocc_gb300.serve import PHASES, Request, poisson_arrivals, run_batch, serve
    from mocc_gb300.tune import tune_sweep
    m.load_library()
    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    cases, bases, reqs = branch_workload(args.cases)
    n = len(reqs)
    n_pin_max = max(P.sizes["npin"] for P, _ in bases.values())

    # work-unit shape x segment-ring shape: autotuned on a 64-case sample
    tune = tune_sweep(lambda b: m.BatchEngine(precision=1, capacity=64, bundles_per_unit=b), reqs[:64])
    bpu, ring = tune["best"]["bundles_per_unit"], tune["best"]["shape"]

    def engine(**kw):
        e = m.BatchEngine(precision=1, bundles_per_unit=bpu, **kw)
        e.set_sweep_shape(ring)
        return e

    sizes = [size for size, ng, xml, xsl in cases]

    def plan_name(plan):
        if isinstance(plan, int):
            return f"{plan} round robin"
        return f"{plan[1]}: largest lattices on {plan[2]} of them"

    def lane_of(plan, i):
        """Lane of case i: round robin over n lanes, or ("size", n, b): the
        largest lattices round robin over b lanes of their own and the rest
        round robin over the other n - b."""
        if isinstance(plan, int):
            return i % plan
        _, nl, nb = plan
        big = max(sizes)
        return i % nb if sizes[i] == big else nb + i % (nl - nb)

    def make_lanes(plan):
        keys = sorted({lane_of(plan, i) for i in range(n)})
        cap = {k: sum(1 for i in range(n) if lane_of(plan, i) == k) for k in keys}
        return {k: engine(capacity=cap[k]) for k in keys}

    def timed_batch(lanes, plan):
        """One batch of all cases over the lanes; device span of the run from
        CUDA events on every lane's stream, and the results."""
        streams = {k: torch.cuda.ExternalStream(e.stream()) for k, e in lanes.items()}
        ev0 = {k: torch.cuda.Event(enable_timing=True) for k in lanes}
        ev1 = {k: torch.cuda.Event(enable_timing=True) for k in lanes}
        for k in lanes:
            ev0[k].record(streams[k])
        res = run_batch(lanes, [(P, x, lane_of(plan, i)) for i, (P, x) in enumerate(reqs)], n_pin_max)
        for k in lanes:
            ev1[k].record(streams[k])
        torch.cuda.synchronize()
        first = next(iter(lanes))
        span = max(ev0[first].elapsed_time(ev1[k]) for k in lanes) - min(
            ev0[first].elapsed_time(ev0[k]) for k in lanes)
        return span, res

    # lanes: one engine, or several engines on their own streams whose outer
    # iterations overlap on the GPU (one lane's latency-bound CMFD beside the
    # others' sweeps); the count is measured, not assumed
    lane_ms = {}
    for plan in (1, 2, 3, 4, ("size", 3, 1), ("size", 4, 2), ("size", 5, 2), ("size", 5, 3)):
        L = make_lanes(plan)
        timed_batch(L, plan)
        lane_ms[plan] = timed_batch(L, plan)[0]
        for e in L.values():
            e.close()
    plan = min(lane_ms, key=lane_ms.get)
    lanes = make_lanes(plan)
    for _ in range(args.warmup):
        timed_batch(lanes, plan)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    barrier(world)
    torch.cuda.synchronize()
    clocks = Clocks()
    l0 = m.launch_count()
    h0, d0 = m.copy_bytes()
    wall, span_ms = 0.0, 0.0
    results = None
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sp, results = timed_batch(lanes, plan)
        wall += time.perf_counter() - t0
        span_ms += sp
    launches = m.launch_count() - l0
    h1, d1 = m.copy_bytes()
    barrier(world)
    clk = clocks.stop()
    for e in lanes.values():
        e.close()

    span_ms = max_over_ranks(span_ms, world)
    wall = max_over_ranks(wall, world)
    value = world * n * args.steps / (span_ms / 1e3)
    e2e = world * n * args.steps / wall
    assert all(r["error"] == 0 and r["converged"] == 1 for r in results), [r for r in results if r["error"]][:2]
    peak, peak_kind = measured_peaks()

    # Roofline pass: the same 256 solves in one engine with CUDA events
    # around every sweep launch (the lanes of the timed run overlap their
    # sweeps with each other's CMFD, which would stretch each launch's
    # events); replays stepped one at a time, so the launches made while all
    # 256 solves are active are reported on their own.
    RE = engine(capacity=n)
    RE.set_pipeline_depth(1)
    for P, x in reqs:
        RE.submit(P, x)
    RE.run()  # captures the graph
    RE.set_timing(True)
    ids = [RE.submit(P, x) for P, x in reqs]
    flush.zero_()
    torch.cuda.synchronize()
    full = {"sweep_ms": 0.0, "sweep_bytes": 0.0, "sweep_launches": 0, "sweep_sgu": 0}
    tot = dict(full)
    replay_ms = 0.0
    while True:
        s0 = RE.stats()
        active_before = s0["active"] + s0["queued"]
        left = RE.step()
        s1 = RE.stats()
        replay_ms += s1["replay_ms"] - s0["replay_ms"]
        for k in full:
            d = s1[k] - s0[k]
            tot[k] += d
            if active_before == n:
                full[k] += d
        if left == 0 and s1["queued"] == 0:
            break
    for i in ids:
        RE.take(i)
    RE.close()
    achieved = tot["sweep_bytes"] / (tot["sweep_ms"] / 1e3) / 1e9
    achieved_full = full["sweep_bytes"] / (full["sweep_ms"] / 1e3) / 1e9 if full["sweep_ms"] else None

    # plain single-solve GPU path on the same cases (sequential, one handle each)
    plain_t, plain_k = [], []
    for P, x in reqs:
        S = m.MoCSweeper(P, 1, xsl=x)
        torch.cuda.synchronize()
        t = time.perf_counter()
        r = m.EigenSolver(P, sweeper=S).solve()
        torch.cuda.synchronize()
        plain_t.append(time.perf_counter() - t)
        plain_k.append(r["k"])
        S.close()
    plain = n / sum(plain_t)
    k_vs_plain = max(pcm(r["k"], k) for r, k in zip(results, plain_k))

    line = {"metric": "solves/s", "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": span_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": CONFIG,
            "setup": {"cases": n, "bundles_per_unit": bpu,
                      "sweep_ring": {"rows": tune["best"]["rows"], "stages": tune["best"]["stages"]},
                      "lanes": plan_name(plan), "replicas": world, "pipeline_depth": 2},
            "lanes_ms_per_batch": {plan_name(k): v for k, v in lane_ms.items()},
            "sgu_per_s": tot["sweep_sgu"] / (tot["sweep_ms"] / 1e3),
            "sgu_per_s_whole_run": world * args.steps * sum(
                r["iterations"] * CONFIG["groups"] * CONFIG["n_inner"] * bases[(c[0], c[1])][0].sizes["nseg"]
                for r, c in zip(results, cases)) / (span_ms / 1e3),
            "e2e": {"value": e2e, "unit": "solves/s", "h2d_bytes_per_step": int((h1 - h0) / args.steps),
                    "d2h_bytes_per_step": int((d1 - d0) / args.steps)},
            "plain": {"value": plain, "unit": "solves/s", "speedup": value / plain, "speedup_e2e": e2e / plain,
                      "k_max_diff_pcm_vs_batched": k_vs_plain,
                      "what": "sequential EigenSolver solves of the same cases, FP32 sweep, one handle each"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": profiled_traffic(),
                         "traffic_note": "DRAM bytes per launch from profiles/kb_sweep_fast_dram_branch256.md "
                                         "(launches with all 256 solves active): the shared geometries stay in L2",
                         "kernel": "kb_sweep_fast",
                         "bytes_per_launch": tot["sweep_bytes"] / max(tot["sweep_launches"], 1),
                         "ms_per_launch": tot["sweep_ms"] / max(tot["sweep_launches"], 1), "peak_source": peak_kind,
                         "measured": "one batch of the 256 solves in one engine after the timed run, CUDA events "
                                     "on the engine's stream around every sweep launch, L2 flushed before it",
                         "all_256_active": {"achieved": achieved_full,
                                            "frac": achieved_full / peak if achieved_full else None,
                                            "launches": full["sweep_launches"],
                                            "ms_per_launch": full["sweep_ms"] / max(full["sweep_launches"], 1)},
                         "sweep_share_of_replay": tot["sweep_ms"] / replay_ms,
                         "secondary": secondary_ceilings(achieved, tot["sweep_sgu"] / (tot["sweep_ms"] / 1e3), clk)},
            "tuning": tune, "clocks": clk, "gpu_launches": int(launches),
            "outer_iterations": int(sum(r["iterations"] for r in results))}

    # served request stream: Poisson arrivals at several rates; requests come
    # as MOCC input text (the engine traces each distinct lattice once)
    serve_cases = []
    if not args.no_serve:
        scases = W.branch_cases(512, seed=11, weights=(0.4, 0.3, 0.2, 0.1), groups=(7, 23))
        # one lane per (group count, lattice class): small solves (1x1, 3x3)
        # do not wait on the replays of large ones, 7-group solves not on
        # 23-group ones; the lanes' iterations overlap on the GPU
        def lane_of_s(size, ng):
            return (ng, "small" if size <= 3 else "large")

        keys = [(ng, c) for ng in (7, 23) for c in ("small", "large")]
        free_b = torch.cuda.mem_get_info()[0]
        SE = {k: engine(capacity=256, mem_budget=0.8 * free_b / len(keys)) for k in keys}
        # one outer iteration in flight per lane: a lane admits arriving
        # requests only between its replays, and with a second replay queued
        # behind the first an arrival waits for both (measured: at 400 req/s
        # p50 33 ms at depth 1 against 196 ms at depth 2, the same solves/s)
        for e in SE.values():
            e.set_pipeline_depth(1)
        warm = [Request(xml, xsl, 0.0, lane_of_s(size, ng)) for size, ng, xml, xsl in scases[:96]]
        serve(SE, warm, n_pin_max)  # traces the lattices, captures the graphs
        st0 = {k: e.stats() for k, e in SE.items()}
        runs = []
        for rate, nreq in ((50.0, 100), (100.0, 200), (400.0, 512), (1600.0, 512), (2000.0, 512)):
            arr = poisson_arrivals(nreq, rate, seed=5)
            rq = [Request(xml, xsl, float(a), lane_of_s(size, ng))
                  for (size, ng, xml, xsl), a in zip(scases[:nreq], arr)]
            rep = serve(SE, rq, n_pin_max)
            per_class = {}
            for (size, ng, _, _), lat, ph in zip(scases[:nreq], rep.latencies_s, rep.phases_s):
                per_class.setdefault(f"{size}x{size} {ng}g", []).append((lat, ph))

            def pct(v, q):
                return 1e3 * float(np.percentile(v, q))

            def phase_ms(rows):
                return {p: 1e3 * float(np.mean([ph[p] for _, ph in rows])) for p in PHASES}

            slow = sorted(zip(rep.latencies_s, rep.phases_s), key=lambda x: x[0])[-max(1, nreq // 100):]
            runs.append({"rate_req_per_s": rate, "requests": nreq, "solves_per_s": rep.solves_per_s,
                         "p50_ms": rep.percentile_ms(50), "p99_ms": rep.percentile_ms(99),
                         "per_class_ms": {c: {"n": len(v), "p50": pct([x[0] for x in v], 50),
                                              "p99": pct([x[0] for x in v], 99),
                                              "queue_p50": pct([x[1]["queue"] for x in v], 50),
                                              "run_p50": pct([x[1]["run"] for x in v], 50)}
                                          for c, v in sorted(per_class.items())},
                         "slowest_1pct_phases_ms": phase_ms(slow),
                         "all_ok": all(r is not None and r["error"] == 0 for r in rep.results)})
            if rate == 400.0:
                serve_cases = [(c, r) for c, r in zip(scases[:nreq], rep.results)]
        st1 = {k: e.stats() for k, e in SE.items()}
        req = sum(st1[k]["submitted"] - st0[k]["submitted"] for k in SE)
        line["serving"] = {"runs": runs, "mix": "sizes 1/3/7/17 weighted 0.4/0.3/0.2/0.1, groups 7 or 23",
                           "budget": "80% of free device memory, split between the lanes", "capacity": 256,
                           "lanes": "one engine per (group count, lattice class 1-3 / 7-17 pins), pipelined on "
                                    "four streams, one outer iteration in flight per lane",
                           "latency": "request arrival to result read on the host; phases: host (arrival to "
                                      "submit), queue (submit to admission into a slot), run (admission to the "
                                      "replay that retired it), collect (to the host read)",
                           "setup_ms_per_request": {
                               "trace": sum(st1[k]["trace_ms"] - st0[k]["trace_ms"] for k in SE) / req,
                               "cross_sections": sum(st1[k]["xs_ms"] - st0[k]["xs_ms"] for k in SE) / req,
                               "traces_reused": sum(st1[k]["trace_hits"] - st0[k]["trace_hits"] for k in SE),
                               "traces_made": sum(st1[k]["trace_misses"] - st0[k]["trace_misses"] for k in SE),
                               "what": "host time per request in submit: the ray trace (once per distinct "
                                       "lattice input, cached) and the cross-section read"}}
        for e in SE.values():
            e.close()

    if rank == 0 and not args.no_cpu:
        import oracle
        # every batched result against the FP64 oracle, which traces each
        # case's input itself
        errs, tcpu, cores, sgu, nsamp = [], 0.0, None, 0, 0
        for i, (size, ng, xml, xsl) in enumerate(cases):
            O = oracle.OracleSolver.from_xml(xml, xsl)
            t = time.perf_counter()
            ro = O.solve()
            dt = time.perf_counter() - t
            cores = O.threads
            if i in {j for j, _, _ in oracle_sample(cases)}:
                tcpu += dt
                sgu += ro["sweeps"] * O.n_seg
                nsamp += 1
            errs.append((size, pcm(results[i]["k"], ro["k"]), max_pin_err(results[i]["pin_powers"],
                                                                           O.pin_powers())))
        by = {}
        for size, e, pe in errs:
            b = by.setdefault(size, [0, 0.0, 0.0])
            b[0] += 1
            b[1] = max(b[1], e)
            b[2] = max(b[2], pe)
        line["accuracy"] = {"vs": "FP64 CPU oracle on its own trace of the same input", "cases": len(errs),
                            "by_size": {f"{s}x{s}": {"n": v[0], "k_err_pcm_max": v[1], "max_pin_err": v[2]}
                                        for s, v in sorted(by.items())},
                            "k_err_pcm_max": max(e for _, e, _ in errs), "max_pin_err": max(p for _, _, p in errs),
                            "tolerance": {"k_pcm": 10.0, "pin": 1e-3}}
        if serve_cases:
            # one served result per (lattice size, group count) class
            seen, serr = set(), []
            for (size, ng, xml, xsl), r in serve_cases:
                if (size, ng) in seen or r is None:
                    continue
                seen.add((size, ng))
                O = oracle.OracleSolver.from_xml(xml, xsl)
                ro = O.solve()
                serr.append({"class": f"{size}x{size} {ng}g", "k_err_pcm": pcm(r["k"], ro["k"]),
                             "max_pin_err": max_pin_err(r["pin_powers"], O.pin_powers())})
            line["serving"]["accuracy"] = {"vs": "FP64 CPU oracle, one served result per class (400 req/s run)",
                                           "cases": serr, "k_err_pcm_max": max(e["k_err_pcm"] for e in serr),
                                           "max_pin_err": max(e["max_pin_err"] for e in serr)}
        # one thread, on the 3x3 case of the sample
        i3, xml3, xsl3 = next(c for c in oracle_sample(cases) if cases[c[0]][0] == 3)
        O1 = oracle.OracleSolver.from_xml(xml3, xsl3, n_threads=1)
        t = time.perf_counter()
        r1 = O1.solve()
        t1 = time.perf_counter() - t
        line["cpu_baseline"] = {"value": nsamp / tcpu, "unit": "solves/s", "cores": cores, "kind": "port",
                                "sample": "one full FP64 solve of one case of each lattice size (1x1, 3x3, 7x7, "
                                          "17x17) with all host threads, traced by the oracle",
                                "sgu_per_s": sgu / tcpu,
                                "single_thread": {"sample": "the 3x3 case", "solves_per_s": 1.0 / t1,
                                                  "sgu_per_s": r1["sweeps"] * O1.n_seg / t1}}
    if rank == 0:
        print(json.dumps(line), flush=True)


SINGLE = {
    "pin3x3": "pin3x3: 3x3 pins (24 FSRs each), 8 azimuths/octant, 3 polar, 0.05 cm",
    "assembly17": "assembly17: 17x17 assembly, 16 azimuths/octant, 3 polar, 0.03 cm",
    "minicore": "minicore: 3x3 assemblies of 17x17 pins (3 fuel compositions) + a 21.42 cm reflector row on "
                "two sides (68x68 pins), vacuum on the reflector sides, 16 azimuths/octant, 3 polar, 0.03 cm",
}


def run_single(args, rank, world):
    """One solve of a single lattice per step (the 17x17 assembly or the
    mini-core), mixed precision timed; the plain FP64 path and a full FP64
    solve of the oracle on the same input alongside."""
    import numpy as np
    import torch

    import mocc_gb300 as m
    from mocc_gb300 import workloads as W
    m.load_library()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    xml, xsl = getattr(W, args.workload)(precision="mixed")
    P = m.Problem(xml, xsl)

    def timed(precision, steps, warmup):
        S = m.MoCSweeper(P, precision)
        E = m.EigenSolver(P, sweeper=S)
        stream = torch.cuda.ExternalStream(S.stream())
        flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
        for _ in range(warmup):
            E.solve()
        ms, r = [], None
        for _ in range(steps):
            flush.zero_()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            r = E.solve()
            e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        return S, r, ms

    clocks = Clocks()
    l0 = m.launch_count()
    S, r, ms_steps = timed(1, args.steps, args.warmup)
    launches = m.launch_count() - l0
    clk = clocks.stop()
    value = world * args.steps / (max_over_ranks(sum(ms_steps), world) / 1e3)
    pins = S.pin_powers()
    db, sweep_bytes = S.bytes()
    ms, nl = S.time_sweep(0, 20)
    achieved = sweep_bytes / (ms / 20 / 1e3) / 1e9 if nl else None
    S64, r64, ms64 = timed(0, 1, 1)
    pins64 = S64.pin_powers()
    peak, peak_kind = measured_peaks()
    line = {"metric": "solves/s", "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": statistics.median(ms_steps), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": SINGLE[args.workload], "segments": P.sizes["nseg"],
                       "l2": "flushed (256 MB write) before each timed solve"},
            "k": r["k"], "outer_iterations": r["iterations"],
            "plain_fp64": {"ms_per_solve": ms64[0], "k": r64["k"],
                           "mixed_vs_fp64_pcm": pcm(r["k"], r64["k"]), "mixed_vs_fp64_pin": max_pin_err(pins, pins64)},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak if achieved else None,
                         "traffic": profiled_traffic("k_sweep_fast_minicore.md", "traffic_bytes_per_group_sweep")
                         if args.workload == "minicore" else None,
                         "traffic_note": "DRAM bytes of one group sweep (two launches, the unit of `achieved` "
                                         "here) from profiles/k_sweep_fast_minicore.md"
                         if args.workload == "minicore" else "not captured for this workload",
                         "kernel": "k_sweep_fast",
                         "peak_source": peak_kind,
                         "secondary": secondary_ceilings(achieved, P.sizes["nseg"] / (ms / 20 / 1e3) if nl else None,
                                                         clk)},
            "clocks": clk, "gpu_launches": int(launches)}
    if rank == 0 and not args.no_cpu:
        import oracle
        # a full FP64 solve by the oracle, on its own trace of the same input
        O = oracle.OracleSolver.from_xml(xml, xsl)
        t = time.perf_counter()
        ro = O.solve()
        tc = time.perf_counter() - t
        line["cpu_baseline"] = {"value": 1.0 / tc, "unit": "solves/s", "cores": O.threads, "kind": "port",
                                "sample": "one full FP64 solve, traced by the oracle",
                                "outer_iterations": ro["iterations"]}
        pref = O.pin_powers()
        line["accuracy"] = {"vs": "FP64 CPU oracle on its own trace of the same input", "k_ref": ro["k"],
                            "k_err_pcm": pcm(r["k"], ro["k"]), "max_pin_err": max_pin_err(pins, pref),
                            "fp64_k_err_pcm": pcm(r64["k"], ro["k"]), "fp64_max_pin_err": max_pin_err(pins64, pref),
                            "tolerance": {"k_pcm": 10.0, "pin": 1e-3}}
    if rank == 0:
        print(json.dumps(line), flush=True)


def profile_once(args):
    """One untimed run, then one inside the NVTX range ``mocgpu_timed`` so
    that a profiler can restrict itself to the second, e.g.

        ncu --nvtx --nvtx-include "mocgpu_timed/" --metrics gpu__time_duration.sum \\
            --clock-control none --csv --log-file launches.csv python bench.py --profile-once --cases 256
    """
    import torch

    import mocc_gb300 as m
    from mocc_gb300 import workloads as W
    m.load_library()
    if args.workload in SINGLE:
        P = m.Problem(*getattr(W, args.workload)(precision="mixed"))
        S = m.MoCSweeper(P, 1)
        E = m.EigenSolver(P, sweeper=S)
        E.solve()
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push("mocgpu_timed")
        t = time.perf_counter()
        r = E.solve()
        torch.cuda.synchronize()
        wall = time.perf_counter() - t
        torch.cuda.nvtx.range_pop()
        print(json.dumps({"workload": args.workload, "wall_s": wall, "k": r["k"], "iterations": r["iterations"],
                          "converged": r["converged"]}))
        return 0 if r["converged"] else 1
    cases, bases, reqs = branch_workload(args.cases)
    E = m.BatchEngine(precision=1, capacity=max(1, args.cases), bundles_per_unit=args.bundles_per_unit)
    E.set_sweep_shape(args.sweep_ring)

    def batch():
        ids = [E.submit(P, x) for P, x in reqs]
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
    print(json.dumps({"cases": args.cases, "wall_s": wall, "replay_ms": s1["replay_ms"] - s0["replay_ms"],
                      "replays": s1["graph_replays"] - s0["graph_replays"], "all_converged": ok}))
    return 0 if ok else 1


def main():
    args = parse()
    if args.profile_once:
        raise SystemExit(profile_once(args))
    rank, world = dist_init(args)
    if args.impl == "reference":
        run_reference(args, rank, world)
    elif args.workload in SINGLE:
        run_single(args, rank, world)
    else:
        run_branch(args, rank, world)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
