"""Request loop over batch engines: continuous batching of arriving solves.

Requests arrive on a schedule (a seeded Poisson process for the benchmark);
each is submitted as soon as its arrival time has passed to the engine
(lane) its key selects, the engine admits it into a free slot once its
geometry and state fit the device-memory budget, every active solve of a
lane advances one power iteration per graph replay, and results are
collected as solves retire. Lanes run on their own CUDA streams and are
stepped in a pipeline (each lane keeps up to its pipeline depth of outer
iterations in flight; the host collects a lane's oldest finished iteration
and launches its next, then moves on), so their iterations overlap on the
GPU: solves with few energy groups need not wait for the replays of
23-group solves, and one lane's latency-bound CMFD phase runs beside
another lane's sweeps. Latency is
measured from a request's arrival time to the moment its result is read on
the host, so queueing is included. Each latency is split into its phases: the
host loop's delay in submitting the request after it arrived, the wait in the
engine's queue for a slot (admission), the solve's outer iterations on the
GPU up to the replay that retired it, and the delay until the host read the
result.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Request:
    problem: object          # mocc_gb300.Problem whose traced geometry is used, or MOCC XML input text
                             # (the engine traces each distinct text once)
    xsl: str | None = None   # cross sections for its materials (None: its own)
    arrival: float = 0.0     # seconds after the start of the run
    lane: object = 0         # key of the engine that runs it


PHASES = ("host", "queue", "run", "collect")


@dataclass
class ServeReport:
    n: int
    wall_s: float
    latencies_s: list = field(default_factory=list)
    results: list = field(default_factory=list)
    phases_s: list = field(default_factory=list)  # per request: {phase: seconds} (PHASES)

    @property
    def solves_per_s(self) -> float:
        return self.n / self.wall_s

    def percentile_ms(self, q: float) -> float:
        return 1e3 * float(np.percentile(np.asarray(self.latencies_s), q))


def poisson_arrivals(n: int, rate: float, seed: int) -> np.ndarray:
    """Arrival times (s) of n requests of a Poisson process of `rate` per s."""
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate, size=n))


def serve(engines, requests: list[Request], max_pins: int = 1 << 12) -> ServeReport:
    """Runs the request stream to completion on `engines` (one BatchEngine, or
    a dict lane key -> BatchEngine); returns latencies and results in request
    order."""
    if not isinstance(engines, dict):
        engines = {0: engines}
        requests = [Request(r.problem, r.xsl, r.arrival, 0) for r in requests]
    order = sorted(range(len(requests)), key=lambda i: requests[i].arrival)
    t0 = time.perf_counter()
    nxt = 0
    outstanding = {k: {} for k in engines}  # lane -> {solve id: request index}
    lat = [0.0] * len(requests)
    res = [None] * len(requests)
    phases = [None] * len(requests)
    done = 0
    # engine clock -> this loop's clock
    off = {k: (time.perf_counter() - t0) - eng.stats()["now"] for k, eng in engines.items()}

    def admit_arrivals():
        nonlocal nxt
        now = time.perf_counter() - t0
        while nxt < len(order) and requests[order[nxt]].arrival <= now:
            i = order[nxt]
            r = requests[i]
            eng = engines[r.lane]
            sid = eng.submit_xml(r.problem, r.xsl) if isinstance(r.problem, str) else eng.submit(r.problem, r.xsl)
            outstanding[r.lane][sid] = i
            nxt += 1

    def harvest(k, eng):
        nonlocal done
        for sid in eng.ready():
            if sid not in outstanding[k]:
                continue
            r = eng.take(sid, max_pins)
            i = outstanding[k].pop(sid)
            now = time.perf_counter() - t0
            lat[i] = now - requests[i].arrival
            res[i] = r
            phases[i] = {"host": r["t_submit"] + off[k] - requests[i].arrival,
                         "queue": r["t_admit"] - r["t_submit"], "run": r["t_done"] - r["t_admit"],
                         "collect": now - (r["t_done"] + off[k])}
            done += 1

    while done < len(requests):
        admit_arrivals()
        busy = False
        progressed = False
        for k, eng in engines.items():
            # the oldest iteration in flight first: retire and collect
            while eng.in_flight() and (len(engines) == 1 and eng.in_flight() >= eng.depth or eng.poll()):
                progressed = True
                eng.finish()
                harvest(k, eng)
                admit_arrivals()
            # keep the lane's pipeline full while it has work
            while outstanding[k] and eng.in_flight() < eng.depth:
                if eng.launch() == 0:
                    break
                progressed = True
            if eng.in_flight():
                busy = True
            elif outstanding[k]:
                # nothing active: finished solves not yet read, or refused ones
                eng.finish()
                harvest(k, eng)
        if busy and not progressed:
            time.sleep(5e-5)  # every lane is on the GPU
        if not busy and nxt < len(order):
            wait = requests[order[nxt]].arrival - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(min(wait, 1e-3))
    wall = time.perf_counter() - t0
    return ServeReport(n=len(requests), wall_s=wall, latencies_s=lat, results=res, phases_s=phases)


def run_batch(engines, jobs, max_pins: int = 1 << 12) -> list:
    """Submits every (problem, xsl, lane) job at once and runs the lanes in a
    pipeline until all finish; returns the results in job order."""
    reqs = [Request(p, x, 0.0, lane) for p, x, lane in jobs]
    if not isinstance(engines, dict):
        engines = {0: engines}
        reqs = [Request(r.problem, r.xsl, 0.0, 0) for r in reqs]
    return serve(engines, reqs, max_pins).results
