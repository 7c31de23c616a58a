"""Request loop over the batch engine: continuous batching of arriving solves.

Requests arrive on a schedule (a seeded Poisson process for the benchmark);
each is submitted to the :class:`~mocc_gb300.BatchEngine` as soon as its
arrival time has passed, the engine admits it into a free slot once its
geometry and state fit the device-memory budget, every active solve advances
one power iteration per graph replay, and results are collected as solves
retire. Latency is measured from a request's arrival time to the moment its
result is read on the host, so queueing is included.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Request:
    problem: object          # mocc_gb300.Problem whose traced geometry is used
    xsl: str | None = None   # cross sections for its materials (None: its own)
    arrival: float = 0.0     # seconds after the start of the run


@dataclass
class ServeReport:
    n: int
    wall_s: float
    latencies_s: list = field(default_factory=list)
    results: list = field(default_factory=list)

    @property
    def solves_per_s(self) -> float:
        return self.n / self.wall_s

    def percentile_ms(self, q: float) -> float:
        return 1e3 * float(np.percentile(np.asarray(self.latencies_s), q))


def poisson_arrivals(n: int, rate: float, seed: int) -> np.ndarray:
    """Arrival times (s) of n requests of a Poisson process of `rate` per s."""
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate, size=n))


def serve(engine, requests: list[Request], max_pins: int = 1 << 12) -> ServeReport:
    """Runs the request stream to completion; returns latencies and results
    in request order."""
    order = sorted(range(len(requests)), key=lambda i: requests[i].arrival)
    t0 = time.perf_counter()
    nxt = 0
    outstanding: dict[int, int] = {}  # solve id -> request index
    lat = [0.0] * len(requests)
    res = [None] * len(requests)
    done = 0
    while done < len(requests):
        now = time.perf_counter() - t0
        while nxt < len(order) and requests[order[nxt]].arrival <= now:
            i = order[nxt]
            outstanding[engine.submit(requests[i].problem, requests[i].xsl)] = i
            nxt += 1
        if outstanding:
            engine.step()
            for sid in list(outstanding):
                r = engine.take(sid, max_pins)
                if r is None:
                    continue
                i = outstanding.pop(sid)
                lat[i] = time.perf_counter() - t0 - requests[i].arrival
                res[i] = r
                done += 1
        elif nxt < len(order):
            wait = requests[order[nxt]].arrival - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(min(wait, 1e-3))
    wall = time.perf_counter() - t0
    return ServeReport(n=len(requests), wall_s=wall, latencies_s=lat, results=res)
