"""Host logic of the request loop and the autotuner, on CPU with a stand-in
engine: requests are submitted only once their arrival time has passed,
every result comes back to the request that asked for it, lanes that are
still busy do not block the others, each lane keeps its pipeline of
outer iterations full, and the autotuner keeps the work-unit shape with
the least device time per solve."""
import time

from mocc_gb300.serve import Request, poisson_arrivals, run_batch, serve
from mocc_gb300.tune import tune_bundles_per_unit, tune_sweep


class FakeEngine:
    """The BatchEngine calls serve() makes: each solve needs `outers` outer
    iterations; up to `depth` iterations may be launched before the oldest
    is finished, and each completes after `poll_delay` polls (a blocking
    finish() waits for it). As on the device, a solve that ended in one
    iteration is skipped by the ones launched after it. Its clock starts at
    t0; results carry their submit, admission and retirement times on it."""

    def __init__(self, outers=3, poll_delay=2, t0=None, replay_ms=1.0, depth=2):
        self.outers, self.poll_delay, self.replay_ms, self.depth = outers, poll_delay, replay_ms, depth
        self.t0 = t0 if t0 is not None else time.perf_counter()
        self.next_id, self.active, self.done, self.taken = 0, {}, {}, set()
        self.submits, self.flights, self.replays, self.closed = [], [], 0, False
        self.max_in_flight = 0
        self.times = {}

    def submit(self, problem, xsl=None):
        i = self.next_id
        self.next_id += 1
        self.active[i] = [problem, xsl, 0]
        self.submits.append((problem, time.perf_counter() - self.t0))
        self.times[i] = [self.now(), None, None]
        return i

    def now(self):
        return time.perf_counter() - self.t0

    def in_flight(self):
        return len(self.flights)

    def launch(self):
        assert len(self.flights) < self.depth
        if not self.active:
            return 0
        self.flights.append({"solves": list(self.active), "polls": 0})
        for i in self.active:
            if self.times[i][1] is None:
                self.times[i][1] = self.now()
        self.max_in_flight = max(self.max_in_flight, len(self.flights))
        return len(self.active)

    def poll(self):
        if not self.flights:
            return True
        self.flights[0]["polls"] += 1
        return self.flights[0]["polls"] >= self.poll_delay

    def finish(self):
        if not self.flights:
            return len(self.active)
        f = self.flights.pop(0)
        self.replays += 1
        for i in f["solves"]:
            if i not in self.active:
                continue  # ended in an earlier iteration: skipped
            self.active[i][2] += 1
            if self.active[i][2] >= self.outers:
                p, x, _ = self.active.pop(i)
                self.done[i] = (p, x)
                self.times[i][2] = self.now()
        return len(self.active)

    def step(self):
        self.launch()
        return self.finish()

    def run(self):
        while self.active:
            self.step()

    def ready(self):
        return [i for i in self.done if i not in self.taken]

    def take(self, i, n_pin_max=0):
        if i not in self.done or i in self.taken:
            return None
        self.taken.add(i)
        p, x = self.done[i]
        ts, ta, td = self.times[i]
        return {"id": i, "error": 0, "problem": p, "xsl": x, "converged": 1, "t_submit": ts, "t_admit": ta,
                "t_done": td}

    def stats(self):
        return {"replay_ms": self.replays * self.replay_ms, "now": self.now()}

    def close(self):
        self.closed = True


def test_requests_wait_for_arrival_and_results_match_requests():
    t0 = time.perf_counter()
    lanes = {"a": FakeEngine(outers=3, t0=t0), "b": FakeEngine(outers=5, poll_delay=4, t0=t0)}
    arr = poisson_arrivals(40, rate=2000.0, seed=3)
    reqs = [Request(problem=("p", i), xsl=f"x{i}", arrival=float(a), lane="a" if i % 3 else "b")
            for i, a in enumerate(arr)]
    rep = serve(lanes, reqs)
    assert rep.n == 40 and len(rep.results) == 40
    for i, r in enumerate(rep.results):
        assert r["problem"] == ("p", i) and r["xsl"] == f"x{i}"
    assert all(lat >= 0.0 for lat in rep.latencies_s)
    # no request reached an engine before it arrived
    arrival = {("p", i): a for i, a in enumerate(arr)}
    for eng in lanes.values():
        for prob, t in eng.submits:
            assert t >= arrival[prob] - 1e-6
    assert sorted(len(e.submits) for e in lanes.values()) == [14, 26]
    # each latency splits into host delay, queue, run and collection
    for lat, ph in zip(rep.latencies_s, rep.phases_s):
        assert all(v >= -1e-4 for v in ph.values()), ph  # the two clocks are matched to a few us
        assert abs(sum(ph.values()) - lat) < 1e-6


def test_busy_lane_does_not_block_the_other():
    # lane "slow" needs many polls per iteration; lane "fast" finishes its
    # solves while "slow" is still on its first iterations
    slow, fast = FakeEngine(outers=4, poll_delay=50), FakeEngine(outers=2, poll_delay=1)
    reqs = [Request(("s", 0), None, 0.0, "slow")] + [Request(("f", i), None, 0.0, "fast") for i in range(5)]
    rep = serve({"slow": slow, "fast": fast}, reqs)
    assert all(r is not None for r in rep.results)
    assert max(rep.latencies_s[1:]) <= rep.latencies_s[0]
    assert fast.replays >= 2
    # the slow lane's pipeline ran two iterations ahead: one more replay
    # than its solve needed, launched before the host saw it end
    assert slow.replays in (4, 5) and slow.max_in_flight == 2


def test_run_batch_single_engine_returns_job_order():
    eng = FakeEngine(outers=2)
    res = run_batch(eng, [(("j", i), None, 0) for i in range(7)])
    assert [r["problem"] for r in res] == [("j", i) for i in range(7)]


def test_autotuner_keeps_the_fastest_shape():
    made = {}

    def make(bpu):
        made[bpu] = FakeEngine(outers=2, replay_ms={1: 3.0, 2: 1.0, 4: 2.0}[bpu])
        return made[bpu]

    out = tune_bundles_per_unit(make, [(("s", i), None) for i in range(4)])
    assert out["best"] == 2
    assert set(out["ms_per_solve"]) == {1, 2, 4}
    assert all(e.closed for e in made.values())


def test_grid_autotuner_searches_both_dimensions():
    # replay time per iteration as a function of (bundles per unit, ring shape)
    cost = {(b, s): 2.0 + abs(b - 2) + 0.5 * abs(s - 3) for b in (1, 2, 4) for s in range(5)}
    made = []

    class Shaped(FakeEngine):
        def __init__(self, bpu):
            super().__init__(outers=2)
            self.bpu = bpu

        def set_sweep_shape(self, s):
            self.replay_ms = cost[(self.bpu, s)]

    def make(bpu):
        made.append(Shaped(bpu))
        return made[-1]

    out = tune_sweep(make, [(("s", i), None) for i in range(3)])
    assert out["points"] == 15 and len(made) == 15 and all(e.closed for e in made)
    assert out["best"]["bundles_per_unit"] == 2 and out["best"]["shape"] == 3
    import mocc_gb300 as m
    assert (out["best"]["rows"], out["best"]["stages"]) == m.sweep_shapes()[3]
