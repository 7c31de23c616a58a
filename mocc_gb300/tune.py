"""Autotuner for the batched sweep: work-unit shape x streaming shape.

The batched sweep runs one CTA per work unit of 1, 2 or 4 bundles of 32
tracks (two warps per bundle: forward and backward). Small units give more
CTAs and a shorter tail when few large solves dominate; larger units share
the staged cross sections and tally of a unit among more warps. Each warp
streams its bundle's segment rows through a shared-memory ring whose shape
(rows per chunk, chunks in flight; ``mocc_gb300.sweep_shapes()``) trades
prefetch depth against shared memory, and so against resident CTAs. The
best point depends on the mix of lattice sizes, so it is measured: every
(bundles per unit, ring shape) pair runs the same sample batch to
completion on a fresh engine, and the one with the least graph-replay
device time per solve wins.
"""
from __future__ import annotations


def _score(eng, sample, repeats):
    best = None
    for _ in range(repeats + 1):  # the first run captures the graph
        before = eng.stats()["replay_ms"]
        ids = [eng.submit(p, x) for p, x in sample]
        eng.run()
        for i in ids:
            r = eng.take(i)
            if r is None or r["error"]:
                raise RuntimeError(f"tuning solve failed: {r}")
        ms = (eng.stats()["replay_ms"] - before) / len(sample)
        best = ms if best is None else min(best, ms)
    return best


def tune_sweep(make_engine, sample, bundles=(1, 2, 4), shapes=None, repeats: int = 1) -> dict:
    """Grid search. make_engine(bpu) -> BatchEngine (FP32); sample: list of
    (problem, xsl); shapes: indices into sweep_shapes() (default: all).

    Returns {"best": {"bundles_per_unit", "shape", "rows", "stages"},
    "ms_per_solve": {"bpu=B rows=R stages=S": ms}, "points": n}."""
    from . import sweep_shapes
    table = sweep_shapes()
    shapes = range(len(table)) if shapes is None else shapes
    scores = {}
    for bpu in bundles:
        for sh in shapes:
            eng = make_engine(bpu)
            try:
                eng.set_sweep_shape(sh)
                scores[(bpu, sh)] = _score(eng, sample, repeats)
            finally:
                eng.close()
    bpu, sh = min(scores, key=scores.get)
    rows, stages = table[sh]

    def key(b, s):
        return f"bpu={b} rows={table[s][0]} stages={table[s][1]}"

    return {"best": {"bundles_per_unit": bpu, "shape": sh, "rows": rows, "stages": stages},
            "ms_per_solve": {key(b, s): v for (b, s), v in scores.items()}, "points": len(scores)}


def tune_bundles_per_unit(make_engine, sample, candidates=(1, 2, 4), repeats: int = 1) -> dict:
    """Work-unit shape alone, in the default ring shape.

    Returns {"best": bpu, "ms_per_solve": {bpu: ms}}."""
    scores = {}
    for bpu in candidates:
        eng = make_engine(bpu)
        try:
            scores[bpu] = _score(eng, sample, repeats)
        finally:
            eng.close()
    return {"best": min(scores, key=scores.get), "ms_per_solve": scores}
