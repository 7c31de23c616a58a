"""Autotuner for the batched sweep's work-unit shape.

The batched sweep runs one CTA per work unit of 1, 2 or 4 bundles of 32
tracks (two warps per bundle: forward and backward). Small units give more
CTAs and a shorter tail when few large solves dominate; larger units share
the staged cross sections and tally of a unit among more warps. The best
shape depends on the mix of lattice sizes, so it is measured: each
candidate runs the same sample batch to completion on a fresh engine and
the one with the least graph-replay device time per solve wins.
"""
from __future__ import annotations


def tune_bundles_per_unit(make_engine, sample, candidates=(1, 2, 4), repeats: int = 1) -> dict:
    """make_engine(bpu) -> BatchEngine; sample: list of (problem, xsl).

    Returns {"best": bpu, "ms_per_solve": {bpu: ms}}."""
    scores = {}
    for bpu in candidates:
        eng = make_engine(bpu)
        try:
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
            scores[bpu] = best
        finally:
            eng.close()
    return {"best": min(scores, key=scores.get), "ms_per_solve": scores}
