"""Batched solves: each solve in a batch gives the result it gives alone.

The batch engine advances many independent eigenvalue solves together; the
arithmetic of every solve is the single-solve arithmetic, only the launches
are shared, so:

* FP64 batched solves match the FP64 single-solve path (k to 1e-9 absolute,
  pin powers to 1e-8 relative; the sums run in another order);
* mixed-precision batched solves match the FP64 oracle within 10 pcm and
  0.1 % pin power;
* a solve's result does not depend on what else is in the batch (the FP32
  tally's atomic order is the only difference: k within 0.05 pcm, pins 1e-5).
"""
import numpy as np
import pytest

import mocc_gb300 as m
import oracle
from mocc_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def pcm(k, k_ref):
    return 1e5 * abs(k - k_ref) / k_ref


def max_pin_err(p, p_ref):
    p, p_ref = np.ravel(p), np.ravel(p_ref)
    mask = p_ref > 0
    return float(np.max(np.abs(p[mask] - p_ref[mask]) / p_ref[mask]))


def _cases(n, seed=5, sizes=(1, 3, 7), precision="double"):
    """Seeded lattice cases of mixed sizes and cross-section perturbations."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        size = int(sizes[i % len(sizes)])
        out.append(W.lattice_case(size, 8, 0.05, precision, seed=1000 + i,
                                  mod_factor=float(rng.uniform(0.9, 1.1)),
                                  fuel_nf_factor=float(rng.uniform(0.95, 1.05))))
    return out


def _run(engine, problems, xsls=None):
    ids = [engine.submit(P, x) for P, x in zip(problems, xsls or [None] * len(problems))]
    engine.run()
    res = [engine.take(i) for i in ids]
    assert all(r is not None for r in res)
    return res


def test_fp64_batch_matches_single_solves():
    cases = _cases(6)
    probs = [m.Problem(x, s) for x, s in cases]
    E = m.BatchEngine(precision=0, capacity=8, bundles_per_unit=1)
    res = _run(E, probs)
    for P, r in zip(probs, res):
        assert r["error"] == 0, r["message"]
        S = m.EigenSolver(P, 0)
        ref = S.solve()
        assert r["iterations"] == ref["iterations"]
        assert r["converged"] == ref["converged"] == 1
        assert abs(r["k"] - ref["k"]) < 1e-9
        assert max_pin_err(r["pin_powers"], S.pin_powers()) < 1e-8


def test_mixed_batch_matches_oracle():
    cases = _cases(5, seed=9, precision="mixed")
    probs = [m.Problem(x, s) for x, s in cases]
    E = m.BatchEngine(precision=1, capacity=8, bundles_per_unit=2)
    res = _run(E, probs)
    for (x, xs), r in zip(cases, res):
        assert r["error"] == 0, r["message"]
        O = oracle.OracleSolver.from_xml(x, xs)  # the oracle's own trace of the same input
        ref = O.solve()
        assert r["converged"] == 1
        assert pcm(r["k"], ref["k"]) < 10.0
        assert max_pin_err(r["pin_powers"], O.pin_powers()) < 1e-3


@pytest.mark.parametrize("precision,k_tol,pin_tol", [(0, 1e-11, 1e-10), (1, 5e-7, 1e-5)])
def test_result_same_alone_and_in_the_mix(precision, k_tol, pin_tol):
    pstr = "double" if precision == 0 else "mixed"
    target = W.lattice_case(7, 8, 0.05, pstr, seed=77, mod_factor=1.03)
    mix = _cases(11, seed=3, sizes=(1, 3, 7, 5), precision=pstr)
    P = m.Problem(*target)
    alone = _run(m.BatchEngine(precision=precision, capacity=4), [P])[0]
    probs = [m.Problem(x, s) for x, s in mix[:5]] + [P] + [m.Problem(x, s) for x, s in mix[5:]]
    E = m.BatchEngine(precision=precision, capacity=6)  # fewer slots than solves: continuous batching
    res = _run(E, probs)
    inmix = res[5]
    assert alone["error"] == inmix["error"] == 0
    if precision == 0:
        assert alone["iterations"] == inmix["iterations"]
    assert abs(alone["k"] - inmix["k"]) < k_tol
    assert max_pin_err(inmix["pin_powers"], alone["pin_powers"]) < pin_tol
    st = E.stats()
    assert st["completed"] == len(probs) and st["active"] == 0 and st["queued"] == 0


def test_shared_geometry_with_other_cross_sections():
    xml, xsl = W.lattice_case(3, 8, 0.05, "double", seed=1)
    base = m.Problem(xml, xsl)
    xsl2 = W.lattice_case(3, 8, 0.05, "double", seed=1, mod_factor=1.07, fuel_nf_factor=0.97)[1]
    E = m.BatchEngine(precision=0, capacity=4)
    r = _run(E, [base, base], [None, xsl2])
    assert E.stats()["geometries"] == 1
    ref1 = m.EigenSolver(base, 0).solve()
    ref2 = m.EigenSolver(m.Problem(xml, xsl2), 0).solve()
    assert abs(r[0]["k"] - ref1["k"]) < 1e-9
    assert abs(r[1]["k"] - ref2["k"]) < 1e-9
    assert abs(ref1["k"] - ref2["k"]) > 1e-4  # the cross sections did change


def test_memory_budget_gates_admission():
    cases = _cases(4, sizes=(3,))
    probs = [m.Problem(x, s) for x, s in cases]
    E = m.BatchEngine(precision=0, capacity=8)
    E.submit(probs[0])
    E.step()
    st = E.stats()
    geom = st["geometry_bytes"]
    state = st["bytes_in_use"] - geom
    E.run()
    assert geom > 0 and state > 0
    # room for the geometry and about one and a half solves
    E2 = m.BatchEngine(precision=0, capacity=8, mem_budget=2 * geom + 1.5 * state)
    ids = [E2.submit(P) for P in probs]
    peak = 0
    while True:
        n = E2.step()
        peak = max(peak, n)
        s2 = E2.stats()
        assert s2["bytes_in_use"] <= s2["bytes_budget"]
        if n == 0 and s2["queued"] == 0:
            break
    res = [E2.take(i) for i in ids]
    assert all(r["error"] == 0 and r["converged"] == 1 for r in res)
    assert 1 <= peak < len(probs)


def test_solve_larger_than_budget_is_refused():
    P = m.Problem(*W.lattice_case(7, 8, 0.05, "double", seed=2))
    E = m.BatchEngine(precision=0, capacity=2, mem_budget=64 * 1024)
    r = _run(E, [P])[0]
    assert r["error"] == 21 and "budget" in r["message"]


def test_batch_rejects_mismatched_configuration():
    a = m.Problem(*W.pin3x3())
    b = m.Problem(*W.pin3x3())
    b.set_options(n_inner=2)
    E = m.BatchEngine(precision=0, capacity=2)
    E.submit(a)
    with pytest.raises(m.MocgpuError) as e:
        E.submit(b)
    assert e.value.code == 1


def test_pipelined_lanes_give_the_same_results():
    from mocc_gb300.serve import run_batch
    cases = _cases(8, seed=21, sizes=(1, 3, 7))
    probs = [m.Problem(x, s) for x, s in cases]
    one = _run(m.BatchEngine(precision=0, capacity=8), probs)
    lanes = {0: m.BatchEngine(precision=0, capacity=3), 1: m.BatchEngine(precision=0, capacity=3)}
    two = run_batch(lanes, [(P, None, i % 2) for i, P in enumerate(probs)])
    for a, b in zip(one, two):
        assert a["error"] == b["error"] == 0
        assert a["iterations"] == b["iterations"]
        assert abs(a["k"] - b["k"]) < 1e-11
        assert max_pin_err(b["pin_powers"], a["pin_powers"]) < 1e-10


def test_retired_handles_are_reused_without_allocation():
    P = m.Problem(*W.lattice_case(3, 8, 0.05, "double", seed=8))
    E = m.BatchEngine(precision=0, capacity=2)
    first = _run(E, [P, P])
    used = E.stats()["bytes_in_use"]
    again = _run(E, [P, P, P, P])
    assert E.stats()["bytes_in_use"] == used  # the two pooled handles served all four solves
    assert all(abs(r["k"] - first[0]["k"]) < 1e-11 for r in again)


def test_mixed_group_counts_in_one_batch_match_oracle():
    # 7- and 23-group solves in one engine: a solve with G groups takes part
    # only in the first G group launches of a replay
    cases = [W.lattice_case(size, 8, 0.05, "mixed", seed=1007 if ng == 23 else 1000, n_group=ng,
                            mod_factor=mf, fuel_nf_factor=1.0)
             for size, ng, mf in ((3, 23, 0.95), (1, 7, 1.05), (3, 7, 1.0), (1, 23, 1.08))]
    probs = [m.Problem(x, s) for x, s in cases]
    assert sorted(P.sizes["ngroup"] for P in probs) == [7, 7, 23, 23]
    E = m.BatchEngine(precision=1, capacity=4)
    res = _run(E, probs)
    for (x, xs), r in zip(cases, res):
        assert r["error"] == 0, r["message"]
        O = oracle.OracleSolver.from_xml(x, xs)  # the oracle's own trace of the same input
        ref = O.solve()
        assert r["converged"] == 1
        assert pcm(r["k"], ref["k"]) < 10.0
        assert max_pin_err(r["pin_powers"], O.pin_powers()) < 1e-3


def test_23_group_assembly_in_a_batch_matches_oracle():
    # a 17x17 lattice with 23 groups: the CMFD operator of every group does
    # not fit in shared memory, so each group's is copied in per group solve
    xml, xsl = W.lattice_case(17, 8, 0.05, "mixed", seed=1007, n_group=23, mod_factor=1.02, fuel_nf_factor=0.98)
    P = m.Problem(xml, xsl)
    assert P.sizes["ngroup"] == 23 and P.sizes["npin"] == 289
    r = _run(m.BatchEngine(precision=1, capacity=2), [P])[0]
    assert r["error"] == 0, r["message"]
    O = oracle.OracleSolver.from_xml(xml, xsl)
    ref = O.solve()
    assert r["converged"] == 1
    assert pcm(r["k"], ref["k"]) < 10.0
    assert max_pin_err(r["pin_powers"], O.pin_powers()) < 1e-3


def test_requests_given_as_input_text_share_one_trace():
    # two independently written copies of one lattice input with different
    # cross sections: the engine traces the lattice once and both solves
    # run on one device geometry, with the results of separately traced
    # problems
    xml, xsl1 = W.lattice_case(3, 8, 0.05, "mixed", seed=1000, mod_factor=0.97)
    xml2, xsl2 = W.lattice_case(3, 8, 0.05, "mixed", seed=1000, mod_factor=1.04)
    assert xml2 == xml and xsl1 != xsl2
    E = m.BatchEngine(precision=1, capacity=4)
    ids = [E.submit_xml(xml, xsl1), E.submit_xml(xml2, xsl2)]
    E.run()
    res = [E.take(i) for i in ids]
    st = E.stats()
    assert st["trace_misses"] == 1 and st["trace_hits"] == 1 and st["geometries"] == 1
    ref = _run(m.BatchEngine(precision=1, capacity=4), [m.Problem(xml, xsl1), m.Problem(xml2, xsl2)])
    for r, q in zip(res, ref):
        # float reductions (FP32 side path of the tally, crossing currents)
        # add in any order: the same tolerance as a solve alone and in a mix
        assert r["error"] == 0
        assert abs(r["k"] - q["k"]) < 5e-7 * q["k"]
        assert np.allclose(r["pin_powers"], q["pin_powers"], rtol=1e-5)


def test_every_sweep_ring_shape_gives_the_same_results():
    # the streaming shape only changes how segment rows reach shared memory,
    # and with it the order of the FP32 tally's float reductions: the solves
    # may stop one outer iteration apart, so k agrees to a few k_tol (1e-6)
    # and pin powers to the fission-source tolerance
    cases = _cases(6, seed=21, sizes=(1, 3, 7), precision="mixed")
    probs = [m.Problem(x, s) for x, s in cases]
    ref = _run(m.BatchEngine(precision=1, capacity=8), probs)
    for sh in range(1, len(m.sweep_shapes())):
        E = m.BatchEngine(precision=1, capacity=8)
        E.set_sweep_shape(sh)
        for a, b in zip(_run(E, probs), ref):
            assert a["error"] == 0 and a["converged"] == 1
            assert abs(a["k"] - b["k"]) < 3e-6, sh
            assert max_pin_err(a["pin_powers"], b["pin_powers"]) < 1e-4, sh
    with pytest.raises(m.MocgpuError) as e:
        m.BatchEngine(precision=0, capacity=2).set_sweep_shape(1)
    assert e.value.code == 1
