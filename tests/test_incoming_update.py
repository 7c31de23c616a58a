"""MoCSweeper::update_incoming_flux (moc_sweeper.cpp:255-291): the incoming
boundary angular flux rescaled from the CMFD partial currents after each
CMFD solve. MOCC leaves its call commented out (eigen_solver.cpp:289), so it
is off unless <sweeper incoming_update="mocc|surface"> (or the
incoming_update option) asks for it:

* "mocc" (1) reads the partial currents the way MOCC's code does, at the
  index of the track's starting coarse cell, which is the cell's bottom
  z-face: the first CMFD solve sets every entry, vacuum faces included, to
  that face's 2 (J+ + J-) / 4pi, later solves scale it by the face's change;
* "surface" (2) reads the core-boundary surface the track enters through and
  leaves entries on vacuum faces at zero.

The library (FP64) must give the oracle's boundary flux after each CMFD
solve to the CMFD solution's agreement (1e-8 relative) and the oracle's
outer-iteration history; the update must leave the converged k where it is.
"""
import numpy as np
import pytest

import mocc_gb300 as m
import oracle
from mocc_gb300 import workloads as W


def _with(xml, mode):
    return xml.replace('<sweeper type="moc"', f'<sweeper type="moc" incoming_update="{mode}"', 1)


def test_option_is_read_from_the_sweeper_tag():
    xml, xsl = W.pin3x3()
    assert '<sweeper type="moc"' in xml
    assert m.Problem(xml, xsl).options["incoming_update"] == 0
    for mode, v in (("off", 0), ("mocc", 1), ("surface", 2)):
        assert m.Problem(_with(xml, mode), xsl).options["incoming_update"] == v
        assert oracle.Traced(_with(xml, mode), xsl).options["incoming_update"] == v
    with pytest.raises(m.MocgpuError) as e:
        m.Problem(_with(xml, "always"), xsl)
    assert e.value.code == 7


@pytest.mark.parametrize("mode", [1, 2])
def test_oracle_update_keeps_the_converged_eigenvalue(mode):
    xml, xsl = W.lattice_case(3, 8, 0.05, "double", seed=1000)
    tight = dict(k_tol=1e-9, psi_tol=1e-8)
    ra = oracle.OracleSolver.from_xml(xml, xsl, **tight).solve()
    rb = oracle.OracleSolver.from_xml(xml, xsl, incoming_update=mode, **tight).solve()
    assert ra["converged"] and rb["converged"]
    assert abs(ra["k"] - rb["k"]) < 2e-8


def _one_outer(S, G, k):
    for g in range(G):
        S.source_group(g)
        S.sweep(g)
    return S.cmfd_solve(k)


def test_oracle_modes_on_vacuum_faces():
    # after the first CMFD solve: "surface" keeps vacuum-face entries at zero,
    # MOCC's lookup fills them (from the bottom face of the starting cell)
    xml, xsl = W.minicore(n_lat=3, n_azi=4, spacing=0.1, precision="double")
    out = {}
    for mode in (0, 1, 2):
        O = oracle.OracleSolver.from_xml(xml, xsl, incoming_update=mode)
        O.initialize()
        O.set_coarse_data(True)
        O.set_fission_source(O.calc_fission_source(1.0))
        _one_outer(O, O.n_group, 1.0)
        out[mode] = np.concatenate([O.boundary_flux(g) for g in range(O.n_group)])
    vac = out[0] == 0.0
    assert vac.any() and (~vac).any()
    assert np.all(out[2][vac] == 0.0)
    assert np.all(out[1][vac] > 0.0)
    assert np.all(out[2][~vac] > 0.0) and not np.allclose(out[2][~vac], out[0][~vac])


CASES = {
    "pin3x3": lambda: W.pin3x3(),
    "core_vacuum": lambda: W.minicore(n_lat=3, n_azi=4, spacing=0.1, precision="double"),
}


@pytest.mark.gpu
@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("mode", [1, 2])
def test_boundary_flux_after_cmfd_matches_oracle(case, mode):
    xml, xsl = CASES[case]()
    xml = _with(xml, {1: "mocc", 2: "surface"}[mode])
    P = m.Problem(xml, xsl)
    S, O = m.MoCSweeper(P, 0), oracle.OracleSolver.from_xml(xml, xsl)
    assert P.options["incoming_update"] == mode == O._o.incoming_update
    G = P.sizes["ngroup"]
    for X in (S, O):
        X.initialize()
        X.set_coarse_data(True)
    fs = O.calc_fission_source(1.0)
    S.set_fission_source(fs)
    O.set_fission_source(fs)
    ka = kb = 1.0
    # the first solve sets the entries, the second rescales them
    for _ in range(2):
        ka, kb = _one_outer(S, G, ka), _one_outer(O, G, kb)
        assert abs(ka - kb) / kb < 1e-9
        for g in range(G):
            a, b = S.boundary_flux(g), O.boundary_flux(g)
            assert a.shape == b.shape
            assert np.array_equal(a == 0.0, b == 0.0)
            assert np.allclose(a, b, rtol=1e-8, atol=0.0)
        fs = O.calc_fission_source(kb)
        S.set_fission_source(fs)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [1, 2])
def test_eigen_with_update_matches_oracle(mode):
    xml, xsl = W.lattice_case(3, 8, 0.05, "double", seed=1000)
    xml = _with(xml, {1: "mocc", 2: "surface"}[mode])
    P = m.Problem(xml, xsl)
    S = m.MoCSweeper(P, 0)
    O = oracle.OracleSolver.from_xml(xml, xsl)
    ra, rb = m.EigenSolver(P, sweeper=S).solve(), O.solve()
    off = oracle.OracleSolver.from_xml(*W.lattice_case(3, 8, 0.05, "double", seed=1000)).solve()
    assert ra["converged"] and rb["converged"]
    assert ra["iterations"] == rb["iterations"] != off["iterations"]
    assert abs(ra["k"] - rb["k"]) / rb["k"] < 1e-9
    p, q = S.pin_powers(), O.pin_powers()
    assert np.max(np.abs(p - q)[q > 0] / q[q > 0]) < 1e-8


@pytest.mark.gpu
def test_mixed_precision_update_within_tolerance():
    xml, xsl = W.minicore(n_lat=3, n_azi=4, spacing=0.1, precision="double")
    xml = _with(xml, "surface")
    P = m.Problem(xml, xsl)
    S = m.MoCSweeper(P, 1)
    ra = m.EigenSolver(P, sweeper=S).solve()
    rb = oracle.OracleSolver.from_xml(xml, xsl).solve()
    assert ra["converged"]
    assert 1e5 * abs(ra["k"] - rb["k"]) / rb["k"] < 10.0


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [1, 2])
def test_batched_update_matches_single_solves(mode):
    # the batch engine runs the update after each solve's CMFD inside its
    # captured outer iteration; every solve must give its single-solve result
    # (FP64: same iterations, k to 1e-9, pins to 1e-8), vacuum faces included
    name = {1: "mocc", 2: "surface"}[mode]
    cases = [W.lattice_case(n, 8, 0.05, "double", seed=1000 + n) for n in (1, 3)]
    cases.append(CASES["core_vacuum"]())
    probs = [m.Problem(_with(x, name), s) for x, s in cases]
    E = m.BatchEngine(precision=0, capacity=4, bundles_per_unit=1)
    ids = [E.submit(P) for P in probs]
    E.run()
    for P, i in zip(probs, ids):
        r = E.take(i)
        assert r is not None and r["error"] == 0, r
        S = m.EigenSolver(P, 0)
        ref = S.solve()
        assert r["converged"] == ref["converged"]
        assert r["iterations"] == ref["iterations"]
        assert abs(r["k"] - ref["k"]) < 1e-9
        p, q = np.ravel(r["pin_powers"]), np.ravel(S.pin_powers())
        assert np.max(np.abs(p - q)[q > 0] / q[q > 0]) < 1e-8


@pytest.mark.gpu
def test_batch_engine_keeps_one_update_mode():
    # the update is part of the captured launch sequence, so every solve of
    # a batch must ask for the same mode
    xml, xsl = W.lattice_case(3, 8, 0.05, "mixed", seed=1000)
    E = m.BatchEngine(precision=1, capacity=2)
    E.submit_xml(_with(xml, "surface"), xsl)
    for other in ("off", "mocc"):
        with pytest.raises(m.MocgpuError) as e:
            E.submit_xml(_with(xml, other), xsl)
        assert e.value.code == 1


@pytest.mark.gpu
def test_mixed_precision_batched_update_within_tolerance():
    xml, xsl = W.minicore(n_lat=3, n_azi=4, spacing=0.1, precision="mixed")
    xml = _with(xml, "surface")
    E = m.BatchEngine(precision=1, capacity=2)
    i = E.submit_xml(xml, xsl)
    E.run()
    r = E.take(i)
    assert r["error"] == 0 and r["converged"]
    ref = oracle.OracleSolver.from_xml(xml, xsl).solve()
    assert 1e5 * abs(r["k"] - ref["k"]) / ref["k"] < 10.0


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [1, 2])
def test_update_from_given_partial_currents_matches_oracle(mode):
    # the entry point a MOCC build with its own CPU CMFD would call: the
    # partial-current sums come from the caller
    xml, xsl = CASES["core_vacuum"]()
    P = m.Problem(xml, xsl)
    S, O = m.MoCSweeper(P, 0), oracle.OracleSolver.from_xml(xml, xsl)
    G, ns = P.sizes["ngroup"], P.sizes["nsurf"]
    rng = np.random.default_rng(7)
    part, old = rng.uniform(0.5, 2.0, size=(G, ns)), rng.uniform(0.5, 2.0, size=(G, ns))
    old[:, ::7] = 0.0  # surfaces without a previous value keep their entries
    for X in (S, O):
        X.initialize()
        X.update_incoming_flux(part, None, mode)   # first solve: set from the sums
        X.update_incoming_flux(part, old, mode)    # later ones: rescaled by the change
    for g in range(G):
        a, b = S.boundary_flux(g), O.boundary_flux(g)
        assert np.array_equal(a == 0.0, b == 0.0)
        assert np.allclose(a, b, rtol=1e-15, atol=0.0)
