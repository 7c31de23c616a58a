"""MoCSweeper::apply_transverse_leakage (moc_sweeper.cpp:435-472): the hook
through which MOCC's 2-D/3-D sweeper adds the axial transverse leakage of a
group to the MoC source before sweeping it. With <sweeper tl_splitting>, an
FSR whose source plus leakage is negative gets a zero source and its Sigma_t
raised by -(source + leakage) / phi for the sweeps that follow
(XSMesh::expand(group, split_), xs_mesh.hpp:282-296); the self-scatter
source keeps the material's Sigma_tr (source_isotropic.cpp:21-57).

* CPU: the option is read as pugixml's as_bool on both sides; a zero
  leakage leaves the oracle's sweep unchanged; leakages that drive sources
  negative give a negative flux somewhere without splitting and a positive
  one with it;
* GPU (FP64): after source_group, the leakage and one group sweep, the
  scalar flux equals the oracle's to 1e-10, with and without splitting, with
  leakages that drive part of the FSRs' sources negative; a negative flux
  under splitting fails with code 15 on the GPU and in the oracle.
"""
import numpy as np
import pytest

import mocc_gb300 as m
import oracle
from mocc_gb300 import workloads as W


def _with(xml, value):
    return xml.replace('<sweeper type="moc"', f'<sweeper type="moc" tl_splitting="{value}"', 1)


def _case():
    return W.lattice_case(3, 8, 0.05, "double", seed=1000)


def test_option_is_read_as_mocc_reads_it():
    xml, xsl = _case()
    assert m.Problem(xml, xsl).options["tl_splitting"] == 0
    for v, on in (("true", 1), ("yes", 1), ("1", 1), ("false", 0), ("no", 0), ("0", 0)):
        assert m.Problem(_with(xml, v), xsl).options["tl_splitting"] == on
        assert oracle.Traced(_with(xml, v), xsl).options["tl_splitting"] == on


def _oracle_group(xml, xsl, g, tl):
    # from MoCSweeper::initialize's state, the fission source at k = 1
    O = oracle.OracleSolver.from_xml(xml, xsl)
    O.initialize()
    O.set_fission_source(O.calc_fission_source(1.0))
    O.source_group(g)
    if tl is not None:
        O.apply_transverse_leakage(g, tl)
    O.sweep(g)
    return O


def test_zero_leakage_changes_nothing_in_the_oracle():
    xml, xsl = _case()
    for split in ("false", "true"):
        x = _with(xml, split)
        a = _oracle_group(x, xsl, 2, None)
        b = _oracle_group(x, xsl, 2, np.zeros(a.n_reg))
        # the same sweep (the oracle's threads may add in another order)
        np.testing.assert_allclose(b.flux(), a.flux(), rtol=1e-13, atol=0)


def test_oracle_splitting_keeps_the_flux_positive():
    # leakages that drive sources negative: without splitting the group
    # flux goes negative somewhere, with it the negative part moves into
    # Sigma_t and the flux stays positive
    xml, xsl = _case()
    for split, positive in (("false", False), ("true", True)):
        x = _with(xml, split)
        ref = _oracle_group(x, xsl, 2, None)
        tl = _leakage(ref.n_reg, 1.5 * float(np.mean(ref.calc_fission_source(1.0))))
        f = _oracle_group(x, xsl, 2, tl).flux()[:, 2]
        assert np.all(np.isfinite(f))
        assert bool(np.all(f > 0.0)) == positive


def _leakage(n, scale, seed=3):
    # leakages of either sign, large enough to drive the weaker sources negative
    rng = np.random.default_rng(seed)
    return scale * rng.uniform(-1.5, 1.0, size=n)


@pytest.mark.gpu
@pytest.mark.parametrize("split", ["false", "true"])
def test_group_sweep_with_leakage_matches_oracle(split):
    xml, xsl = _case()
    x = _with(xml, split)
    P = m.Problem(x, xsl)
    S = m.MoCSweeper(P, 0)
    n, g = P.sizes["nfsr"], 2
    S.initialize()
    fs = S.calc_fission_source(1.0)
    S.set_fission_source(fs)
    tl = _leakage(n, float(np.mean(fs)))
    O = _oracle_group(x, xsl, g, tl)
    S.source_group(g)
    S.apply_transverse_leakage(g, tl)
    S.sweep(g)
    a, b = S.flux()[:, g], O.flux()[:, g]
    np.testing.assert_allclose(a, b, rtol=1e-10, atol=0)
    # the leakage mattered, and with splitting some FSRs were split
    ref = _oracle_group(x, xsl, g, None).flux()[:, g]
    assert np.max(np.abs(ref - b) / np.abs(b)) > 1e-3


@pytest.mark.gpu
def test_negative_flux_under_splitting_fails_on_both_sides():
    xml, xsl = _case()
    x = _with(xml, "true")
    P = m.Problem(x, xsl)
    S = m.MoCSweeper(P, 0)
    n, G, g = P.sizes["nfsr"], P.sizes["ngroup"], 1
    S.initialize()
    f = np.ones((n, G))
    f[:, g] = -1.0
    S.set_flux(f)
    S.set_fission_source(np.zeros(n))
    S.source_group(g)
    tl = np.full(n, -1.0e3)
    with pytest.raises(m.MocgpuError) as e:
        S.apply_transverse_leakage(g, tl)
    assert e.value.code == 15
    O = oracle.OracleSolver.from_xml(x, xsl)
    O.initialize()
    O.set_flux(f)
    O.set_fission_source(np.zeros(n))
    O.source_group(g)
    with pytest.raises(RuntimeError, match="Negative flux when splitting"):
        O.apply_transverse_leakage(g, tl)
