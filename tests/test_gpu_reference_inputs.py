"""GPU library against the CPU oracle on MOCC's own inputs and on the
benchmark workloads at their stated sizes (the oracle traces every input
with its own restatement of MOCC's tracer).

* examples/3x3.xml with MOCC's C5G7 library (LS quadrature, rectangular
  reflector mesh, two vacuum faces): full eigenvalue solves;
* examples/c5g7_2d.xml (the 2-D quarter core, 87 k FSRs, 9.1 M segments):
  the first outer iterations, iterate by iterate;
* the 17x17 assembly in FP64 (the plain path) and a reduced mini-core with
  the same reflector and vacuum faces (36x36 pins, cluster CMFD).

Tolerances: the FP64 path against the FP64 oracle to the rounding of sums
taken in another order (k 1e-9 relative, pin power 1e-7); the mixed path
(FP32 sweep) k within 10 pcm and every fuel pin power within 0.1 %.
"""
import numpy as np
import pytest

import mocc_gb300 as m
import oracle
from mocc_gb300 import workloads as W

pytestmark = pytest.mark.gpu

PCM_TOL = 10.0
PIN_TOL = 1e-3


def pcm(k, k_ref):
    return 1e5 * abs(k - k_ref) / k_ref


def max_pin_err(p, p_ref):
    p, p_ref = np.ravel(p), np.ravel(p_ref)
    mask = p_ref > 0
    return float(np.max(np.abs(p[mask] - p_ref[mask]) / p_ref[mask]))


def _solve_both(P, xml, xsl, precision, max_outer=-1):
    S = m.MoCSweeper(P, precision)
    ra = m.EigenSolver(P, sweeper=S).solve(max_outer)
    pa = S.pin_powers()
    S.close()
    O = oracle.OracleSolver.from_xml(xml, xsl)  # the oracle's own trace of the same input
    rb = O.solve(max_outer)
    return ra, pa, rb, O.pin_powers()


@pytest.mark.parametrize("precision", [0, 1])
def test_example_3x3_vs_oracle(ref_example, ref_xsl, precision):
    P = m.Problem(ref_example["3x3"], ref_xsl)
    assert P.sizes["nfsr"] == 1251 and P.sizes["pol_per_set"] == 1
    ra, pa, rb, pb = _solve_both(P, ref_example["3x3"], ref_xsl, precision)
    assert ra["converged"] and rb["converged"]
    if precision == 0:
        assert ra["iterations"] == rb["iterations"]
        assert abs(ra["k"] - rb["k"]) / rb["k"] < 1e-9
        assert max_pin_err(pa, pb) < 1e-7
    else:
        assert pcm(ra["k"], rb["k"]) < PCM_TOL
        assert max_pin_err(pa, pb) < PIN_TOL


@pytest.mark.parametrize("precision", [0, 1])
def test_example_c5g7_2d_iterates_vs_oracle(ref_example, ref_xsl, precision):
    P = m.Problem(ref_example["c5g7_2d"], ref_xsl)
    assert P.sizes["nfsr"] > 80000 and P.sizes["nseg"] > 9_000_000
    ra, pa, rb, pb = _solve_both(P, ref_example["c5g7_2d"], ref_xsl, precision, max_outer=3)
    assert ra["iterations"] == rb["iterations"] == 3
    if precision == 0:
        assert abs(ra["k"] - rb["k"]) / rb["k"] < 1e-9
        assert max_pin_err(pa, pb) < 1e-7
    else:
        assert pcm(ra["k"], rb["k"]) < PCM_TOL
        assert max_pin_err(pa, pb) < PIN_TOL


def test_assembly17_fp64_vs_oracle():
    # the plain FP64 path on the 17x17 assembly at its benchmark tracking
    # (16 azimuths per octant, 3 polar angles, 0.03 cm)
    xml, xsl = W.assembly17(precision="double")
    P = m.Problem(xml, xsl)
    ra, pa, rb, pb = _solve_both(P, xml, xsl, 0)
    assert ra["converged"] and rb["converged"]
    assert ra["iterations"] == rb["iterations"]
    assert abs(ra["k"] - rb["k"]) / rb["k"] < 1e-9
    assert max_pin_err(pa, pb) < 1e-7


@pytest.mark.parametrize("precision", [0, 1])
def test_reduced_minicore_vs_oracle(precision):
    # the mini-core's layout (3x3 fuel assemblies of three compositions, a
    # moderator row of assemblies on the two vacuum faces) with 9x9-pin
    # assemblies: 36x36 pins, so CMFD runs on a thread-block cluster
    xml, xsl = W.minicore(n_lat=9, n_azi=8, spacing=0.05, precision="double")
    P = m.Problem(xml, xsl)
    assert P.sizes["npin"] == 36 * 36
    ra, pa, rb, pb = _solve_both(P, xml, xsl, precision)
    assert ra["converged"] and rb["converged"]
    if precision == 0:
        # the cluster's BiCGSTAB sums in another order than the oracle's and
        # may stop one iteration apart at its 1e-8 residual reduction
        assert abs(ra["k"] - rb["k"]) / rb["k"] < 1e-8
        assert max_pin_err(pa, pb) < 1e-6
    else:
        assert pcm(ra["k"], rb["k"]) < PCM_TOL
        assert max_pin_err(pa, pb) < PIN_TOL
