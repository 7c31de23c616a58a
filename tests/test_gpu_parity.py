"""GPU library against the CPU oracle on the same input text (the oracle
traces it with its own restatement of MOCC's tracer; the two traces agree to
rounding, tests/test_oracle_tracer.py).

Tolerances: the FP64 path must agree with the FP64 oracle to 1e-10 relative
per sweep (only the order of floating-point sums differs); the mixed path
(FP32 sweep, FP64 reductions and CMFD) must give k within 10 pcm and every
fuel pin power within 0.1 %.
"""
import numpy as np
import pytest

import mocc_gb300 as m
import oracle
from mocc_gb300 import workloads as W

pytestmark = pytest.mark.gpu

PCM_TOL = 10.0       # k error, pcm
PIN_TOL = 1e-3       # max relative pin-power error
FP64_TOL = 1e-10


def pcm(k, k_ref):
    return 1e5 * abs(k - k_ref) / k_ref


def max_pin_err(p, p_ref):
    mask = p_ref > 0
    return float(np.max(np.abs(p[mask] - p_ref[mask]) / p_ref[mask]))


ORACLE_OPTIONS = {k for k, _ in oracle._O._fields_}


def _pair(xml, xsl, precision, **opt):
    """The library's solve and the oracle on its own trace of the same input."""
    P = m.Problem(xml, xsl)
    if opt:
        P.set_options(**opt)
    O = oracle.OracleSolver.from_xml(xml, xsl, **{k: v for k, v in opt.items() if k in ORACLE_OPTIONS})
    return P, m.MoCSweeper(P, precision), O


@pytest.mark.parametrize("kernel", [0, 1])
@pytest.mark.parametrize("gs", [1, 0])
@pytest.mark.parametrize("currents", [False, True])
def test_group_sweeps_fp64(kernel, gs, currents):
    P, S, O = _pair(*W.pin3x3(), 0, gs_boundary=gs, n_inner=2, sweep_kernel=kernel)
    S.initialize()
    O.initialize()
    S.set_coarse_data(currents)
    O.set_coarse_data(currents)
    rng = np.random.default_rng(11)
    f0 = rng.uniform(0.5, 2.0, size=(P.sizes["nfsr"], P.sizes["ngroup"]))
    S.set_flux(f0)
    O.set_flux(f0)
    fs = O.calc_fission_source(0.9)
    S.set_fission_source(fs)
    for sweep_round in range(2):
        for g in range(P.sizes["ngroup"]):
            S.source_group(g)
            O.source_group(g)
            S.sweep(g)
            O.sweep(g)
    a, b = S.flux(), O.flux()
    assert np.max(np.abs(a - b) / np.abs(b)) < FP64_TOL
    if currents:
        ca, sa = S.coarse_currents()
        cb, sb = O.coarse_currents()
        scale = np.max(np.abs(cb))
        assert np.max(np.abs(ca - cb)) < 1e-10 * scale
        assert np.max(np.abs(sa - sb)) < 1e-10 * np.max(np.abs(sb))


@pytest.mark.parametrize("kernel", [0, 1])
def test_group_sweeps_fp32_close(kernel):
    P, S, O = _pair(*W.pin3x3(), 1, n_inner=2, sweep_kernel=kernel)
    S.initialize()
    O.initialize()
    fs = O.calc_fission_source(1.0)
    S.set_fission_source(fs)
    for g in range(P.sizes["ngroup"]):
        S.source_group(g)
        O.source_group(g)
        S.sweep(g)
        O.sweep(g)
    a, b = S.flux(), O.flux()
    assert np.max(np.abs(a - b) / np.abs(b)) < 2e-5


def test_reductions_and_pin_flux_fp64():
    P, S, O = _pair(*W.pin3x3(), 0)
    S.initialize()
    O.initialize()
    rng = np.random.default_rng(5)
    f0 = rng.uniform(0.5, 2.0, size=(P.sizes["nfsr"], P.sizes["ngroup"]))
    S.set_flux(f0)
    O.set_flux(f0)
    assert abs(S.total_fission() - O.total_fission()) < 1e-12 * O.total_fission()
    assert np.allclose(S.calc_fission_source(1.1), O.calc_fission_source(1.1), rtol=1e-13, atol=0)
    for g in range(P.sizes["ngroup"]):
        a = S.get_pin_flux_1g(g)
        assert np.allclose(a, O.get_pin_flux_1g(g), rtol=1e-13, atol=0)
        tgt = a * rng.uniform(0.8, 1.2, size=a.size)
        ra = S.set_pin_flux_1g(g, tgt)
        rb = O.set_pin_flux_1g(g, tgt)
        assert abs(ra - rb) <= 1e-12 * max(rb, 1e-300)
        assert np.allclose(S.get_pin_flux_1g(g), tgt, rtol=1e-12)
    assert np.allclose(S.flux(), O.flux(), rtol=1e-12)
    assert np.allclose(S.pin_powers(), O.pin_powers(), rtol=1e-12)
    with pytest.raises(m.MocgpuError) as e:
        S.set_pin_flux_1g(0, np.zeros(P.sizes["npin"]))
    assert e.value.code == 11


def test_cmfd_solve_fp64():
    P, S, O = _pair(*W.pin3x3(), 0)
    S.initialize()
    O.initialize()
    S.set_coarse_data(True)
    O.set_coarse_data(True)
    fs = O.calc_fission_source(1.0)
    S.set_fission_source(fs)
    for g in range(P.sizes["ngroup"]):
        S.source_group(g)
        O.source_group(g)
        S.sweep(g)
        O.sweep(g)
    ka = S.cmfd_solve(1.0)
    kb = O.cmfd_solve(1.0)
    assert abs(ka - kb) / kb < 1e-9
    assert np.allclose(S.flux(), O.flux(), rtol=1e-8)


def test_homogenized_xs_matches_oracle():
    # get_homogenized_xsmesh: the device homogenisation of a non-flat flux
    P, S, O = _pair(*W.pin3x3(), 0)
    S.initialize()
    O.initialize()
    fs = O.calc_fission_source(1.0)
    S.set_fission_source(fs)
    for g in range(P.sizes["ngroup"]):
        S.source_group(g)
        O.source_group(g)
        S.sweep(g)
        O.sweep(g)
    h = S.homogenized_xs()
    ref = O.homogenized_nu_fission()  # pins in FSR order
    cell = P.export("pin_cell")
    assert np.allclose(h["xsnf"][cell], ref, rtol=1e-12, atol=0)
    assert np.all(h["xstr"] > 0) and np.all(h["xsrm"] <= h["xstr"])
    assert np.allclose(h["xsrm"], h["xstr"] - np.einsum("pgg->pg", h["scat"]), rtol=1e-12)


def test_cmfd_solve_cluster_fp64():
    # 36x36 pin mesh (1296 cells): the single-solve CMFD runs on a cluster of
    # CTAs, each with a slice of the cells
    xml, xsl = W.minicore(n_lat=9, n_azi=2, spacing=0.1, precision="double")
    P, S, O = _pair(xml, xsl, 0)
    assert P.sizes["npin"] > 1024
    S.initialize()
    O.initialize()
    S.set_coarse_data(True)
    O.set_coarse_data(True)
    fs = O.calc_fission_source(1.0)
    S.set_fission_source(fs)
    for g in range(P.sizes["ngroup"]):
        S.source_group(g)
        O.source_group(g)
        S.sweep(g)
        O.sweep(g)
    ka = S.cmfd_solve(1.0)
    kb = O.cmfd_solve(1.0)
    assert abs(ka - kb) / kb < 1e-9
    assert np.allclose(S.flux(), O.flux(), rtol=1e-8)


@pytest.mark.parametrize("kernel", [0, 1])
@pytest.mark.parametrize("gs", [1, 0])
def test_eigen_fp64_matches_oracle(kernel, gs):
    P, S, O = _pair(*W.pin3x3(), 0, gs_boundary=gs, sweep_kernel=kernel)
    ra = m.EigenSolver(P, sweeper=S).solve()
    rb = O.solve()
    assert ra["converged"] and rb["converged"]
    assert ra["iterations"] == rb["iterations"]
    assert abs(ra["k"] - rb["k"]) / rb["k"] < 1e-9
    assert max_pin_err(S.pin_powers(), O.pin_powers()) < 1e-8


def test_eigen_mixed_within_tolerance():
    P, S, O = _pair(*W.pin3x3(), 1)
    ra = m.EigenSolver(P, sweeper=S).solve()
    rb = O.solve()
    assert ra["converged"]
    assert pcm(ra["k"], rb["k"]) < PCM_TOL
    assert max_pin_err(S.pin_powers(), O.pin_powers()) < PIN_TOL


@pytest.mark.parametrize("precision", [0, 1])
def test_vacuum_boundaries_small_core(precision):
    xml, xsl = W.minicore(n_lat=3, n_azi=4, spacing=0.05, precision="double")
    P, S, O = _pair(xml, xsl, precision)
    ra = m.EigenSolver(P, sweeper=S).solve()
    rb = O.solve()
    assert ra["converged"] and rb["converged"]
    assert pcm(ra["k"], rb["k"]) < (1e-4 if precision == 0 else PCM_TOL)
    assert max_pin_err(S.pin_powers(), O.pin_powers()) < (1e-8 if precision == 0 else PIN_TOL)


@pytest.mark.parametrize("precision", [0, 1])
def test_corner_exits_small_core(precision):
    # 8 azimuths per octant on a core with vacuum faces: many tracks pass
    # through, start or end on pin-cell corners
    xml, xsl = W.minicore(n_lat=3, n_azi=8, spacing=0.05, precision="double")
    P, S, O = _pair(xml, xsl, precision)
    ra = m.EigenSolver(P, sweeper=S).solve()
    rb = O.solve()
    assert ra["converged"] and rb["converged"]
    assert pcm(ra["k"], rb["k"]) < (1e-4 if precision == 0 else PCM_TOL)
    assert max_pin_err(S.pin_powers(), O.pin_powers()) < (1e-8 if precision == 0 else PIN_TOL)


@pytest.mark.parametrize("precision", [0, 1])
def test_ihm_on_gpu(ref_xsl, precision):
    from test_oracle_known_answers import analytic_spectrum, ihm_problem
    # MOCC's 800 inner iterations: C5G7's UO2-3.3 scatters strongly within
    # the thermal groups, so fewer leave the within-group source unconverged
    P = ihm_problem(ref_xsl, n_inner=800)
    k_ref, phi = analytic_spectrum(P)
    S = m.MoCSweeper(P, precision)
    n = P.sizes["nfsr"]
    S.initialize()
    S.set_flux(np.tile(phi, (n, 1)))
    fs = S.calc_fission_source(k_ref)
    assert np.allclose(fs, 1.0, atol=1e-13)
    for g in range(P.sizes["ngroup"]):
        S.source_group(g)
        S.sweep(g)
        assert np.max(np.abs(S.flux()[:, g] - phi[g])) <= 0.005 * phi[g]


@pytest.mark.parametrize("kernel", [0, 1])
def test_assembly17_mixed_vs_oracle(kernel):
    xml, xsl = W.assembly17()
    P, S, O = _pair(xml, xsl, 1, sweep_kernel=kernel)
    ra = m.EigenSolver(P, sweeper=S).solve()
    rb = O.solve()
    assert ra["converged"] and rb["converged"]
    assert pcm(ra["k"], rb["k"]) < PCM_TOL
    assert max_pin_err(S.pin_powers(), O.pin_powers()) < PIN_TOL


def test_small_unit_cap_multi_unit_sweep():
    """A tiny FSR cap forces many work units per track set; results unchanged."""
    # the cap is fixed inside the library; a 7x7 lattice at fine spacing
    # spreads each track set over many units
    xml, xsl = W.lattice_case(7, 8, 0.02, "double", seed=3)
    P, S, O = _pair(xml, xsl, 0, n_inner=1)
    S.initialize()
    O.initialize()
    fs = O.calc_fission_source(1.0)
    S.set_fission_source(fs)
    for g in range(P.sizes["ngroup"]):
        S.source_group(g)
        O.source_group(g)
        S.sweep(g)
        O.sweep(g)
    assert np.max(np.abs(S.flux() - O.flux()) / np.abs(O.flux())) < FP64_TOL


def test_time_sweep_reports_launches():
    P = m.Problem(*W.pin3x3())
    S = m.MoCSweeper(P, 1)
    S.initialize()
    ms, nl = S.time_sweep(0, 3)
    assert nl == 6 and ms > 0.0
    before = m.launch_count()
    S.sweep(0)
    assert m.launch_count() - before >= 2


def test_mixed_wide_flux_range_matches_fp64():
    # mini-core with a 21 cm reflector and vacuum faces at coarse tracking:
    # the group fluxes span more than 20 decades, so a work unit's tally
    # takes contributions far below its largest one (the FP32 sweep's
    # fixed-point tally must hand those to its FP32 side path)
    xml, xsl = W.minicore(n_azi=2, spacing=0.1)
    P = m.Problem(xml, xsl)
    res, pins, flux = {}, {}, {}
    for precision in (0, 1):
        S = m.MoCSweeper(P, precision)
        res[precision] = m.EigenSolver(P, sweeper=S).solve()
        pins[precision] = S.pin_powers()
        flux[precision] = S.flux()
        S.close()
    assert res[0]["converged"] and res[1]["converged"]
    assert flux[0].max() / flux[0][flux[0] > 0].min() > 1e20
    assert (flux[1] > 0).all()
    assert pcm(res[1]["k"], res[0]["k"]) < PCM_TOL
    assert max_pin_err(pins[1], pins[0]) < PIN_TOL


@pytest.mark.parametrize("precision", [0, 1])
def test_row_windows_match_whole_units(precision):
    # units staged 16 rows at a time (two tables, the fixed-point scale
    # renewed per window) against the oracle, on a core with vacuum faces
    xml, xsl = W.minicore(n_lat=3, n_azi=4, spacing=0.05, precision="double")
    P, S, O = _pair(xml, xsl, precision, window_rows=16)
    lay = S.layout()
    assert lay["window_rows"] == 16
    ra = m.EigenSolver(P, sweeper=S).solve()
    rb = O.solve()
    assert ra["converged"] and rb["converged"]
    if precision == 0:
        assert ra["iterations"] == rb["iterations"]
        assert abs(ra["k"] - rb["k"]) / rb["k"] < 1e-9
        assert max_pin_err(S.pin_powers(), O.pin_powers()) < 1e-8
    else:
        assert pcm(ra["k"], rb["k"]) < PCM_TOL
        assert max_pin_err(S.pin_powers(), O.pin_powers()) < PIN_TOL
    # the same solve in whole units
    P0, S0, _ = _pair(xml, xsl, precision, window_rows=0)
    assert S0.layout()["window_rows"] == 0
    r0 = m.EigenSolver(P0, sweeper=S0).solve()
    assert abs(r0["k"] - ra["k"]) < (1e-12 if precision == 0 else 3e-6)


@pytest.mark.parametrize("option", ["angle_correction", "no_correction", "pin_trig", "chebyshev_gauss"])
def test_eigen_fp64_under_ray_options(option):
    # MOCC's other <rays> and quadrature options: the oracle traces the same
    # input itself (its tracer equals the library's, test_oracle_tracer.py)
    from test_oracle_tracer import RAY_OPTIONS
    xml, xsl = W.lattice_case(3, 8, 0.05, "double", seed=1000)
    old, new = RAY_OPTIONS[option]
    xml = xml.replace(old, new, 1)
    P, S, O = _pair(xml, xsl, 0)
    ra, rb = m.EigenSolver(P, sweeper=S).solve(), O.solve()
    assert ra["converged"] and rb["converged"]
    assert ra["iterations"] == rb["iterations"]
    assert abs(ra["k"] - rb["k"]) / rb["k"] < 1e-9
    assert max_pin_err(S.pin_powers(), O.pin_powers()) < 1e-8
