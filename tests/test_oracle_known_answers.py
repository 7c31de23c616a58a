"""The CPU oracle against MOCC's own known-answer tests.

* test_Exponential.cpp: table exponential within 2e-8 of exp on [-10, 0)
* test_MoC_IHM.cpp: infinite homogeneous medium -- after one sweep per group
  from the analytic spectrum the FSR flux equals the spectrum within 0.5 %
* test_MoCSweeper.cpp: get -> set -> get pin flux is the identity
The IHM case uses MOCC's own UO2-3.3 from its C5G7 library, as the reference
test does.
"""
import math

import numpy as np
import pytest

import mocc_gb300 as m
import oracle
from mocc_gb300 import workloads as W

IHM_GEOM = ('<mesh id="1" type="rect" pitch="1.26"><sub_x>3</sub_x><sub_y>3</sub_y></mesh>'
            '<pin id="1" mesh="1">1 1 1 1 1 1 1 1 1</pin>'
            '<lattice id="1" nx="3" ny="2">1 1 1 1 1 1</lattice>'
            '<assembly id="1" np="1" hz="0.5"><lattices>1</lattices></assembly>'
            '<core nx="1" ny="1" north="reflect" south="reflect" east="reflect" west="reflect" '
            'top="reflect" bottom="reflect">1</core>'
            '<material_lib path="x.xsl"><material id="1" name="UO2-3.3" /></material_lib>')


def ihm_problem(ref_xsl, n_inner=800, quad='<ang_quad type="ls" order="2" />', spacing=0.01, extra=""):
    solver = (f'<solver type="eigenvalue" k_tol="1e-8" psi_tol="1e-8" max_iter="300"><source scattering="P0" />'
              f'<sweeper type="moc" n_inner="{n_inner}" {extra}>{quad}<rays spacing="{spacing}" /></sweeper></solver>')
    return m.Problem(solver + IHM_GEOM, ref_xsl)


def analytic_spectrum(P):
    G = P.sizes["ngroup"]
    xstr = P.export("xstr").reshape(-1, G)[0]
    nf = P.export("xsnf").reshape(-1, G)[0]
    chi = P.export("xsch").reshape(-1, G)[0]
    S = P.export("scat").reshape(-1, G, G)[0]
    M = np.diag(xstr) - S
    phi = np.linalg.solve(M, chi)
    return float(nf @ phi), phi


def test_exponential_table():
    xs = np.arange(-10.0, 0.0, 0.1)
    err = max(abs(oracle.table_exp(x) - math.exp(x)) for x in xs)
    assert err < 2e-8
    # table nodes reproduce exp exactly (spacing 1e-3)
    for i in (0, 1, 137, 5000, 9999):
        x = -10.0 + i * (10.0 / 10000)
        assert abs(oracle.table_exp(x) - math.exp(x)) < 1e-15
    # outside the table the library exponential is used
    assert oracle.table_exp(-12.5) == pytest.approx(math.exp(-12.5), rel=1e-15)


def test_ihm_analytic_spectrum(ref_xsl):
    P = ihm_problem(ref_xsl)
    k_ref, phi = analytic_spectrum(P)
    o = oracle.OracleSolver(P)
    n, G = P.sizes["nfsr"], P.sizes["ngroup"]
    o.set_flux(np.tile(phi, (n, 1)))
    fs = o.calc_fission_source(k_ref)
    assert np.allclose(fs, 1.0, atol=1e-14)
    for g in range(G):
        o.source_group(g)
        o.sweep(g)
        f = o.flux()[:, g]
        assert np.max(np.abs(f - phi[g])) <= 0.005 * phi[g]


def test_ihm_eigenvalue_converges_to_k_inf(ref_xsl):
    # C5G7's UO2-3.3 scatters strongly with upscatter in the thermal groups:
    # ten inner iterations per group keep the power iteration short
    P = ihm_problem(ref_xsl, n_inner=10)
    k_ref, _ = analytic_spectrum(P)
    r = oracle.OracleSolver(P, max_iter=1000).solve()
    assert r["converged"]
    assert abs(r["k"] - k_ref) / k_ref < 5e-5


def test_pin_flux_get_set_identity(ref_xsl):
    from mocc_gb300 import workloads as W
    xml, xsl = W.pin3x3()
    P = m.Problem(xml, xsl)
    o = oracle.OracleSolver(P)
    o.initialize()
    rng = np.random.default_rng(3)
    o.set_flux(rng.uniform(0.5, 2.0, size=(P.sizes["nfsr"], P.sizes["ngroup"])))
    for g in (0, 3):
        a = o.get_pin_flux_1g(g)
        o.set_pin_flux_1g(g, a)
        b = o.get_pin_flux_1g(g)
        assert np.allclose(a, b, rtol=1e-13, atol=0)
    with pytest.raises(RuntimeError):
        o.set_pin_flux_1g(0, np.zeros(P.sizes["npin"]))


def test_jacobi_and_gauss_seidel_reach_same_k():
    from mocc_gb300 import workloads as W
    xml, xsl = W.pin3x3()
    P = m.Problem(xml, xsl)
    gs = oracle.OracleSolver(P, k_tol=1e-9, psi_tol=1e-8).solve()
    ja = oracle.OracleSolver(P, k_tol=1e-9, psi_tol=1e-8, gs_boundary=0).solve()
    nocmfd = oracle.OracleSolver(P, k_tol=1e-9, psi_tol=1e-8, cmfd=0, max_iter=2000).solve()
    for r in (gs, ja, nocmfd):
        assert r["converged"]
    assert abs(gs["k"] - ja["k"]) / gs["k"] < 1e-7
    assert abs(gs["k"] - nocmfd["k"]) / gs["k"] < 1e-6
    # CMFD accelerates: far fewer outer iterations
    assert gs["iterations"] < nocmfd["iterations"]


def test_thread_count_does_not_change_the_answer():
    from mocc_gb300 import workloads as W
    xml, xsl = W.pin3x3()
    P = m.Problem(xml, xsl)
    a = oracle.OracleSolver(P, n_threads=1).solve()
    b = oracle.OracleSolver(P, n_threads=4).solve()
    assert a["iterations"] == b["iterations"]
    assert abs(a["k"] - b["k"]) < 1e-12


def test_coarse_currents_balance_every_pin_cell():
    """The tallied coarse-surface currents close the neutron balance of every
    pin cell: the net outflow equals the one-group source minus the collision
    rate of the cell's FSRs. Eight azimuths per octant on a core with vacuum
    faces: many tracks pass through pin-cell corners, and some start or end
    on one, where the coarse walk must follow the traced segments."""
    import mocc_gb300 as m
    from mocc_gb300 import workloads as W
    import oracle
    xml, xsl = W.minicore(n_lat=3, n_azi=8, spacing=0.05, precision="double")
    P = m.Problem(xml, xsl)
    s = P.sizes
    O = oracle.OracleSolver(P, n_inner=1)
    O.initialize()
    O.set_coarse_data(True)
    G, nf, nx, ny = s["ngroup"], s["nfsr"], s["nx"], s["ny"]
    phi0 = np.random.default_rng(1).uniform(0.5, 2.0, size=(nf, G))
    O.set_flux(phi0)
    fs = O.calc_fission_source(1.0)
    g = 0
    O.source_group(g)
    O.sweep(g)
    phi1 = O.flux()[:, g]
    mat, vol = P.export("fsr_mat"), P.export("fsr_vol")
    xstr = P.export("xstr").reshape(-1, G)
    xsch = P.export("xsch").reshape(-1, G)
    scat = P.export("scat").reshape(-1, G, G)
    src = xsch[mat, g] * fs + np.einsum("rg,rg->r", scat[mat, g, :], phi0)
    coll = vol * (xstr[mat, g] * phi1 - src)
    pfr, pcell = P.export("pin_first_reg"), P.export("pin_cell")
    cur = O.coarse_currents()[0][g]
    dx, dy = P.export("dx"), P.export("dy")
    nxy = nx * ny
    worst = 0.0
    for ip in range(s["npin"]):
        c = pcell[ip]
        ix, iy = c % nx, c // nx
        e, w = nxy + (nx + 1) * iy + ix + 1, nxy + (nx + 1) * iy + ix
        n, so = nxy + (nx + 1) * ny + (ny + 1) * ix + iy + 1, nxy + (nx + 1) * ny + (ny + 1) * ix + iy
        out = (cur[e] - cur[w]) * dy[iy] + (cur[n] - cur[so]) * dx[ix]
        lhs = coll[pfr[ip]:pfr[ip + 1]].sum()
        worst = max(worst, abs(lhs + out) / abs(lhs))
    assert worst < 1e-10


def test_vacuum_core_with_corner_crossings_converges():
    import mocc_gb300 as m
    from mocc_gb300 import workloads as W
    import oracle
    xml, xsl = W.minicore(n_lat=3, n_azi=8, spacing=0.05, precision="double")
    P = m.Problem(xml, xsl)
    r = oracle.OracleSolver(P).solve()
    r0 = oracle.OracleSolver(P, cmfd=0).solve()
    assert r["converged"] and r["iterations"] < 20
    assert abs(r["k"] - r0["k"]) / r0["k"] < 2e-5  # CMFD accelerates, it does not move k


def test_homogenized_nu_fission_xsmesh_known_answers(golden, ref_xsl):
    """test_XSMeshHomogenized.cpp with MOCC's own C5G7 library: flat-flux
    (volume-weighted) pin-homogenised group-1 nu-Sigma_f of the 2x3
    UO2/MOX lattice (0.0125521 for a MOX pin, 0.0115752 for a UO2 pin) and
    of solid UO2 pins (2.005998e-2), each to the reference's 1e-6."""
    h = golden["xsmesh_homogenized"]
    solver = ('<solver type="eigenvalue" k_tol="1e-6" psi_tol="1e-5" max_iter="10"><sweeper type="moc" n_inner="1">'
              '<ang_quad type="ls" order="4" /><rays spacing="0.05" /></sweeper></solver>')
    pat = h["nu_fission_pattern"]
    assert sorted(set(pat)) == [0.0115752, 0.0125521]
    for key, solid in (("lattice_xml", False), ("solid_xml", True)):
        P = m.Problem(solver + h[key], ref_xsl)
        O = oracle.OracleSolver(P)
        O.initialize()  # flat flux: volume weighting
        hom = O.homogenized_nu_fission()[:, 0]
        assert P.sizes["npin"] == 72
        if solid:
            assert np.all(np.abs(hom - h["solid_uo2_nu_fission"]) < h["tol"])
            continue
        # the reference lists each 2x3 lattice's pins row by row from the
        # bottom; here pins are located by their coarse cell (x fastest)
        nx = P.sizes["nx"]
        cell = P.export("pin_cell")
        j = (cell // nx % 3) * 2 + (cell % nx % 2)
        assert np.all(np.abs(hom - np.array(pat)[j]) < h["tol"])


@pytest.mark.parametrize("case", ["lattice7", "core_vacuum"])
def test_cmfd_power_iteration_reaches_the_system_eigenvalue(case):
    """The CMFD restatement (homogenisation, setup_solve's operator, the power
    iteration with a BiCGSTAB solve per group) converges to the dominant
    eigenvalue of the CMFD system it builds, M phi = (1/k) F phi, with
    M = the per-group 5-point operators minus the in-scatter coupling and
    F = chi nu-Sigma_f, both times the cell volumes -- found here with a
    dense eigensolver. This pins the CMFD arithmetic independently of
    BiCGSTAB's own iterates (MOCC's BiCGSTAB is Eigen's, not vendored)."""
    if case == "lattice7":
        xml, xsl = W.lattice_case(7, 8, 0.05, "double", seed=1003, mod_factor=1.04)
    else:
        xml, xsl = W.minicore(n_lat=3, n_azi=4, spacing=0.05, precision="double")
    P = m.Problem(xml, xsl)
    O = oracle.OracleSolver(P, cmfd_k_tol=1e-13, cmfd_psi_tol=1e-12, cmfd_resid_reduction=1e-10,
                            cmfd_max_iter=3000)
    O.initialize()
    O.set_coarse_data(True)
    fs = O.calc_fission_source(1.0)
    for g in range(P.sizes["ngroup"]):
        O.source_group(g)
        O.sweep(g)
    sysd = O.cmfd_system()
    k_cmfd = O.cmfd_solve(1.0)
    op, G, n, nx = sysd["op"], P.sizes["ngroup"], P.sizes["npin"], P.sizes["nx"]
    vol = sysd["vol"]
    M = np.zeros((G * n, G * n))
    F = np.zeros((G * n, G * n))
    for g in range(G):
        r0 = g * n
        for i in range(n):
            M[r0 + i, r0 + i] = op[g, 0, i]
            ix = i % nx
            if ix > 0:
                M[r0 + i, r0 + i - 1] = op[g, 1, i]
            if ix < nx - 1:
                M[r0 + i, r0 + i + 1] = op[g, 2, i]
            if i >= nx:
                M[r0 + i, r0 + i - nx] = op[g, 3, i]
            if i + nx < n:
                M[r0 + i, r0 + i + nx] = op[g, 4, i]
            for gg in range(G):
                if gg != g:
                    M[r0 + i, gg * n + i] -= sysd["scat"][i, g, gg] * vol[i]
                F[r0 + i, gg * n + i] = sysd["xsch"][i, g] * sysd["xsnf"][i, gg] * vol[i]
    ev = np.linalg.eigvals(np.linalg.solve(M, F))
    k_eig = float(np.max(ev.real))
    assert abs(k_cmfd - k_eig) / k_eig < 1e-9
