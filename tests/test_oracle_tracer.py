"""The oracle's own input reader, core mesh, quadrature and ray tracer
(oracle/tracer.cpp, a restatement of MOCC's) against the library's tracer on
the same input text: every array of the flat problem must agree, integers
exactly and volumes and angles to rounding (the Gauss polar angles come from
Newton iterations whose last bits may differ), segment lengths to 1e-10 cm;
also under MOCC's other <rays> options (angle and no volume correction, pin
modularity, trigonometric modularisation) and the Chebyshev-Gauss
quadrature.

The library follows MOCC's coarse walk except at pin-cell corners (pin-line
crossings within 1e-10 cm of a ray end dropped, crossings shorter than
1e-9 cm folded into their neighbour, the surfaces between two crossings
taken from their cells). The oracle keeps MOCC's own walk as a mode, and the
last tests show where the two differ: nowhere on regular lattices, on a few
corner tracks of a core with vacuum faces, where MOCC's walk breaks the
pin-cell neutron balance and the documented one keeps it.
"""
from pathlib import Path

import numpy as np
import pytest

import mocc_gb300 as m
import oracle
from mocc_gb300 import workloads as W

GOLDEN = Path(__file__).resolve().parent / "golden"
SIZES = (("ng", "ngroup"), ("n_fsr", "nfsr"), ("n_mat", "nmat"), ("ndir_oct", "ndir_oct"), ("n_ang", "nang"),
         ("n_sets", "nsets"), ("pol_per_set", "pol_per_set"), ("nx", "nx"), ("ny", "ny"), ("n_pin", "npin"),
         ("n_surf", "nsurf"), ("n_fuel_2d", "nfuel"), ("n_tracks", "ntracks"), ("n_seg", "nseg"))
FIELDS = [f for f, t in oracle._P._fields_ if t is oracle.C.c_void_p]


def _case(name):
    c5 = (GOLDEN / "c5g7.xsl").read_text()
    if name.startswith("branch"):
        return W.lattice_case(int(name[6:]), 8, 0.05, "mixed", seed=1000)
    if name == "pin3x3":
        return W.pin3x3()
    if name == "core_corners":
        return W.minicore(n_lat=3, n_azi=8, spacing=0.05, precision="double")
    if name == "example_3x3":
        return (GOLDEN / "example_3x3.xml").read_text(), c5
    if name == "example_c5g7_2d":
        return (GOLDEN / "example_c5g7_2d.xml").read_text(), c5
    if name == "ihm":
        from test_oracle_known_answers import IHM_GEOM
        solver = ('<solver type="eigenvalue" k_tol="1e-8" psi_tol="1e-8" max_iter="300"><source scattering="P0" />'
                  '<sweeper type="moc" n_inner="2"><ang_quad type="ls" order="2" /><rays spacing="0.01" />'
                  '</sweeper></solver>')
        return solver + IHM_GEOM, c5
    raise KeyError(name)


@pytest.mark.parametrize("name", ["pin3x3", "branch1", "branch3", "branch7", "branch17", "core_corners",
                                  "example_3x3", "example_c5g7_2d", "ihm"])
def test_oracle_tracer_matches_library(name):
    xml, xsl = _case(name)
    P = m.Problem(xml, xsl)
    T = oracle.Traced(xml, xsl)
    s = P.sizes
    for k, src in SIZES:
        assert getattr(T.problem, k) == s[src], k
    assert T.problem.hz == P.export("hz")[0]
    assert list(T.problem.bc) == list(P.export("bc"))
    for f in FIELDS:
        a, b = np.asarray(P.export(f)), T.array(f)
        assert a.shape == b.shape, f
        if a.dtype.kind == "f":
            # angles in rad, weights, areas: rounding only; a segment length
            # can move by more where a track nearly grazes a ring (the chord
            # length is steep in the track's angle there)
            tol = 1e-10 if f == "seg_len" else 1e-13
            assert np.max(np.abs(a - b) / np.maximum(np.abs(a), 1.0), initial=0.0) < tol, f
        else:
            assert np.array_equal(a, b), f
    o = T.options
    for k, v in P.options.items():
        if k in o and k != "precision":
            assert o[k] == pytest.approx(v), k


RAY_OPTIONS = {
    "angle_correction": ('<rays spacing="0.05"', '<rays spacing="0.05" volume_correction="angle"'),
    "no_correction": ('<rays spacing="0.05"', '<rays spacing="0.05" volume_correction="none"'),
    "pin_modular": ('<rays spacing="0.05"', '<rays spacing="0.05" modularity="pin"'),
    "trig_modularisation": ('<rays spacing="0.05"', '<rays spacing="0.05" modularization="trig"'),
    "pin_trig": ('<rays spacing="0.05"', '<rays spacing="0.05" modularity="pin" modularization="trig"'),
    "chebyshev_gauss": ('type="cy"', 'type="cg"'),
}


@pytest.mark.parametrize("option", sorted(RAY_OPTIONS))
def test_oracle_tracer_matches_library_ray_options(option):
    # the <rays> and <ang_quad> options of ray_data.cpp:67-134 and
    # angular_quadrature.cpp on a 3x3 lattice: MOCC's other volume
    # corrections, pin modularity, trigonometric modularisation and the
    # Chebyshev-Gauss product quadrature
    xml, xsl = W.lattice_case(3, 8, 0.05, "double", seed=1000)
    old, new = RAY_OPTIONS[option]
    assert old in xml
    xml = xml.replace(old, new, 1)
    P = m.Problem(xml, xsl)
    T = oracle.Traced(xml, xsl)
    assert T.problem.n_seg == P.sizes["nseg"] and T.problem.n_tracks == P.sizes["ntracks"]
    for f in FIELDS:
        a, b = np.asarray(P.export(f)), T.array(f)
        assert a.shape == b.shape, f
        if a.dtype.kind == "f":
            tol = 1e-10 if f == "seg_len" else 1e-13
            assert np.max(np.abs(a - b) / np.maximum(np.abs(a), 1.0), initial=0.0) < tol, f
        else:
            assert np.array_equal(a, b), f
    if option == "no_correction":
        # uncorrected lengths: each set's segment volumes differ from the areas
        v = np.zeros(P.sizes["nfsr"])
        sb, ln, fs = T.array("trk_seg_begin"), T.array("seg_len"), T.array("seg_fsr")
        s0 = T.array("set_first_track")
        sp = T.array("set_spacing")
        for t in range(s0[0], s0[1]):
            np.add.at(v, fs[sb[t]:sb[t + 1]], ln[sb[t]:sb[t + 1]] * sp[0])
        assert not np.allclose(v, T.array("fsr_area"), rtol=1e-9)


def _coarse(T, t):
    b = T.array("trk_cm_begin")
    return (T.array("trk_cm_cell_fw")[t], T.array("trk_cm_cell_bw")[t], T.array("trk_cm_surf_fw")[t],
            T.array("trk_cm_surf_bw")[t],
            *(tuple(T.array(k)[b[t]:b[t + 1]]) for k in ("cm_fw", "cm_bw", "cm_nseg_fw", "cm_nseg_bw")))


@pytest.mark.parametrize("name", ["pin3x3", "branch7"])
def test_mocc_literal_walk_is_the_same_away_from_corners(name):
    xml, xsl = _case(name)
    A, B = oracle.Traced(xml, xsl), oracle.Traced(xml, xsl, mocc_literal=True)
    for f in FIELDS:
        assert np.array_equal(A.array(f), B.array(f)), f


def test_mocc_literal_walk_differs_at_corners_and_breaks_the_balance():
    xml, xsl = _case("core_corners")
    A, B = oracle.Traced(xml, xsl), oracle.Traced(xml, xsl, mocc_literal=True)
    n = A.problem.n_tracks
    ba, bb = A.array("trk_seg_begin"), B.array("trk_seg_begin")
    la, lb = A.array("seg_len"), B.array("seg_len")
    differ = [t for t in range(n) if _coarse(A, t) != _coarse(B, t)]
    assert 0 < len(differ) < 0.01 * n
    # the segments MOCC's walk keeps and the documented one drops are
    # corner slivers
    for t in range(n):
        sa, sb = la[ba[t]:ba[t + 1]], lb[bb[t]:bb[t + 1]]
        if len(sb) != len(sa):
            assert len(sb) > len(sa) and np.sort(sb)[:len(sb) - len(sa)].max() < 1e-9
    # pin-cell balance of one sweep: net coarse-surface outflow equals the
    # cell's source minus its collisions (the documented walk keeps it)
    worst = {}
    for mode, T in (("documented", A), ("mocc", B)):
        O = oracle.OracleSolver(T, n_inner=1)
        O.initialize()
        O.set_coarse_data(True)
        G, nf, nx, ny = O.n_group, O.n_reg, O.nx, O.ny
        phi0 = np.random.default_rng(1).uniform(0.5, 2.0, size=(nf, G))
        O.set_flux(phi0)
        fs = O.calc_fission_source(1.0)
        O.source_group(0)
        O.sweep(0)
        phi1 = O.flux()[:, 0]
        mat, vol = T.array("fsr_mat"), T.array("fsr_vol")
        xstr = T.array("xstr").reshape(-1, G)
        xsch = T.array("xsch").reshape(-1, G)
        scat = T.array("scat").reshape(-1, G, G)
        src = xsch[mat, 0] * fs + np.einsum("rg,rg->r", scat[mat, 0, :], phi0)
        coll = vol * (xstr[mat, 0] * phi1 - src)
        pfr, pcell = T.array("pin_first_reg"), T.array("pin_cell")
        cur = O.coarse_currents()[0][0]
        dx, dy = T.array("dx"), T.array("dy")
        nxy = nx * ny
        w = 0.0
        for ip in range(nxy):
            c = pcell[ip]
            ix, iy = c % nx, c // nx
            e, wst = nxy + (nx + 1) * iy + ix + 1, nxy + (nx + 1) * iy + ix
            nn, so = nxy + (nx + 1) * ny + (ny + 1) * ix + iy + 1, nxy + (nx + 1) * ny + (ny + 1) * ix + iy
            out = (cur[e] - cur[wst]) * dy[iy] + (cur[nn] - cur[so]) * dx[ix]
            lhs = coll[pfr[ip]:pfr[ip + 1]].sum()
            w = max(w, abs(lhs + out) / abs(lhs))
        worst[mode] = w
    assert worst["documented"] < 1e-10
    assert worst["mocc"] > 1e-3


def test_oracle_solve_on_its_own_trace_matches_the_library_arrays():
    xml, xsl = _case("branch3")
    a = oracle.OracleSolver.from_xml(xml, xsl).solve()
    b = oracle.OracleSolver(m.Problem(xml, xsl)).solve()
    assert a["iterations"] == b["iterations"]
    assert abs(a["k"] - b["k"]) < 1e-12
