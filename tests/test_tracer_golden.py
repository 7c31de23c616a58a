"""Ray tracer against MOCC's own known answers (src/sweepers/moc/tests)."""
import math

import numpy as np

import mocc_gb300 as m

SURF = {"EAST": 0, "NORTH": 1, "WEST": 2, "SOUTH": 3}


def test_weird_ray_segments(golden, ref_xsl):
    # test_Ray.cpp weird_ray: 36 segments, golden FSR ids, lengths to 1e-15
    w = golden["weird_ray"]
    r = m.trace_ray(w["xml"], ref_xsl, w["p1"], w["p2"])
    assert list(r["seg_fsr"]) == w["seg_index"]
    assert np.max(np.abs(r["seg_len"] - np.array(w["seg_len"]))) <= w["tol"]


def test_simple_ray_coarse_data(golden, ref_xsl):
    # test_Ray.cpp simple_ray on 6x5.xml: coarse cells/surfaces and crossings
    for c in golden["simple_ray"]:
        r = m.trace_ray(golden["six_by_five_xml"], ref_xsl, c["p1"], c["p2"])
        assert r["cm_surf_fw"] == c["cm_surf_fw"]
        assert r["cm_cell_fw"] == c["cm_cell_fw"]
        assert r["cm_surf_bw"] == c["cm_surf_bw"]
        assert r["cm_cell_bw"] == c["cm_cell_bw"]
        assert len(r["seg_len"]) == c["nseg"]
        assert len(r["cm"]) == c["ncseg"]
        if "fw" in c:
            assert list(r["cm"][:, 0]) == [SURF[s] for s in c["fw"]]
            assert list(r["cm"][:, 1]) == [SURF[s] for s in c["bw"]]
            assert list(r["cm"][:, 2]) == c["nseg_cm"]
            assert list(r["cm"][:, 3]) == c["nseg_cm"]
            assert np.allclose(r["seg_len"], c["seg_len"], atol=1e-5)


def test_big_ray_single_crossing(golden, ref_xsl):
    b = golden["big_ray"]
    r = m.trace_ray(golden["large_xml"], ref_xsl, b["p1"], b["p2"])
    assert len(r["cm"]) == b["ncseg"]


def _square_problem(golden, ref_xsl, quad, spacing, extra=""):
    solver = (f'<solver type="eigenvalue" k_tol="1e-6" psi_tol="1e-5" max_iter="10">'
              f'<sweeper type="moc" n_inner="1" {extra}>{quad}<rays spacing="{spacing}" /></sweeper></solver>')
    return m.Problem(solver + golden["square_xml"], ref_xsl)


def test_raydata_volume_conservation(golden, ref_xsl):
    # test_RayData.cpp: sum len * spacing * w * 2pi over octants 1-2 == area * 4pi
    v = golden["raydata_volume"]
    P = _square_problem(golden, ref_xsl, v["ang_quad"], v["spacing"])
    s = P.sizes
    w = P.export("ang_weight")
    sp = P.export("set_spacing")
    ft = P.export("set_first_track")
    sb = P.export("trk_seg_begin")
    L = P.export("seg_len")
    F = P.export("seg_fsr")
    nd, pol = s["ndir_oct"], s["pol_per_set"]
    vol = np.zeros(s["nfsr"])
    for iang in range(2 * nd):
        st = (iang % nd) // pol + (iang // nd) * (s["nsets"] // 2)
        a, b = sb[ft[st]], sb[ft[st + 1]]
        np.add.at(vol, F[a:b], L[a:b] * sp[st] * w[iang] * 2.0 * math.pi)
    assert np.max(np.abs(vol - v["area_4pi"] * 4.0 * math.pi)) < v["tol"]


def test_quadrature_reflect_reverse_weights(golden, ref_xsl):
    # test_AngularQuadrature.cpp: reflections negate one cosine, LS4 reverse
    # maps, weights sum to 8 over all octants (here octants 1-4 sum to 4)
    P = _square_problem(golden, ref_xsl, '<ang_quad type="ls" order="4" />', 0.05)
    ox, oy, w = P.export("ang_ox"), P.export("ang_oy"), P.export("ang_weight")
    nd = P.sizes["ndir_oct"]
    assert nd == 3
    assert abs(w.sum() - 4.0) < 1e-13
    tabx = [1, 0, 3, 2]
    taby = [3, 2, 1, 0]
    for i in range(4 * nd):
        o = i // nd
        jx = i + (tabx[o] - o) * nd
        jy = i + (taby[o] - o) * nd
        assert abs(ox[i] + ox[jx]) < 1e-13 and abs(oy[i] - oy[jx]) < 1e-13
        assert abs(oy[i] + oy[jy]) < 1e-13 and abs(ox[i] - ox[jy]) < 1e-13
    rev = lambda i: (i + 2 * nd) % (4 * nd)
    assert rev(1) == 7 and rev(11) == 5


def test_chebyshev_yamamoto_modularised_weights(golden, ref_xsl):
    P = _square_problem(golden, ref_xsl, '<ang_quad type="cy" n_azimuthal="4" n_polar="3" />', 0.05)
    w = P.export("ang_weight")
    assert abs(w.sum() - 4.0) < 1e-12
    # modularised azimuths keep the set symmetric about pi/4
    al = P.export("ang_alpha")[: P.sizes["ndir_oct"]: 3]
    assert np.allclose(al + al[::-1], math.pi / 2, atol=1e-12)


def test_every_fsr_has_segments_and_flat_correction(golden, ref_xsl):
    P = _square_problem(golden, ref_xsl, '<ang_quad type="cy" n_azimuthal="4" n_polar="3" />', 0.02)
    s = P.sizes
    F = P.export("seg_fsr")
    assert F.min() >= 0 and F.max() < s["nfsr"]
    assert len(np.unique(F)) == s["nfsr"]
    # flat correction: per track set, sum len*spacing == FSR area exactly
    sp, ft, sb, L = P.export("set_spacing"), P.export("set_first_track"), P.export("trk_seg_begin"), P.export("seg_len")
    area = P.export("fsr_area")
    for st in range(s["nsets"]):
        a, b = sb[ft[st]], sb[ft[st + 1]]
        v = np.zeros(s["nfsr"])
        np.add.at(v, F[a:b], L[a:b] * sp[st])
        assert np.allclose(v, area, rtol=1e-13)
