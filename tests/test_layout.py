"""Host-side checks of the bundled sweep layout (every real segment appears
exactly once, in its own track's lane, with its FSR and length; padding is
zero-length on the unit's padding slot; units respect the FSR cap)."""
import numpy as np
import pytest

import mocc_gb300 as m
from mocc_gb300 import workloads as W


@pytest.mark.parametrize("gs", [True, False])
@pytest.mark.parametrize("tpu,cap", [(32, 16384), (64, 16384), (256, 16384), (64, 200)])
def test_layout_covers_every_segment(gs, tpu, cap):
    P = m.Problem(*W.pin3x3())
    st = P.layout_stats(gs=gs, tracks_per_unit=tpu, max_local=cap)
    assert st["real_segments"] == P.sizes["nseg"]
    assert st["len_sum"] == pytest.approx(P.export("seg_len").sum(), rel=1e-12)
    assert st["max_local"] <= cap + 1  # the unit's FSRs and its padding slot
    assert st["phases"] == (2 if gs else 1)
    assert st["rows"] * 32 >= st["real_segments"]


def test_layout_assembly17_padding_small():
    P = m.Problem(*W.assembly17())
    st = P.layout_stats(gs=True, tracks_per_unit=32, max_local=16384)
    assert st["real_segments"] == P.sizes["nseg"]
    # tracks are sorted by length inside a unit: padding stays modest
    assert st["padding"] < 0.25


def test_layout_rejects_nothing_for_level_symmetric(golden, ref_xsl):
    solver = ('<solver type="eigenvalue" k_tol="1e-6" psi_tol="1e-5" max_iter="10"><sweeper type="moc" n_inner="1">'
              '<ang_quad type="ls" order="4" /><rays spacing="0.05" /></sweeper></solver>')
    P = m.Problem(solver + golden["square_xml"], ref_xsl)
    st = P.layout_stats(gs=True, tracks_per_unit=64)
    assert st["real_segments"] == P.sizes["nseg"]
