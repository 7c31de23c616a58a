"""Failure paths of the library, each made on the host (no GPU fault):
a corrupt or unphysical cross-section library is refused with
MOCGPU_ERR_XS; a batched solve cancelled while queued or while running
retires with MOCGPU_ERR_CANCELLED and leaves the others' results as they
are alone; a device allocation that fails (injected through a test hook)
surfaces as MOCGPU_ERR_CUDA and leaves the engine usable."""
import numpy as np
import pytest

import mocc_gb300 as m
from mocc_gb300 import workloads as W


def _corrupt(xsl, which):
    lines = xsl.splitlines()
    i = next(k for k, l in enumerate(lines) if l.startswith("XSMACRO")) + 1
    vals = lines[i].split()
    if which == "text":
        vals[0] = "nan"
    else:
        # absorption so negative that the transport cross section is too
        vals[0] = "-1.0e3"
    lines[i] = " " + " ".join(vals)
    return "\n".join(lines) + "\n"


@pytest.mark.parametrize("which", ["text", "negative"])
def test_corrupt_cross_sections_are_refused(which):
    xml, xsl = W.pin3x3()
    with pytest.raises(m.MocgpuError) as e:
        m.Problem(xml, _corrupt(xsl, which))
    assert e.value.code == 4


@pytest.mark.gpu
@pytest.mark.parametrize("which", ["text", "negative"])
def test_corrupt_cross_sections_refused_at_submit(which):
    xml, xsl = W.lattice_case(3, 8, 0.05, "mixed", seed=1000)
    E = m.BatchEngine(precision=1, capacity=2)
    with pytest.raises(m.MocgpuError) as e:
        E.submit(m.Problem(xml, xsl), _corrupt(xsl, which))
    assert e.value.code == 4
    # the engine still runs good requests
    i = E.submit(m.Problem(xml, xsl), xsl)
    E.run()
    assert E.take(i)["error"] == 0


def _solo(xml, xsl):
    E = m.BatchEngine(precision=1, capacity=1)
    i = E.submit_xml(xml, xsl)
    E.run()
    r = E.take(i)
    E.close()
    return r


@pytest.mark.gpu
def test_cancelled_solves_leave_the_others_undisturbed():
    cases = [W.lattice_case(n, 8, 0.05, "mixed", seed=1000, mod_factor=f) for n, f in
             ((3, 0.95), (7, 1.0), (3, 1.05), (1, 1.02))]
    E = m.BatchEngine(precision=1, capacity=3)  # the fourth waits in the queue
    ids = [E.submit_xml(x, s) for x, s in cases]
    E.launch()  # three admitted, one replay in flight
    assert E.cancel(ids[1])  # running
    assert E.cancel(ids[3])  # queued
    assert not E.cancel(12345)
    E.run()
    res = [E.take(i) for i in ids]
    assert res[1]["error"] == 14 and res[3]["error"] == 14
    for k in (0, 2):
        ref = _solo(*cases[k])
        assert res[k]["error"] == 0 and res[k]["converged"] == 1
        assert abs(res[k]["k"] - ref["k"]) < 5e-7 * ref["k"]
        assert np.allclose(res[k]["pin_powers"], ref["pin_powers"], rtol=1e-5)
    assert not E.cancel(ids[0])  # finished


@pytest.mark.gpu
def test_failed_allocation_leaves_the_engine_usable():
    xml7, xsl7 = W.lattice_case(7, 8, 0.05, "mixed", seed=1000)
    xml3, xsl3 = W.lattice_case(3, 8, 0.05, "mixed", seed=1000)
    E = m.BatchEngine(precision=1, capacity=4)
    a = E.submit_xml(xml3, xsl3)
    E.run()
    assert E.take(a)["error"] == 0
    try:
        # the next device allocation (admitting a solve of a new lattice
        # shape needs its geometry and state) fails as out of memory
        m.fail_allocations_after(0)
        b = E.submit_xml(xml7, xsl7)
        with pytest.raises(m.MocgpuError) as e:
            E.run()
        assert e.value.code == 20 and "out of memory" in str(e.value)
    finally:
        m.fail_allocations_after(-1)
    # the request stayed queued: the engine admits and solves it now
    E.run()
    r = E.take(b)
    assert r["error"] == 0 and r["converged"] == 1
    assert abs(r["k"] - _solo(xml7, xsl7)["k"]) < 5e-7 * r["k"]
