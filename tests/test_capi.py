"""C ABI: every declared symbol is exported; host-side errors map to codes."""
import ctypes
import re
from pathlib import Path

import pytest

import mocc_gb300 as m

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        names |= set(re.findall(r"\b(mocgpu_[a-z0-9_]+)\s*\(", h.read_text()))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(str(m.load_library()._name))
    syms = declared_symbols()
    assert len(syms) >= 30
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_error_codes():
    from mocc_gb300 import workloads as W
    xml, xsl = W.pin3x3()
    with pytest.raises(m.MocgpuError) as e:
        m.Problem("<solver", xsl)
    assert e.value.code == 2
    with pytest.raises(m.MocgpuError) as e:
        m.Problem(xml.replace('<solver type="eigenvalue"', '<solver type="fixed_source"'), xsl)
    assert e.value.code == 7
    with pytest.raises(m.MocgpuError) as e:
        m.Problem(xml, xsl.replace("fuel1", "fuelX"))
    assert e.value.code == 4
    with pytest.raises(m.MocgpuError) as e:
        m.Problem(xml.replace('spacing="0.05"', 'spacing="-1"'), xsl)
    assert e.value.code == 6
    with pytest.raises(m.MocgpuError) as e:
        m.Problem(xml.replace('np="1"', 'np="2"'), xsl)
    assert e.value.code == 5


def test_options_round_trip():
    from mocc_gb300 import workloads as W
    P = m.Problem(*W.pin3x3())
    o = P.options
    assert o["n_inner"] == 5 and o["cmfd"] == 1 and o["gs_boundary"] == 1 and o["precision"] == 0
    P.set_options(n_inner=3, precision=1)
    assert P.options["n_inner"] == 3 and P.options["precision"] == 1


def test_problem_sizes_pin3x3():
    from mocc_gb300 import workloads as W
    P = m.Problem(*W.pin3x3())
    s = P.sizes
    assert s["nfsr"] == 9 * 24 and s["npin"] == 9 and s["ngroup"] == 7
    assert s["nsets"] == 16 and s["pol_per_set"] == 3
    assert s["nsurf"] == 4 * 3 + 4 * 3 + 2 * 9
    b = P.export("trk_seg_begin")
    assert b[-1] == s["nseg"] and len(b) == s["ntracks"] + 1


def test_sweeper_requires_a_gpu():
    from conftest import has_gpu
    if has_gpu():
        pytest.skip("GPU present")
    from mocc_gb300 import workloads as W
    P = m.Problem(*W.pin3x3())
    with pytest.raises(m.MocgpuError) as e:
        m.MoCSweeper(P)
    assert e.value.code == 20


def test_batch_engine_requires_a_gpu():
    from conftest import has_gpu
    if has_gpu():
        pytest.skip("GPU present")
    with pytest.raises(m.MocgpuError) as e:
        m.BatchEngine(precision=1, capacity=4)
    assert e.value.code == 20


def test_sweep_ring_shapes_are_listed():
    shapes = m.sweep_shapes()
    assert len(shapes) == 5 and shapes[0] == (8, 2)
    assert len(set(shapes)) == len(shapes)
    assert all(r % 4 == 0 and s >= 2 for r, s in shapes)
