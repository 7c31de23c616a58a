import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built sm_103a library")
    config.addinivalue_line("markers", "slow: longer CPU oracle runs")


def has_gpu():
    import mocc_gb300 as m
    import ctypes
    lib = m.load_library()
    n = ctypes.c_int(0)
    lib.mocgpu_device_count(ctypes.byref(n))
    return n.value > 0


@pytest.fixture(scope="session")
def golden():
    import json
    return json.loads((ROOT / "tests" / "golden" / "reference_known_answers.json").read_text())


@pytest.fixture(scope="session")
def ref_xsl():
    """MOCC's own 7-group C5G7 library (the c5g7.xsl of its tests and
    examples), copied into tests/golden by make_golden.py."""
    return (ROOT / "tests" / "golden" / "c5g7.xsl").read_text()


@pytest.fixture(scope="session")
def ref_example():
    """MOCC's example inputs, unchanged: name -> XML text."""
    g = ROOT / "tests" / "golden"
    return {"3x3": (g / "example_3x3.xml").read_text(), "c5g7_2d": (g / "example_c5g7_2d.xml").read_text()}
