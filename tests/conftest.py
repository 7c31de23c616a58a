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
    """Synthetic library whose material names match MOCC's test inputs."""
    import mocc_gb300 as m
    return (m.synthetic_xsl(1, 7, 2).replace("fuel1", "UO2-3.3").replace("fuel2", "MOX-4.3")
            .replace("moderator", "Moderator"))
