"""The MOCC binding of INTEGRATION.md, compiled: tests/binding/moc_sweeper_gpu.hpp
(a TransportSweeper forwarding every duty to the C ABI) against a stand-in
of MOCC's interface, driven by a restatement of MOCC's EigenSolver::solve /
step and FixedSourceSolver::step (tests/binding/eigen_driver.cpp). It must
build and link against libmocgpu.so with -Wall clean; without a GPU it exits
with the library's no-device error. On a GPU, the binding's solve of a 3x3
lattice and of MOCC's own examples/3x3.xml (with MOCC's c5g7.xsl) gives the
library's own eigen solve to rounding and the FP64 oracle's k."""
import json
import subprocess
from pathlib import Path

import pytest

import mocc_gb300 as m
import oracle
from mocc_gb300 import workloads as W

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    lib = m.load_library()
    out = tmp_path_factory.mktemp("binding") / "eigen_driver"
    libdir = Path(lib._name).parent
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Werror", f"-I{ROOT / 'include'}", f"-I{ROOT / 'tests' / 'binding'}",
           str(ROOT / "tests" / "binding" / "eigen_driver.cpp"), f"-L{libdir}", "-lmocgpu", f"-Wl,-rpath,{libdir}",
           "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def _inputs(tmp_path, xml, xsl):
    (tmp_path / "in.xml").write_text(xml)
    (tmp_path / "lib.xsl").write_text(xsl)
    return str(tmp_path / "in.xml"), str(tmp_path / "lib.xsl")


def test_binding_builds_and_reports_missing_gpu(driver, tmp_path):
    from conftest import has_gpu
    if has_gpu():
        pytest.skip("GPU present")
    r = subprocess.run([str(driver), *_inputs(tmp_path, *W.pin3x3())], capture_output=True, text=True)
    assert r.returncode == 3, (r.returncode, r.stderr)
    assert "CUDA" in r.stderr


def _run(driver, tmp_path, xml, xsl, precision=0):
    r = subprocess.run([str(driver), *_inputs(tmp_path, xml, xsl), str(precision)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return json.loads(r.stdout)


@pytest.mark.gpu
def test_binding_solve_matches_library_and_oracle(driver, tmp_path):
    xml, xsl = W.pin3x3()
    rb = _run(driver, tmp_path, xml, xsl)
    ra = m.EigenSolver(m.Problem(xml, xsl), 0).solve()
    ro = oracle.OracleSolver.from_xml(xml, xsl).solve()
    assert rb["converged"] == 1 and rb["iterations"] == ra["iterations"] == ro["iterations"]
    assert abs(rb["k"] - ra["k"]) < 1e-12
    assert abs(rb["k"] - ro["k"]) / ro["k"] < 1e-9


@pytest.mark.gpu
def test_binding_on_mocc_example_input(driver, tmp_path, ref_example, ref_xsl):
    rb = _run(driver, tmp_path, ref_example["3x3"], ref_xsl)
    ra = m.EigenSolver(m.Problem(ref_example["3x3"], ref_xsl), 0).solve()
    assert rb["converged"] == ra["converged"] and rb["iterations"] == ra["iterations"]
    assert abs(rb["k"] - ra["k"]) < 1e-12
