"""mocgpu_cmfd_solve_static against mocgpu_cmfd_solve through the C ABI.

Two sweepers of one problem get the same flux, fission source and one FP64
sweep of every group (which tallies the coarse currents); one then runs the
CMFD solve with its work vectors in the handle's buffer, the other with them
in the library's fixed scratch array. Two calls in a row on each must agree
(k to 1e-10 relative, fine flux to 1e-8 relative; the sweeps' atomic
tallies are the only source of difference). The second call reuses the
scratch left by the first. This file is collected last so that it also runs
after every other GPU test in the same process.
"""
import ctypes as C

import numpy as np
import pytest

import mocc_gb300 as m
from mocc_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _lib():
    lib = m.load_library()
    for name in ("mocgpu_cmfd_solve", "mocgpu_cmfd_solve_static"):
        fn = getattr(lib, name)
        fn.restype = C.c_int
        fn.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
    return lib


def _prepared(P):
    S = m.MoCSweeper(P, 0)
    S.initialize()
    S.set_coarse_data(True)
    rng = np.random.default_rng(3)
    S.set_flux(rng.uniform(0.5, 2.0, size=(P.sizes["nfsr"], P.sizes["ngroup"])))
    S.set_fission_source(np.full(P.sizes["nfsr"], 1.0))
    for g in range(P.sizes["ngroup"]):
        S.source_group(g)
        S.sweep(g)
    return S


@pytest.mark.parametrize("case", ["pin3x3", "lattice7"])
def test_static_scratch_cmfd_matches_handle_buffer(case):
    xml, xsl = W.pin3x3() if case == "pin3x3" else W.lattice_case(7, 8, 0.05, "double", seed=4)
    P = m.Problem(xml, xsl)
    lib = _lib()
    a, b = _prepared(P), _prepared(P)
    ka, kb = C.c_double(1.0), C.c_double(1.0)
    for call in range(2):
        assert lib.mocgpu_cmfd_solve(a.handle, C.byref(ka)) == 0, lib.mocgpu_last_error()
        assert lib.mocgpu_cmfd_solve_static(b.handle, C.byref(kb)) == 0, lib.mocgpu_last_error()
        assert np.isfinite(ka.value) and ka.value > 0.0
        assert abs(ka.value - kb.value) < 1e-10 * ka.value, (call, ka.value, kb.value)
        fa, fb = a.flux(), b.flux()
        assert np.max(np.abs(fa - fb) / np.abs(fa)) < 1e-8, call
