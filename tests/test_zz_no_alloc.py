"""mocgpu_cmfd_solve_static against mocgpu_cmfd_solve through the C ABI.

Two sweepers of one problem get the same flux, fission source and one FP64
sweep of every group (which tallies the coarse currents); one then runs the
CMFD solve with its work vectors in the handle's buffer, the other with them
in the library's fixed scratch array. Three outer steps on each (the CMFD
solve, then a sweep of every group from the rescaled flux) must agree: k to
1e-10 relative and fine flux to 1e-8 relative where both run
the single-CTA solver (the sweeps' atomic tallies are the only source of
difference); on a mesh above 1024 cells the buffered solve runs on a
thread-block cluster, so there the two agree to the BiCGSTAB tolerance.
A sweep separates the calls as in the power iteration: a CMFD solve started
from its own converged coarse flux asks BiCGSTAB for a residual far below
rounding, where MOCC's iteration (and the oracle's restatement of it) breaks
down. Calls after the first reuse the scratch left by the one before and must
leave free device memory unchanged; a mesh over the array's 8192 cells is
refused with MOCGPU_ERR_CAPACITY and the handle is left as it was. This
file is collected last so that it also runs after every other GPU test in
the same process.
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


def _sweep_all(S, G):
    for g in range(G):
        S.source_group(g)
        S.sweep(g)


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


def _case(name):
    if name == "pin3x3":
        return W.pin3x3()
    if name == "lattice7":
        return W.lattice_case(7, 8, 0.05, "double", seed=4)
    # 36x36 pins (1296 cells): the buffered solve runs on a thread-block
    # cluster there, the static one on a single CTA
    return W.minicore(n_lat=9, n_azi=2, spacing=0.1, precision="double")


# k and fine-flux agreement per case: the same solver on one CTA agrees to
# the sweeps' atomic-order rounding; against the cluster solver the BiCGSTAB
# iterations round differently and stop within their own tolerance
TOL = {"pin3x3": (1e-10, 1e-8), "lattice7": (1e-10, 1e-8), "core36": (1e-9, 1e-6)}


@pytest.mark.parametrize("case", ["pin3x3", "lattice7", "core36"])
def test_static_scratch_cmfd_matches_handle_buffer(case):
    import torch
    P = m.Problem(*_case(case))
    lib = _lib()
    a, b = _prepared(P), _prepared(P)
    ka, kb = C.c_double(1.0), C.c_double(1.0)
    k_tol, f_tol = TOL[case]
    free_before = None
    for call in range(3):
        assert lib.mocgpu_cmfd_solve(a.handle, C.byref(ka)) == 0, lib.mocgpu_last_error()
        if call == 1:
            # after the first call has loaded the kernel and looked up the
            # array: the static calls must not change free device memory
            torch.cuda.synchronize()
            free_before = torch.cuda.mem_get_info()[0]
        assert lib.mocgpu_cmfd_solve_static(b.handle, C.byref(kb)) == 0, lib.mocgpu_last_error()
        if call == 2:
            torch.cuda.synchronize()
            assert torch.cuda.mem_get_info()[0] == free_before
        assert np.isfinite(ka.value) and ka.value > 0.0
        assert abs(ka.value - kb.value) < k_tol * ka.value, (call, ka.value, kb.value)
        fa, fb = a.flux(), b.flux()
        assert np.max(np.abs(fa - fb) / np.abs(fa)) < f_tol, call
        if call < 2:
            # the next outer's transport sweep: the same fission source on both
            fs = a.calc_fission_source(ka.value)
            for S in (a, b):
                S.set_fission_source(fs)
                _sweep_all(S, P.sizes["ngroup"])


def test_static_scratch_refuses_oversized_mesh():
    # 92x92 pins = 8464 coarse cells, over the 8192 the array holds
    xml, xsl = W.minicore(n_lat=23, n_azi=2, spacing=0.5, precision="double")
    P = m.Problem(xml, xsl)
    assert P.sizes["npin"] > 8192
    lib = _lib()
    S = m.MoCSweeper(P, 0)
    S.initialize()
    S.set_coarse_data(True)
    before = S.flux()
    k = C.c_double(1.0)
    assert lib.mocgpu_cmfd_solve_static(S.handle, C.byref(k)) == 21
    assert b"8192" in lib.mocgpu_last_error()
    assert k.value == 1.0
    assert np.array_equal(S.flux(), before)
