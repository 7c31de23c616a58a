"""CPU oracle for the GPU library -- TEST INFRASTRUCTURE ONLY.

FP64 OpenMP restatement of MOCC's 2-D MoC eigenvalue path (see oracle.h for
the routine-by-routine citations). Used by tests/, ``__graft_entry__.smoke``
and the CPU legs of ``bench.py`` as the checker; the product never loads it.

``OracleSolver.from_xml(xml, xsl)`` builds the problem with the oracle's own
restatement of MOCC's input reading, core mesh, quadrature and ray tracer
(tracer.cpp) and loads nothing of the library it checks; ``Traced`` exposes
those traced arrays for comparison. ``OracleSolver(problem)`` instead takes
the flat arrays of a traced ``mocc_gb300.Problem`` (unit checks of one
routine on exactly the library's geometry).

``build()`` compiles ``oracle/_build/liboracle.so`` from oracle.cpp and
tracer.cpp with g++ (``oracle/Makefile`` holds the same recipe).
"""
from __future__ import annotations

import ctypes as C
import hashlib
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build"
_LIB = None


class _P(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("ng", "n_fsr", "n_mat", "ndir_oct", "n_ang", "n_sets", "pol_per_set",
                                       "nx", "ny", "n_pin", "n_surf", "n_fuel_2d", "n_tracks")] + [
        ("n_seg", C.c_int64), ("hz", C.c_double), ("bc", C.c_int * 6)] + [
        (n, C.c_void_p) for n in ("xstr", "xsnf", "xsf", "xsch", "scat", "fsr_mat", "fsr_vol", "fsr_area",
                                  "ang_ox", "ang_oy", "ang_oz", "ang_alpha", "ang_theta", "ang_weight",
                                  "ang_rsintheta", "set_nx", "set_ny", "set_first_track", "set_spacing",
                                  "trk_bc0", "trk_bc1", "trk_set", "trk_seg_begin", "trk_cm_cell_fw",
                                  "trk_cm_cell_bw", "trk_cm_surf_fw", "trk_cm_surf_bw", "trk_cm_begin", "cm_fw",
                                  "cm_bw", "cm_nseg_fw", "cm_nseg_bw", "seg_len", "seg_fsr", "dx", "dy",
                                  "pin_first_reg", "pin_cell", "pin_fuel", "pin_area")]


class _O(C.Structure):
    _fields_ = [("k_tol", C.c_double), ("psi_tol", C.c_double), ("max_iter", C.c_int), ("min_iter", C.c_int),
                ("cmfd", C.c_int), ("cmfd_enabled", C.c_int), ("cmfd_k_tol", C.c_double),
                ("cmfd_psi_tol", C.c_double), ("cmfd_resid_reduction", C.c_double), ("cmfd_max_iter", C.c_int),
                ("cmfd_negative_fixup", C.c_int), ("n_inner", C.c_int), ("gs_boundary", C.c_int),
                ("precision", C.c_int), ("incoming_update", C.c_int), ("tl_splitting", C.c_int)]


class _R(C.Structure):
    _fields_ = [("k", C.c_double), ("iterations", C.c_int), ("converged", C.c_int), ("error_k", C.c_double),
                ("error_psi", C.c_double), ("seconds", C.c_double), ("sweeps", C.c_int64),
                ("cmfd_iterations", C.c_int64)]


def build(force: bool = False) -> Path:
    srcs = [HERE / "oracle.cpp", HERE / "tracer.cpp"]
    hdr = HERE / "oracle.h"
    cmd = ["g++", "-std=c++17", "-O3", "-fopenmp", "-fPIC", "-shared"] + [str(x) for x in srcs] + ["-o"]
    digest = hashlib.sha256(b"".join(x.read_bytes() for x in srcs) + hdr.read_bytes()
                            + " ".join(cmd).encode()).hexdigest()
    OUT.mkdir(exist_ok=True)
    lib, stamp = OUT / "liboracle.so", OUT / "liboracle.stamp"
    if not force and lib.exists() and stamp.exists() and stamp.read_text() == digest:
        return lib
    tmp = OUT / "liboracle.so.tmp"
    r = subprocess.run(cmd + [str(tmp)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    tmp.replace(lib)
    stamp.write_text(digest)
    return lib


def load():
    global _LIB
    if _LIB is None:
        lib = C.CDLL(str(build()))
        V, I, D = C.c_void_p, C.c_int, C.c_double
        DP = C.POINTER(C.c_double)
        for name, res, args in [
            ("orc_last_error", C.c_char_p, []), ("orc_create", I, [C.POINTER(_P), C.POINTER(_O), I, C.POINTER(V)]),
            ("orc_destroy", None, [V]), ("orc_threads", I, [V]), ("orc_initialize", I, [V]),
            ("orc_set_coarse_data", I, [V, I]), ("orc_calc_fission_source", I, [V, D, DP]),
            ("orc_set_fission_source", I, [V, DP]), ("orc_store_old_flux", I, [V]),
            ("orc_source_group", I, [V, I]), ("orc_sweep_group", I, [V, I]), ("orc_total_fission", I, [V, I, DP]),
            ("orc_flux_residual", I, [V, DP]), ("orc_get_flux", I, [V, DP]), ("orc_set_flux", I, [V, DP]),
            ("orc_get_pin_flux_1g", I, [V, I, DP]), ("orc_set_pin_flux_1g", I, [V, I, DP, DP]),
            ("orc_pin_powers", I, [V, DP]), ("orc_get_coarse_currents", I, [V, DP, DP]),
            ("orc_get_boundary", I, [V, I, DP, C.POINTER(C.c_int64)]),
            ("orc_update_incoming", I, [V, DP, DP, I, I]),
            ("orc_cmfd_solve", I, [V, DP]), ("orc_homogenized_nu_fission", I, [V, DP]),
            ("orc_cmfd_system", I, [V, DP, DP, DP, DP, DP]), ("orc_eigen_solve", I, [V, I, C.POINTER(_R)]),
            ("orc_history", I, [V, C.POINTER(C.POINTER(C.c_double)), C.POINTER(C.c_int64)]),
            ("orc_apply_transverse_leakage", I, [V, I, DP]),
            ("orc_table_exp", D, [D]),
            ("orc_trace_error", C.c_char_p, []), ("orc_trace", I, [C.c_char_p, C.c_char_p, I, C.POINTER(V)]),
            ("orc_traced_destroy", None, [V]), ("orc_traced_problem", C.POINTER(_P), [V]),
            ("orc_traced_options", C.POINTER(_O), [V]),
            ("orc_traced_array", I, [V, C.c_char_p, C.POINTER(V), C.POINTER(C.c_int64), C.POINTER(I)]),
        ]:
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = lib
    return _LIB


def _chk(rc):
    if rc != 0:
        raise RuntimeError("oracle: " + _LIB.orc_last_error().decode())


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def table_exp(x: float) -> float:
    return load().orc_table_exp(x)


class Traced:
    """A problem traced by the oracle itself from MOCC input text
    (``mocc_literal``: MOCC's own corner handling of the coarse walk)."""

    def __init__(self, xml: str, xsl: str, mocc_literal: bool = False):
        lib = load()
        h = C.c_void_p()
        if lib.orc_trace(xml.encode(), xsl.encode(), 1 if mocc_literal else 0, C.byref(h)) != 0:
            raise RuntimeError("oracle tracer: " + lib.orc_trace_error().decode())
        self._h, self._lib = h, lib
        self.problem = lib.orc_traced_problem(h).contents
        o = lib.orc_traced_options(h).contents
        self.options = {k: getattr(o, k) for k, _ in _O._fields_}

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.orc_traced_destroy(self._h)
            self._h = None

    def array(self, name: str) -> np.ndarray:
        """Copy of one traced array (the orc_problem field names)."""
        d, n, kind = C.c_void_p(), C.c_int64(), C.c_int()
        if self._lib.orc_traced_array(self._h, name.encode(), C.byref(d), C.byref(n), C.byref(kind)) != 0:
            raise KeyError(name)
        ct = {0: C.c_int32, 1: C.c_double, 2: C.c_int64}[kind.value]
        if n.value == 0:
            return np.zeros(0, dtype=np.dtype(ct))
        return np.ctypeslib.as_array(C.cast(d, C.POINTER(ct)), shape=(n.value,)).copy()


class OracleSolver:
    """FP64 restatement of MOCC's eigenvalue path on one problem: built with
    the oracle's own tracer (``from_xml``) or over the flat arrays of a
    traced ``mocc_gb300.Problem``."""

    FIELDS = [f for f, t in _P._fields_ if t is C.c_void_p]

    def __init__(self, problem, n_threads: int = 0, **option_overrides):
        lib = load()
        if isinstance(problem, Traced):
            self._traced = problem
            p = problem.problem
            opts = dict(problem.options)
        else:
            s = problem.sizes
            self._keep = {f: np.ascontiguousarray(problem.export(f)) for f in self.FIELDS}
            p = _P()
            for k, src in (("ng", "ngroup"), ("n_fsr", "nfsr"), ("n_mat", "nmat"), ("ndir_oct", "ndir_oct"),
                           ("n_ang", "nang"), ("n_sets", "nsets"), ("pol_per_set", "pol_per_set"), ("nx", "nx"),
                           ("ny", "ny"), ("n_pin", "npin"), ("n_surf", "nsurf"), ("n_fuel_2d", "nfuel"),
                           ("n_tracks", "ntracks")):
                setattr(p, k, int(s[src]))
            p.n_seg = int(s["nseg"])
            p.hz = float(problem.export("hz")[0])
            bc = problem.export("bc")
            for i in range(6):
                p.bc[i] = int(bc[i])
            for f, arr in self._keep.items():
                setattr(p, f, arr.ctypes.data_as(C.c_void_p))
            opts = dict(problem.options)
        self._p = p
        opts.update(option_overrides)
        o = _O(**{k: opts[k] for k, _ in _O._fields_})
        self._o = o
        h = C.c_void_p()
        _chk(lib.orc_create(C.byref(p), C.byref(o), n_threads, C.byref(h)))
        self._h = h
        self._lib = lib
        self.n_group, self.n_reg, self.n_pin = int(p.ng), int(p.n_fsr), int(p.n_pin)
        self.nx, self.ny, self.n_surf = int(p.nx), int(p.ny), int(p.n_surf)
        self.n_seg = int(p.n_seg)

    @classmethod
    def from_xml(cls, xml: str, xsl: str, n_threads: int = 0, **option_overrides):
        """The oracle on a problem it traces itself from MOCC input text."""
        return cls(Traced(xml, xsl), n_threads=n_threads, **option_overrides)

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.orc_destroy(self._h)
            self._h = None

    @property
    def threads(self):
        return self._lib.orc_threads(self._h)

    def initialize(self):
        _chk(self._lib.orc_initialize(self._h))

    def set_coarse_data(self, on=True):
        _chk(self._lib.orc_set_coarse_data(self._h, 1 if on else 0))

    def calc_fission_source(self, k):
        fs = np.empty(self.n_reg)
        _chk(self._lib.orc_calc_fission_source(self._h, k, _dp(fs)))
        return fs

    def set_fission_source(self, fs):
        fs = np.ascontiguousarray(fs, dtype=np.float64)
        _chk(self._lib.orc_set_fission_source(self._h, _dp(fs)))

    def store_old_flux(self):
        _chk(self._lib.orc_store_old_flux(self._h))

    def source_group(self, g):
        _chk(self._lib.orc_source_group(self._h, g))

    def sweep(self, g):
        _chk(self._lib.orc_sweep_group(self._h, g))

    def total_fission(self, old=False):
        v = C.c_double()
        _chk(self._lib.orc_total_fission(self._h, 1 if old else 0, C.byref(v)))
        return v.value

    def flux(self):
        f = np.empty((self.n_reg, self.n_group))
        _chk(self._lib.orc_get_flux(self._h, _dp(f)))
        return f

    def set_flux(self, f):
        f = np.ascontiguousarray(f, dtype=np.float64)
        _chk(self._lib.orc_set_flux(self._h, _dp(f)))

    def get_pin_flux_1g(self, g):
        out = np.empty(self.n_pin)
        _chk(self._lib.orc_get_pin_flux_1g(self._h, g, _dp(out)))
        return out

    def set_pin_flux_1g(self, g, pf):
        pf = np.ascontiguousarray(pf, dtype=np.float64)
        r = C.c_double()
        _chk(self._lib.orc_set_pin_flux_1g(self._h, g, _dp(pf), C.byref(r)))
        return r.value

    def pin_powers(self):
        out = np.empty(self.n_pin)
        _chk(self._lib.orc_pin_powers(self._h, _dp(out)))
        return out.reshape(self.ny, self.nx)

    def coarse_currents(self):
        cur = np.empty((self.n_group, self.n_surf))
        sfl = np.empty((self.n_group, self.n_surf))
        _chk(self._lib.orc_get_coarse_currents(self._h, _dp(cur), _dp(sfl)))
        return cur, sfl

    def update_incoming_flux(self, part, part_old=None, mode=1):
        """update_incoming_flux from given 2 (J+ + J-) per [G][n_surf]."""
        part = np.ascontiguousarray(part, dtype=np.float64)
        old = None if part_old is None else np.ascontiguousarray(part_old, dtype=np.float64)
        _chk(self._lib.orc_update_incoming(self._h, _dp(part), None if old is None else _dp(old),
                                           0 if old is None else 1, mode))

    def boundary_flux(self, g):
        """Incoming boundary angular flux of group g (MOCC's per-group layout)."""
        n = C.c_int64()
        _chk(self._lib.orc_get_boundary(self._h, g, None, C.byref(n)))
        out = np.empty(n.value)
        _chk(self._lib.orc_get_boundary(self._h, g, _dp(out), C.byref(n)))
        return out

    def homogenized_nu_fission(self):
        """Pin-homogenised nu-Sigma_f of the current flux, [n_pin (FSR order)][G]."""
        out = np.empty((self.n_pin, self.n_group))
        _chk(self._lib.orc_homogenized_nu_fission(self._h, out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

    def cmfd_system(self):
        """The unsolved CMFD system of the current state: op [G][5][n_cell]
        (diagonal, W, E, S, N), nu-Sigma_f and chi [n_cell][G], scattering
        [n_cell][G (to)][G (from)], cell volumes [n_cell]."""
        n, G = self.n_pin, self.n_group
        op, nf, ch = np.empty((G, 5, n)), np.empty((n, G)), np.empty((n, G))
        sc, vol = np.empty((n, G, G)), np.empty(n)
        dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
        _chk(self._lib.orc_cmfd_system(self._h, dp(op), dp(nf), dp(ch), dp(sc), dp(vol)))
        return {"op": op, "xsnf": nf, "xsch": ch, "scat": sc, "vol": vol}

    def cmfd_solve(self, k):
        kk = C.c_double(k)
        _chk(self._lib.orc_cmfd_solve(self._h, C.byref(kk)))
        return kk.value

    def solve(self, max_outer=-1):
        r = _R()
        _chk(self._lib.orc_eigen_solve(self._h, max_outer, C.byref(r)))
        return {f: getattr(r, f) for f, _ in _R._fields_}

    def apply_transverse_leakage(self, g, tl):
        tl = np.ascontiguousarray(tl, dtype=np.float64)
        _chk(self._lib.orc_apply_transverse_leakage(self._h, g, _dp(tl)))

    def history(self) -> np.ndarray:
        """The last solve's outer iterations, [n][4]: k, error_k, error_psi,
        seconds since the solve began."""
        d, n = C.POINTER(C.c_double)(), C.c_int64()
        _chk(self._lib.orc_history(self._h, C.byref(d), C.byref(n)))
        if n.value == 0:
            return np.zeros((0, 4))
        return np.ctypeslib.as_array(d, shape=(n.value, 4)).copy()

    def output(self) -> dict:
        """The datasets MOCC's EigenSolver::output writes after a solve (see
        mocc_output), from this solver's own trace."""
        if not hasattr(self, "_traced"):
            raise ValueError("output needs a solver built from input text (from_xml)")
        return mocc_output(self._traced, self)


def mocc_output(traced: Traced, solver: OracleSolver) -> dict:
    """Restatement of what MOCC writes to its HDF5 output after an eigenvalue
    solve, as {dataset path: array}:

    * ``EigenSolver::output`` (eigen_solver.cpp:293-322): convergence/k,
      error_k, error_psi per outer iteration, iteration_time and abscissae
      (both the iteration times);
    * ``FixedSourceSolver::output`` (fixed_source_solver.cpp:119-129): ng and
      eubounds (the library's group bounds);
    * ``MoCSweeper::output`` (moc_sweeper.cpp:533-585): flux/001.. of the pin
      flux (``get_pin_flux``), the whole [pin][group] array scaled by
      ``Normalize`` (utils.hpp:29-52: to sum to its count of positive
      entries), each group shaped (nz, ny, nx); pin_powers (nz, ny, nx);
    * ``AngularQuadrature::output`` (angular_quadrature.cpp:213-248):
      ang_quad/n_polar, n_azimuthal and every angle's alpha, theta,
      omega_x/y/z and weight."""
    h = solver.history()
    G, ny, nx = solver.n_group, solver.ny, solver.nx
    flux = np.stack([solver.get_pin_flux_1g(g) for g in range(G)], axis=1)  # [pin][g]
    n_pos = int(np.count_nonzero(flux > 0.0))
    flux = flux * (n_pos / flux.sum())
    out = {
        "convergence/k": h[:, 0].copy(), "convergence/error_k": h[:, 1].copy(),
        "convergence/error_psi": h[:, 2].copy(), "convergence/iteration_time": h[:, 3].copy(),
        "convergence/abscissae": h[:, 3].copy(),
        "ng": np.array(G, dtype=np.int32), "eubounds": traced.array("group_bounds"),
    }
    for g in range(G):
        out[f"flux/{g + 1:03d}"] = flux[:, g].reshape(1, ny, nx).copy()
    out["pin_powers"] = solver.pin_powers().reshape(1, ny, nx)
    npol, nazi = (int(v) for v in traced.array("quad_n"))
    out["ang_quad/n_polar"] = np.array(npol, dtype=np.int32)
    out["ang_quad/n_azimuthal"] = np.array(nazi, dtype=np.int32)
    for key, name in (("alpha", "quad_alpha"), ("theta", "quad_theta"), ("omega_x", "quad_ox"),
                      ("omega_y", "quad_oy"), ("omega_z", "quad_oz"), ("weight", "quad_weight")):
        out["ang_quad/" + key] = traced.array(name)
    return out
