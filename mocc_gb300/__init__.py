"""mocc_gb300: GB300 2-D Method-of-Characteristics sweep and CMFD power iteration.

Python mirror of MOCC's sweeper/solver interface over the library's C ABI
(``include/mocgpu.h``). The classes keep MOCC's names and argument meanings:

* :class:`Problem`    -- XML input processing, core mesh and ray tracing
  (``src/input_proc.cpp``, ``src/core/core_mesh.cpp``,
  ``src/sweepers/moc/ray_data.cpp``)
* :class:`MoCSweeper` -- ``mocc::moc::MoCSweeper`` / ``TransportSweeper``
  (``src/core/transport_sweeper.hpp:41-351``)
* :class:`EigenSolver` -- ``mocc::EigenSolver`` (``src/solvers/eigen_solver.cpp``)

Everything numeric runs in ``libmocgpu.so`` on the GPU; there is no CPU
fallback, and constructing a sweeper without a CUDA device raises
:class:`MocgpuError`. Errors that MOCC reports with ``EXCEPT`` surface as
:class:`MocgpuError` carrying the C status code.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

__all__ = ["MocgpuError", "Problem", "MoCSweeper", "EigenSolver", "BatchEngine", "synthetic_xsl", "load_library",
           "SIZES"]

_LIB = None

SIZES = ["ngroup", "nfsr", "nmat", "ndir_oct", "nang", "nsets", "pol_per_set", "nx", "ny", "npin",
         "nsurf", "nfuel", "ntracks", "nseg", "ncm", "maxseg"]


class MocgpuError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[mocgpu {code}] {msg}")
        self.code = code


class _Options(C.Structure):
    _fields_ = [("k_tol", C.c_double), ("psi_tol", C.c_double), ("max_iter", C.c_int), ("min_iter", C.c_int),
                ("cmfd", C.c_int), ("cmfd_enabled", C.c_int), ("cmfd_k_tol", C.c_double),
                ("cmfd_psi_tol", C.c_double), ("cmfd_resid_reduction", C.c_double), ("cmfd_max_iter", C.c_int),
                ("cmfd_negative_fixup", C.c_int), ("n_inner", C.c_int), ("gs_boundary", C.c_int),
                ("precision", C.c_int), ("sweep_kernel", C.c_int), ("bundles_per_unit", C.c_int),
                ("window_rows", C.c_int), ("incoming_update", C.c_int), ("tl_splitting", C.c_int),
                ("dump_fsr_flux", C.c_int)]


class _Result(C.Structure):
    _fields_ = [("k", C.c_double), ("iterations", C.c_int), ("converged", C.c_int), ("error_k", C.c_double),
                ("error_psi", C.c_double), ("seconds", C.c_double), ("sweeps", C.c_int64),
                ("cmfd_iterations", C.c_int64)]


class _BatchResult(C.Structure):
    _fields_ = [("id", C.c_int64), ("error", C.c_int), ("message", C.c_char * 128), ("k", C.c_double),
                ("iterations", C.c_int), ("converged", C.c_int), ("error_k", C.c_double),
                ("error_psi", C.c_double), ("cmfd_iterations", C.c_int64), ("t_submit", C.c_double),
                ("t_admit", C.c_double), ("t_done", C.c_double), ("n_pin", C.c_int)]


class _BatchStats(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("completed", C.c_int64), ("outer_iterations", C.c_int64),
                ("graph_replays", C.c_int64), ("captures", C.c_int64), ("active", C.c_int), ("queued", C.c_int),
                ("capacity", C.c_int), ("geometries", C.c_int), ("bundles_per_unit", C.c_int),
                ("bytes_in_use", C.c_double), ("bytes_budget", C.c_double), ("geometry_bytes", C.c_double),
                ("now", C.c_double), ("replay_ms", C.c_double), ("sweep_ms", C.c_double),
                ("sweep_launches", C.c_int64), ("sweep_bytes", C.c_double), ("sweep_sgu", C.c_int64),
                ("trace_hits", C.c_int64), ("trace_misses", C.c_int64), ("trace_ms", C.c_double),
                ("xs_ms", C.c_double)]


def library_path() -> Path:
    return Path(__file__).resolve().parent / "_build" / "libmocgpu.so"


def load_library(build: bool = True):
    """Loads libmocgpu.so (building it in-tree first when ``build``)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if build:
        from . import _build
        path = _build.build_library()
    if not path.exists():
        raise MocgpuError(99, f"libmocgpu.so not built at {path}")
    lib = C.CDLL(str(path))
    P, I, D, VP, CP = C.c_void_p, C.c_int, C.c_double, C.c_void_p, C.c_char_p
    DP, IP, I64P = C.POINTER(C.c_double), C.POINTER(C.c_int), C.POINTER(C.c_int64)
    sig = {
        "mocgpu_last_error": (CP, []),
        "mocgpu_version": (I, []),
        "mocgpu_device_count": (I, [IP]),
        "mocgpu_problem_create": (I, [CP, CP, CP, C.POINTER(P)]),
        "mocgpu_problem_destroy": (None, [P]),
        "mocgpu_problem_sizes": (I, [P, I64P]),
        "mocgpu_problem_quadrature": (I, [P, IP, IP, DP, C.c_int64, I64P]),
        "mocgpu_problem_group_bounds": (I, [P, DP, I, IP]),
        "mocgpu_eigen_history": (I, [P, DP, C.c_int64, I64P]),
        "mocgpu_apply_transverse_leakage": (I, [P, I, DP]),
        "mocgpu_problem_options": (I, [P, C.POINTER(_Options)]),
        "mocgpu_problem_set_options": (I, [P, C.POINTER(_Options)]),
        "mocgpu_problem_export": (I, [P, CP, VP, C.c_int64]),
        "mocgpu_problem_field_bytes": (I, [P, CP, I64P]),
        "mocgpu_synthetic_xsl": (I, [C.c_uint64, I, I, DP, D, D, C.c_char_p, C.c_int64, I64P]),
        "mocgpu_trace_ray": (I, [CP, CP, D, D, D, D, IP, DP, IP, I, IP, IP, IP, I]),
        "mocgpu_sweeper_create": (I, [P, I, C.POINTER(P)]),
        "mocgpu_sweeper_create_xsl": (I, [P, I, CP, C.POINTER(P)]),
        "mocgpu_sweeper_destroy": (None, [P]),
        "mocgpu_sweeper_set_options": (I, [P, C.POINTER(_Options)]),
        "mocgpu_initialize": (I, [P]),
        "mocgpu_calc_fission_source": (I, [P, D, DP]),
        "mocgpu_set_fission_source": (I, [P, DP]),
        "mocgpu_store_old_flux": (I, [P]),
        "mocgpu_source_group": (I, [P, I]),
        "mocgpu_sweep_group": (I, [P, I]),
        "mocgpu_set_coarse_data": (I, [P, I]),
        "mocgpu_total_fission": (I, [P, I, DP]),
        "mocgpu_flux_residual": (I, [P, DP]),
        "mocgpu_get_flux": (I, [P, DP]),
        "mocgpu_set_flux": (I, [P, DP]),
        "mocgpu_get_pin_flux_1g": (I, [P, I, DP]),
        "mocgpu_get_boundary_flux": (I, [P, I, DP, C.c_int64, C.POINTER(C.c_int64)]),
        "mocgpu_update_incoming_flux": (I, [P, DP, DP, I, I]),
        "mocgpu_sweeper_layout": (I, [P, IP, IP, IP, IP]),
        "mocgpu_set_pin_flux_1g": (I, [P, I, DP, DP]),
        "mocgpu_pin_powers": (I, [P, DP]),
        "mocgpu_get_coarse_currents": (I, [P, DP, DP]),
        "mocgpu_homogenized_xs": (I, [P, DP, DP, DP, DP, DP, DP]),
        "mocgpu_cmfd_solve": (I, [P, DP]),
        "mocgpu_eigen_solve": (I, [P, I, C.POINTER(_Result)]),
        "mocgpu_sweeper_bytes": (I, [P, I64P, DP]),
        "mocgpu_sweeper_stream": (I, [P, C.POINTER(C.c_void_p)]),
        "mocgpu_time_sweep": (I, [P, I, I, DP, IP]),
        "mocgpu_launch_count": (I, [I64P]),
        "mocgpu_layout_stats": (I, [P, I, I, I, I, I64P, DP]),
        "mocgpu_batch_create": (I, [I, I, D, I, C.POINTER(P)]),
        "mocgpu_batch_destroy": (None, [P]),
        "mocgpu_batch_submit": (I, [P, P, CP, I64P]),
        "mocgpu_batch_submit_xml": (I, [P, CP, CP, CP, I64P]),
        "mocgpu_batch_step": (I, [P, IP]),
        "mocgpu_batch_run": (I, [P]),
        "mocgpu_batch_launch": (I, [P, IP]),
        "mocgpu_batch_finish": (I, [P, IP]),
        "mocgpu_batch_poll": (I, [P, IP]),
        "mocgpu_batch_set_pipeline_depth": (I, [P, I]),
        "mocgpu_batch_set_sweep_shape": (I, [P, I]),
        "mocgpu_sweep_shape_info": (I, [I, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
        "mocgpu_batch_cancel": (I, [P, C.c_int64, IP]),
        "mocgpu_debug_fail_allocations": (I, [C.c_int64]),
        "mocgpu_batch_in_flight": (I, [P, IP]),
        "mocgpu_batch_take": (I, [P, C.c_int64, IP, C.POINTER(_BatchResult), DP, I]),
        "mocgpu_batch_get_stats": (I, [P, C.POINTER(_BatchStats)]),
        "mocgpu_batch_ready": (I, [P, I64P, I, IP]),
        "mocgpu_batch_stream": (I, [P, C.POINTER(C.c_void_p)]),
        "mocgpu_batch_set_timing": (I, [P, I]),
        "mocgpu_copy_bytes": (I, [I64P, I64P]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def _check(rc: int):
    if rc != 0:
        raise MocgpuError(rc, _LIB.mocgpu_last_error().decode())


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def synthetic_xsl(seed: int, n_group: int = 7, n_fuel: int = 1, fuel_nf_scale=None, mod_factor: float = 1.0,
                  fuel_nf_factor: float = 1.0) -> str:
    """Seeded synthetic .xsl library (materials fuel1..fuelN, moderator)."""
    lib = load_library()
    sc = None
    if fuel_nf_scale is not None:
        sc_arr = np.ascontiguousarray(fuel_nf_scale, dtype=np.float64)
        assert sc_arr.size == n_fuel
        sc = _dp(sc_arr)
    need = C.c_int64(0)
    _check(lib.mocgpu_synthetic_xsl(seed, n_group, n_fuel, sc, mod_factor, fuel_nf_factor, None, 0, C.byref(need)))
    buf = C.create_string_buffer(need.value)
    _check(lib.mocgpu_synthetic_xsl(seed, n_group, n_fuel, sc, mod_factor, fuel_nf_factor, buf, need.value,
                                    C.byref(need)))
    return buf.value.decode()


class Problem:
    """A traced 2-D problem from MOCC XML input (host side only)."""

    INT_FIELDS = {"fsr_mat", "set_nx", "set_ny", "set_first_track", "trk_bc0", "trk_bc1", "trk_set",
                  "trk_cm_cell_fw", "trk_cm_cell_bw", "trk_cm_surf_fw", "trk_cm_surf_bw", "trk_cm_begin",
                  "cm_fw", "cm_bw", "cm_nseg_fw", "cm_nseg_bw", "seg_fsr", "pin_first_reg", "pin_cell",
                  "pin_fuel", "bc"}
    I64_FIELDS = {"trk_seg_begin"}

    def __init__(self, xml: str, xsl: str | None = None, base_dir: str | None = None):
        lib = load_library()
        h = C.c_void_p()
        _check(lib.mocgpu_problem_create(xml.encode(), xsl.encode() if xsl else None,
                                         base_dir.encode() if base_dir else None, C.byref(h)))
        self._h = h
        self._lib = lib
        arr = (C.c_int64 * len(SIZES))()
        _check(lib.mocgpu_problem_sizes(h, arr))
        self.sizes = dict(zip(SIZES, list(arr)))

    @classmethod
    def from_file(cls, path: str, xsl: str | None = None):
        p = Path(path)
        return cls(p.read_text(), xsl, str(p.parent))

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.mocgpu_problem_destroy(self._h)
            self._h = None

    @property
    def handle(self):
        return self._h

    def quadrature(self) -> dict:
        """The traced (modularised) angular quadrature: n_polar and
        n_azimuthal per octant, and alpha, theta, omega_x/y/z and weight of
        every angle of all 8 octants (what AngularQuadrature::output writes)."""
        npol, nazi, nd = C.c_int(), C.c_int(), C.c_int64()
        _check(self._lib.mocgpu_problem_quadrature(self._h, C.byref(npol), C.byref(nazi), None, 0, C.byref(nd)))
        a = np.empty((nd.value, 6))
        _check(self._lib.mocgpu_problem_quadrature(self._h, C.byref(npol), C.byref(nazi), _dp(a), nd.value,
                                                   C.byref(nd)))
        out = {"n_polar": npol.value, "n_azimuthal": nazi.value}
        for j, key in enumerate(("alpha", "theta", "omega_x", "omega_y", "omega_z", "weight")):
            out[key] = a[:, j].copy()
        return out

    def group_bounds(self) -> np.ndarray:
        """Upper energy bounds of the cross-section library's groups."""
        n = C.c_int()
        _check(self._lib.mocgpu_problem_group_bounds(self._h, None, 0, C.byref(n)))
        out = np.empty(n.value)
        _check(self._lib.mocgpu_problem_group_bounds(self._h, _dp(out), n.value, C.byref(n)))
        return out

    def export(self, field: str) -> np.ndarray:
        n = C.c_int64(0)
        _check(self._lib.mocgpu_problem_field_bytes(self._h, field.encode(), C.byref(n)))
        dt = np.int32 if field in self.INT_FIELDS else np.int64 if field in self.I64_FIELDS else np.float64
        out = np.empty(n.value // np.dtype(dt).itemsize, dtype=dt)
        _check(self._lib.mocgpu_problem_export(self._h, field.encode(), out.ctypes.data_as(C.c_void_p), n.value))
        return out

    def layout_stats(self, gs: bool = True, tracks_per_unit: int = 64, max_local: int = 16384,
                     window_rows: int = 0) -> dict:
        """Host-side build of the GPU sweep's bundled layout, with checks."""
        st = (C.c_int64 * 8)()
        sd = (C.c_double * 2)()
        _check(self._lib.mocgpu_layout_stats(self._h, 1 if gs else 0, tracks_per_unit, max_local, window_rows, st,
                                             sd))
        keys = ["units", "bundles", "rows", "real_segments", "max_local", "phases", "max_windows", "windows"]
        d = dict(zip(keys, list(st)))
        d["len_sum"], d["padding"] = sd[0], sd[1]
        return d

    @property
    def options(self) -> dict:
        o = _Options()
        _check(self._lib.mocgpu_problem_options(self._h, C.byref(o)))
        return {f: getattr(o, f) for f, _ in _Options._fields_}

    def set_options(self, **kw):
        o = _Options()
        _check(self._lib.mocgpu_problem_options(self._h, C.byref(o)))
        for k, v in kw.items():
            if k not in dict(_Options._fields_):
                raise KeyError(k)
            setattr(o, k, v)
        _check(self._lib.mocgpu_problem_set_options(self._h, C.byref(o)))


def trace_ray(xml: str, xsl: str, p1, p2, cap: int = 4096):
    """MOCC's Ray(p1, p2, bc, 0, mesh) on the geometry in ``xml``."""
    lib = load_library()
    nseg, ncm = C.c_int(0), C.c_int(0)
    L = np.zeros(cap)
    F = np.zeros(cap, dtype=np.int32)
    co = np.zeros(4, dtype=np.int32)
    cm = np.zeros(4 * cap, dtype=np.int32)
    ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int))
    _check(lib.mocgpu_trace_ray(xml.encode(), xsl.encode() if xsl else None, p1[0], p1[1], p2[0], p2[1],
                                C.byref(nseg), _dp(L), ip(F), cap, ip(co), C.byref(ncm), ip(cm), cap))
    n, m = nseg.value, ncm.value
    return {"seg_len": L[:n].copy(), "seg_fsr": F[:n].copy(), "cm_cell_fw": int(co[0]), "cm_cell_bw": int(co[1]),
            "cm_surf_fw": int(co[2]), "cm_surf_bw": int(co[3]), "cm": cm[:4 * m].reshape(m, 4).copy()}


class MoCSweeper:
    """Device-resident MoC sweeper (MOCC's MoCSweeper API).

    ``precision``: 0 = FP64 sweep, 1 = FP32 sweep with FP64 reductions and
    CMFD, -1 = the ``<sweeper precision>`` of the input. ``xsl``: another
    cross-section library for the problem's materials (the traced geometry
    is reused).
    """

    def __init__(self, problem: Problem, precision: int = -1, xsl: str | None = None):
        self.problem = problem
        self._lib = load_library()
        h = C.c_void_p()
        if xsl:
            _check(self._lib.mocgpu_sweeper_create_xsl(problem.handle, precision, xsl.encode(), C.byref(h)))
        else:
            _check(self._lib.mocgpu_sweeper_create(problem.handle, precision, C.byref(h)))
        self._h = h
        s = problem.sizes
        self.n_group, self.n_reg, self.n_pin = s["ngroup"], s["nfsr"], s["npin"]
        self.nx, self.ny, self.n_surf = s["nx"], s["ny"], s["nsurf"]

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.mocgpu_sweeper_destroy(self._h)
            self._h = None

    def close(self):
        self.__del__()

    @property
    def handle(self):
        return self._h

    def set_options(self, **kw):
        o = _Options()
        _check(self._lib.mocgpu_problem_options(self.problem.handle, C.byref(o)))
        for k, v in kw.items():
            setattr(o, k, v)
        _check(self._lib.mocgpu_sweeper_set_options(self._h, C.byref(o)))

    def initialize(self):
        _check(self._lib.mocgpu_initialize(self._h))

    def set_coarse_data(self, enabled: bool = True):
        _check(self._lib.mocgpu_set_coarse_data(self._h, 1 if enabled else 0))

    def calc_fission_source(self, k: float) -> np.ndarray:
        fs = np.empty(self.n_reg)
        _check(self._lib.mocgpu_calc_fission_source(self._h, k, _dp(fs)))
        return fs

    def set_fission_source(self, fs: np.ndarray):
        fs = np.ascontiguousarray(fs, dtype=np.float64)
        _check(self._lib.mocgpu_set_fission_source(self._h, _dp(fs)))

    def store_old_flux(self):
        _check(self._lib.mocgpu_store_old_flux(self._h))

    def source_group(self, g: int):
        _check(self._lib.mocgpu_source_group(self._h, g))

    def sweep(self, g: int):
        _check(self._lib.mocgpu_sweep_group(self._h, g))

    def total_fission(self, old: bool = False) -> float:
        v = C.c_double()
        _check(self._lib.mocgpu_total_fission(self._h, 1 if old else 0, C.byref(v)))
        return v.value

    def flux_residual(self) -> float:
        v = C.c_double()
        _check(self._lib.mocgpu_flux_residual(self._h, C.byref(v)))
        return v.value

    def flux(self) -> np.ndarray:
        f = np.empty((self.n_reg, self.n_group))
        _check(self._lib.mocgpu_get_flux(self._h, _dp(f)))
        return f

    def set_flux(self, f: np.ndarray):
        f = np.ascontiguousarray(f, dtype=np.float64).reshape(self.n_reg, self.n_group)
        _check(self._lib.mocgpu_set_flux(self._h, _dp(f)))

    def update_incoming_flux(self, part: np.ndarray, part_old: np.ndarray | None = None, mode: int = 1):
        """MoCSweeper::update_incoming_flux from given 2 (J+ + J-) per [G][n_surf]
        (part_old: the previous CMFD solve's, None on the first)."""
        part = np.ascontiguousarray(part, dtype=np.float64)
        old = None if part_old is None else np.ascontiguousarray(part_old, dtype=np.float64)
        _check(self._lib.mocgpu_update_incoming_flux(self._h, _dp(part), None if old is None else _dp(old),
                                                     0 if old is None else 1, mode))

    def apply_transverse_leakage(self, g: int, tl: np.ndarray):
        """MoCSweeper::apply_transverse_leakage: adds tl [n_fsr] to group g's
        source (after source_group(g)), split into Sigma_t where negative
        when the tl_splitting option is on."""
        tl = np.ascontiguousarray(tl, dtype=np.float64).reshape(self.n_reg)
        _check(self._lib.mocgpu_apply_transverse_leakage(self._h, g, _dp(tl)))

    def layout(self) -> dict:
        """Bundled sweep layout of this handle's geometry."""
        v = [C.c_int() for _ in range(4)]
        _check(self._lib.mocgpu_sweeper_layout(self._h, *[C.byref(x) for x in v]))
        return dict(zip(("units", "tracks_per_unit", "window_rows", "table_slots"), (x.value for x in v)))

    def boundary_flux(self, g: int) -> np.ndarray:
        """Incoming boundary angular flux of group g (MOCC's per-group layout)."""
        n = C.c_int64()
        _check(self._lib.mocgpu_get_boundary_flux(self._h, g, None, 0, C.byref(n)))
        out = np.empty(n.value)
        _check(self._lib.mocgpu_get_boundary_flux(self._h, g, _dp(out), n.value, C.byref(n)))
        return out

    def get_pin_flux_1g(self, g: int) -> np.ndarray:
        out = np.empty(self.n_pin)
        _check(self._lib.mocgpu_get_pin_flux_1g(self._h, g, _dp(out)))
        return out

    def set_pin_flux_1g(self, g: int, pf: np.ndarray) -> float:
        pf = np.ascontiguousarray(pf, dtype=np.float64)
        r = C.c_double()
        _check(self._lib.mocgpu_set_pin_flux_1g(self._h, g, _dp(pf), C.byref(r)))
        return r.value

    def pin_powers(self) -> np.ndarray:
        out = np.empty(self.n_pin)
        _check(self._lib.mocgpu_pin_powers(self._h, _dp(out)))
        return out.reshape(self.ny, self.nx)

    def coarse_currents(self):
        cur = np.empty((self.n_group, self.n_surf))
        sfl = np.empty((self.n_group, self.n_surf))
        _check(self._lib.mocgpu_get_coarse_currents(self._h, _dp(cur), _dp(sfl)))
        return cur, sfl

    def homogenized_xs(self) -> dict:
        """Pin-homogenised cross sections of the current flux (MOCC's
        get_homogenized_xsmesh): xstr, xsnf, xsf, xsch, xsrm [n_pin][G] and
        scat [n_pin][G (to)][G (from)], pins in coarse-cell order."""
        shp = (self.n_pin, self.n_group)
        out = {k: np.empty(shp) for k in ("xstr", "xsnf", "xsf", "xsch", "xsrm")}
        out["scat"] = np.empty(shp + (self.n_group,))
        _check(self._lib.mocgpu_homogenized_xs(self._h, *(_dp(out[k]) for k in
                                                          ("xstr", "xsnf", "xsf", "xsch", "xsrm", "scat"))))
        return out

    def cmfd_solve(self, k: float) -> float:
        kk = C.c_double(k)
        _check(self._lib.mocgpu_cmfd_solve(self._h, C.byref(kk)))
        return kk.value

    def bytes(self):
        db, sb = C.c_int64(), C.c_double()
        _check(self._lib.mocgpu_sweeper_bytes(self._h, C.byref(db), C.byref(sb)))
        return db.value, sb.value

    def stream(self) -> int:
        p = C.c_void_p()
        _check(self._lib.mocgpu_sweeper_stream(self._h, C.byref(p)))
        return p.value or 0

    def time_sweep(self, g: int, reps: int):
        """(summed ms of the sweep kernels, number of sweep launches)."""
        ms, nl = C.c_double(), C.c_int()
        _check(self._lib.mocgpu_time_sweep(self._h, g, reps, C.byref(ms), C.byref(nl)))
        return ms.value, nl.value


def copy_bytes() -> tuple[int, int]:
    """(host->device, device->host) bytes the library has copied so far."""
    h, d = C.c_int64(), C.c_int64()
    _check(load_library().mocgpu_copy_bytes(C.byref(h), C.byref(d)))
    return h.value, d.value


def fail_allocations_after(n: int):
    """Test hook: after n more device allocations the next fails as out of
    memory (once); a negative n switches it off."""
    _check(load_library().mocgpu_debug_fail_allocations(n))


def sweep_shapes() -> list:
    """(rows per chunk, chunks in flight) of every built batched-sweep shape."""
    lib, out = load_library(), []
    r, s = C.c_int(), C.c_int()
    i = 0
    while lib.mocgpu_sweep_shape_info(i, C.byref(r), C.byref(s)) == 0:
        out.append((r.value, s.value))
        i += 1
    return out


def launch_count() -> int:
    n = C.c_int64()
    _check(load_library().mocgpu_launch_count(C.byref(n)))
    return n.value


class EigenSolver:
    """k-eigenvalue power iteration with optional CMFD (MOCC's EigenSolver)."""

    def __init__(self, problem: Problem, precision: int = -1, sweeper: MoCSweeper | None = None):
        self.problem = problem
        self.sweeper = sweeper or MoCSweeper(problem, precision)

    def solve(self, max_outer: int = -1) -> dict:
        r = _Result()
        _check(self.sweeper._lib.mocgpu_eigen_solve(self.sweeper.handle, max_outer, C.byref(r)))
        return {f: getattr(r, f) for f, _ in _Result._fields_}

    def pin_powers(self) -> np.ndarray:
        return self.sweeper.pin_powers()

    def history(self) -> np.ndarray:
        """The last solve's outer iterations, [n][4]: k, error_k, error_psi,
        seconds since the solve began."""
        lib, h, n = self.sweeper._lib, self.sweeper.handle, C.c_int64()
        _check(lib.mocgpu_eigen_history(h, None, 0, C.byref(n)))
        out = np.empty((n.value, 4))
        _check(lib.mocgpu_eigen_history(h, _dp(out), n.value, C.byref(n)))
        return out

    def output(self, dump_fsr_flux: bool | None = None) -> dict:
        """The datasets MOCC's EigenSolver::output writes after this solve,
        {HDF5 path: array} (``mocc_gb300.output``); fsr_flux/NNN when
        ``dump_fsr_flux``, by default when the input's <sweeper
        dump_fsr_flux> asks for it."""
        if dump_fsr_flux is None:
            dump_fsr_flux = bool(self.problem.options["dump_fsr_flux"])
        from .output import eigen_output
        return eigen_output(self, dump_fsr_flux=dump_fsr_flux)


class BatchEngine:
    """Many independent k-eigenvalue solves advanced together on one GPU.

    Each submitted solve runs MOCC's EigenSolver power iteration
    (``src/solvers/eigen_solver.cpp:131-253``) with its own k, sources and
    convergence test; every active solve advances one outer iteration per
    replay of one captured CUDA graph. Converged solves retire between
    iterations and queued solves take their slots. ``submit(problem, xsl)``
    reuses ``problem``'s traced geometry with the cross sections of ``xsl``.
    """

    def __init__(self, precision: int = 1, capacity: int = 64, mem_budget: float = 0.0,
                 bundles_per_unit: int = 1):
        self._lib = load_library()
        h = C.c_void_p()
        _check(self._lib.mocgpu_batch_create(precision, capacity, float(mem_budget), bundles_per_unit,
                                             C.byref(h)))
        self._h = h
        self._keep = {}
        self.depth = 2
        self.sweep_shape = 0

    def close(self):
        if getattr(self, "_h", None):
            self._lib.mocgpu_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def submit(self, problem: Problem, xsl: str | None = None) -> int:
        i = C.c_int64()
        _check(self._lib.mocgpu_batch_submit(self._h, problem.handle, xsl.encode() if xsl else None, C.byref(i)))
        return i.value

    def submit_xml(self, xml: str, xsl: str | None = None, base_dir: str = "") -> int:
        """Queues a solve given as MOCC input text; requests with the same XML
        share one traced problem (only their cross sections are read)."""
        i = C.c_int64()
        _check(self._lib.mocgpu_batch_submit_xml(self._h, xml.encode(), xsl.encode() if xsl else None,
                                                 base_dir.encode(), C.byref(i)))
        return i.value

    def step(self) -> int:
        n = C.c_int()
        _check(self._lib.mocgpu_batch_step(self._h, C.byref(n)))
        return n.value

    def run(self):
        _check(self._lib.mocgpu_batch_run(self._h))

    def set_pipeline_depth(self, depth: int):
        """Outer iterations launch() may have in flight (1..4, default 2)."""
        _check(self._lib.mocgpu_batch_set_pipeline_depth(self._h, depth))
        self.depth = depth

    def set_sweep_shape(self, shape: int):
        """Streaming shape of the batched sweep (index into sweep_shapes())."""
        _check(self._lib.mocgpu_batch_set_sweep_shape(self._h, shape))
        self.sweep_shape = shape

    def in_flight(self) -> int:
        n = C.c_int()
        _check(self._lib.mocgpu_batch_in_flight(self._h, C.byref(n)))
        return n.value

    def launch(self) -> int:
        """Enqueues one outer iteration of every active solve; returns at once."""
        n = C.c_int()
        _check(self._lib.mocgpu_batch_launch(self._h, C.byref(n)))
        return n.value

    def poll(self) -> bool:
        """True when finish() would not block."""
        d = C.c_int()
        _check(self._lib.mocgpu_batch_poll(self._h, C.byref(d)))
        return bool(d.value)

    def finish(self) -> int:
        """Waits for the oldest launched iteration and retires the solves it ended."""
        n = C.c_int()
        _check(self._lib.mocgpu_batch_finish(self._h, C.byref(n)))
        return n.value

    def cancel(self, solve_id: int) -> bool:
        """Cancels a queued or active solve; its result reports error 14."""
        f = C.c_int()
        _check(self._lib.mocgpu_batch_cancel(self._h, solve_id, C.byref(f)))
        return bool(f.value)

    def take(self, solve_id: int, n_pin_max: int = 1 << 16):
        """Result dict of a finished solve (None while it runs)."""
        r = _BatchResult()
        ready = C.c_int()
        pins = np.zeros(n_pin_max)
        _check(self._lib.mocgpu_batch_take(self._h, solve_id, C.byref(ready), C.byref(r), _dp(pins), n_pin_max))
        if not ready.value:
            return None
        out = {f: getattr(r, f) for f, _ in _BatchResult._fields_ if f != "message"}
        out["message"] = r.message.decode()
        out["pin_powers"] = pins[:r.n_pin].copy()
        return out

    def ready(self) -> list[int]:
        """Ids of finished solves whose results have not been taken."""
        n = C.c_int()
        _check(self._lib.mocgpu_batch_ready(self._h, None, 0, C.byref(n)))
        if n.value == 0:
            return []
        ids = np.zeros(n.value, dtype=np.int64)
        _check(self._lib.mocgpu_batch_ready(self._h, ids.ctypes.data_as(C.POINTER(C.c_int64)), n.value,
                                            C.byref(n)))
        return [int(i) for i in ids[:n.value]]

    def stats(self) -> dict:
        st = _BatchStats()
        _check(self._lib.mocgpu_batch_get_stats(self._h, C.byref(st)))
        return {f: getattr(st, f) for f, _ in _BatchStats._fields_}

    def stream(self) -> int:
        p = C.c_void_p()
        _check(self._lib.mocgpu_batch_stream(self._h, C.byref(p)))
        return p.value or 0

    def set_timing(self, on: bool = True):
        _check(self._lib.mocgpu_batch_set_timing(self._h, 1 if on else 0))
