"""Synthetic benchmark workloads written as MOCC XML input.

Every workload uses the same pin mesh: a 1.26 cm pitch cylindrical cell with
a 0.54 cm fuel radius split into 2 equal-area rings, the moderator annulus
outside, and 8 azimuthal sectors (24 flat-source regions per pin). Guide-tube
and reflector cells use the same mesh with moderator in every ring. Cross
sections come from the seeded synthetic library (``synthetic_xsl``).

Workloads (sizes as in the benchmark definitions):
  ``pin3x3``      3x3 fuel pins, reflective, 8 azimuths/octant, 3 polar,
                  0.05 cm spacing, FP64, CMFD
  ``assembly17``  17x17 assembly (264 fuel + 25 guide-tube cells), 16
                  azimuths/octant, 3 polar, 0.03 cm spacing
  ``minicore``    3x3 assemblies of 3 fuel compositions (nu-fission scaled
                  1.0/1.15/1.3) plus a 21.42 cm moderator row on the north and
                  east sides (vacuum there, reflective south and west)
  ``branch``      one lattice of 1x1, 3x3, 7x7 or 17x17 pins with seeded
                  moderator and fuel perturbations, 8 azimuths/octant, 0.05 cm
"""
from __future__ import annotations

import math
import random

_M64 = (1 << 64) - 1


class _SplitMix64:
    """splitmix64 stream: raw 64-bit draws identical on every host."""

    def __init__(self, seed: int):
        self.s = (seed * 0x9E3779B97F4A7C15 + 0x632BE59BD9B4E019) & _M64

    def next(self) -> int:
        self.s = (self.s + 0x9E3779B97F4A7C15) & _M64
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _M64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _M64
        return z ^ (z >> 31)

    def uniform(self, a: float = 0.0, b: float = 1.0) -> float:
        u = float(self.next() >> 11) * (1.0 / 9007199254740992.0)
        return a + (b - a) * u

    def log_uniform(self, a: float, b: float) -> float:
        return math.exp(self.uniform(math.log(a), math.log(b)))


def _material(rng, ng: int, fuel: bool):
    """Sigma_a, nu-Sigma_f, Sigma_f, chi and the [to][from] scattering matrix
    of one synthetic material: Sigma_t log-uniform in [0.2, 2.0]; the
    out-scatter of each group a fraction U[0.4, 0.95] of Sigma_t, split into
    self-scatter, downscatter to the next two groups and a small upscatter
    into the last groups only; fuel nu-Sigma_f U[0.005, 0.5] (Sigma_f =
    nu-Sigma_f / 2.43) and chi in the first groups."""
    n_chi = max(3, int(math.floor(3.0 * ng / 7.0 + 0.5)))
    n_up = max(2, int(math.floor(2.0 * ng / 7.0 + 0.5)))
    nu = 2.43
    ab, nf, sf, ch = [0.0] * ng, [0.0] * ng, [0.0] * ng, [0.0] * ng
    sc = [[0.0] * ng for _ in range(ng)]
    for f in range(ng):
        st = rng.log_uniform(0.2, 2.0)
        c = rng.uniform(0.4, 0.95)
        w = [0.0] * ng
        w[f] = rng.uniform(0.4, 0.8)
        for k in (1, 2):
            if f + k < ng:
                w[f + k] = rng.uniform(0.05, 0.4) / k
        if f > 0 and f - 1 >= ng - n_up:
            w[f - 1] = rng.uniform(0.01, 0.05)
        wsum = 0.0
        for v in w:
            wsum += v
        for to in range(ng):
            sc[to][f] = c * st * w[to] / wsum
        ab[f] = st * (1.0 - c)
        if fuel:
            nf[f] = rng.uniform(0.005, 0.5)
            sf[f] = nf[f] / nu
            if f < n_chi:
                ch[f] = rng.uniform(0.1, 1.0)
    return ab, nf, sf, ch, sc


def synthetic_xsl(seed: int, n_group: int = 7, n_fuel: int = 1, fuel_nf_scale=None, mod_factor: float = 1.0,
                  fuel_nf_factor: float = 1.0) -> str:
    """Seeded synthetic .xsl library in MOCC's format: materials fuel1..fuelN
    (one base fuel, nu-Sigma_f and Sigma_f scaled by ``fuel_nf_scale[i] *
    fuel_nf_factor``) and a moderator (absorption and scattering scaled by
    ``mod_factor``). Pure Python, so that a CPU-only run can make the same
    inputs without the GPU library (same text as ``mocgpu_synthetic_xsl``)."""
    if n_group < 3:
        raise ValueError("synthetic library needs at least 3 groups")
    rng = _SplitMix64(seed)
    ab, nf, sf, ch, sc = _material(rng, n_group, True)
    mats = []
    for i in range(n_fuel):
        k = (fuel_nf_scale[i] if fuel_nf_scale is not None and i < len(fuel_nf_scale) else 1.0)
        mats.append((f"fuel{i + 1}", ab, [v * (k * fuel_nf_factor) for v in nf], [v * (k * fuel_nf_factor) for v in sf],
                     ch, sc))
    mab, mnf, msf, mch, msc = _material(rng, n_group, False)
    mats.append(("moderator", [v * mod_factor for v in mab], mnf, msf, mch,
                 [[v * mod_factor for v in row] for row in msc]))
    out = ["Synthetic macroscopic cross sections\n", f" {n_group} {len(mats)}\n"]
    out.append("".join(" %.6e" % (2.0e7 * math.pow(1.0e-8, g / n_group)) for g in range(n_group)) + "\n")
    for name, a, b, c, d, s in mats:
        out.append(f"XSMACRO {name} 0\n")
        for g in range(n_group):
            out.append(" %.17e %.17e %.17e %.17e\n" % (a[g], b[g], c[g], d[g]))
        for to in range(n_group):
            out.append("".join(" %.17e" % s[to][f] for f in range(n_group)) + "\n")
    return "".join(out)

PITCH = 1.26

# Guide-tube positions of a 17x17 lattice (row, col), 24 tubes + centre.
_GT17 = {(2, 5), (2, 8), (2, 11), (3, 3), (3, 13), (5, 2), (5, 5), (5, 8), (5, 11), (5, 14), (8, 2), (8, 5),
         (8, 8), (8, 11), (8, 14), (11, 2), (11, 5), (11, 8), (11, 11), (11, 14), (13, 3), (13, 13), (14, 5),
         (14, 8), (14, 11)}


def lattice_rows(n: int, fuel_pin: int = 1, gt_pin: int = 10):
    """Rows (top row first, as MOCC's <lattice> lists them) of an n x n lattice."""
    rows = []
    for r in range(n):
        row = []
        for c in range(n):
            gt = (n == 17 and (r, c) in _GT17) or (n == 7 and r == 3 and c == 3)
            row.append(gt_pin if gt else fuel_pin)
        rows.append(row)
    return rows


def _mesh_xml():
    return ('<mesh id="1" type="cyl" pitch="1.26">\n  <radii>0.54</radii>\n  <sub_radii>2</sub_radii>\n'
            '  <sub_azi>8</sub_azi>\n</mesh>\n')


def _solver_xml(n_azi, spacing, precision, n_inner=5, k_tol=1e-6, psi_tol=1e-5, max_iter=200, cmfd=True,
                resid_reduction=None, boundary_update="gs"):
    rr = f' residual_reduction="{resid_reduction:g}"' if resid_reduction else ""
    return (f'<solver type="eigenvalue" k_tol="{k_tol:g}" psi_tol="{psi_tol:g}" max_iter="{max_iter}" '
            f'cmfd="{"t" if cmfd else "f"}">\n'
            f'  <cmfd{rr} />\n'
            f'  <source scattering="P0" />\n'
            f'  <sweeper type="moc" n_inner="{n_inner}" boundary_update="{boundary_update}" precision="{precision}">\n'
            f'    <ang_quad type="cy" n_azimuthal="{n_azi}" n_polar="3" />\n'
            f'    <rays spacing="{spacing:g}" />\n'
            f'  </sweeper>\n</solver>\n')


def _matlib_xml(n_fuel):
    mats = "".join(f'  <material id="{i + 1}" name="fuel{i + 1}" />\n' for i in range(n_fuel))
    return f'<material_lib path="synthetic.xsl">\n{mats}  <material id="9" name="moderator" />\n</material_lib>\n'


def _pins_xml(n_fuel):
    s = "".join(f'<pin id="{i + 1}" mesh="1"> {i + 1} {9} </pin>\n' for i in range(n_fuel))
    return s + '<pin id="10" mesh="1"> 9 9 </pin>\n'


def _lattice_xml(lid, rows):
    body = "\n".join("  " + " ".join(str(v) for v in row) for row in rows)
    return f'<lattice id="{lid}" nx="{len(rows[0])}" ny="{len(rows)}">\n{body}\n</lattice>\n'


def _core_xml(grid, north="reflect", south="reflect", east="reflect", west="reflect"):
    body = "\n".join("  " + " ".join(str(v) for v in row) for row in grid)
    return (f'<core nx="{len(grid[0])}" ny="{len(grid)}" north="{north}" south="{south}" east="{east}" '
            f'west="{west}" top="reflect" bottom="reflect">\n{body}\n</core>\n')


def lattice_case(n: int, n_azi: int, spacing: float, precision: str, seed: int, n_group: int = 7,
                 mod_factor: float = 1.0, fuel_nf_factor: float = 1.0, **solver_kw):
    """(xml, xsl) for a single reflective n x n lattice."""
    xml = (_solver_xml(n_azi, spacing, precision, **solver_kw) + _matlib_xml(1) + _mesh_xml() + _pins_xml(1)
           + _lattice_xml(1, lattice_rows(n)) + '<assembly id="1" np="1" hz="1.0"><lattices>1</lattices></assembly>\n'
           + _core_xml([[1]]))
    xsl = synthetic_xsl(seed, n_group=n_group, n_fuel=1, mod_factor=mod_factor, fuel_nf_factor=fuel_nf_factor)
    return xml, xsl


def pin3x3(seed: int = 20261203, precision: str = "double", **kw):
    return lattice_case(3, 8, 0.05, precision, seed, **kw)


def assembly17(seed: int = 20261203, precision: str = "mixed", **kw):
    return lattice_case(17, 16, 0.03, precision, seed, **kw)


def minicore(seed: int = 20261203, precision: str = "mixed", n_azi: int = 16, spacing: float = 0.03,
             n_lat: int = 17, **kw):
    """3x3 fuel assemblies (compositions 1..3) + moderator row north and east.

    ``n_lat`` shrinks the lattices (17 for the benchmark) for quick checks."""
    kw.setdefault("resid_reduction", 1e-8)
    xml = _solver_xml(n_azi, spacing, precision, **kw) + _matlib_xml(3) + _mesh_xml() + _pins_xml(3)
    for f in range(3):
        xml += _lattice_xml(f + 1, lattice_rows(n_lat, fuel_pin=f + 1))
        xml += f'<assembly id="{f + 1}" np="1" hz="1.0"><lattices>{f + 1}</lattices></assembly>\n'
    xml += _lattice_xml(4, [[10] * n_lat for _ in range(n_lat)])
    xml += '<assembly id="4" np="1" hz="1.0"><lattices>4</lattices></assembly>\n'
    # rows listed top (north) first: reflector on the top row and east column
    grid = [[4, 4, 4, 4]]
    for r in range(3):
        grid.append([(r + c) % 3 + 1 for c in range(3)] + [4])
    xml += _core_xml(grid, north="vacuum", east="vacuum", south="reflect", west="reflect")
    xsl = synthetic_xsl(seed, n_group=7, n_fuel=3, fuel_nf_scale=[1.0, 1.15, 1.3])
    return xml, xsl


BRANCH_SIZES = (1, 3, 7, 17)


def branch_cases(n_cases: int, seed: int = 7, weights=None, groups=(7,), precision: str = "mixed",
                 n_azi: int = 8, spacing: float = 0.05, **kw):
    """Seeded list of (size, n_group, xml, xsl) branch cases."""
    rng = random.Random(seed)
    out = []
    for i in range(n_cases):
        n = rng.choices(BRANCH_SIZES, weights=weights)[0] if weights else rng.choice(BRANCH_SIZES)
        ng = rng.choice(groups)
        mf = rng.uniform(0.9, 1.1)
        ff = rng.uniform(0.95, 1.05)
        xml, xsl = lattice_case(n, n_azi, spacing, precision, seed=1000 + (ng == 23) * 7, n_group=ng,
                                mod_factor=mf, fuel_nf_factor=ff, **kw)
        out.append((n, ng, xml, xsl))
    return out
