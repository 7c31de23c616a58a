"""MOCC's output datasets after an eigenvalue solve (EigenSolver::output,
eigen_solver.cpp:293-322, and the FixedSourceSolver, MoCSweeper and
AngularQuadrature output it calls): the same paths, shapes and scaling as
the oracle's restatement of them (``oracle.mocc_output``) on the oracle's
own trace of the same input.

* CPU: the input-side datasets (quadrature of all 8 octants after
  modularisation, group bounds) from the library's trace equal the
  oracle tracer's, on MOCC's example 3x3 input with its C5G7 library and on
  a synthetic lattice;
* GPU: after an FP64 solve every dataset matches: the pin flux under MOCC's
  Normalize and the pin powers to 1e-8, k per outer iteration to 1e-9, the
  convergence errors to 1e-9 absolute; the archive written by save_npz
  reads back the same.
"""
import numpy as np
import pytest

import mocc_gb300 as m
import oracle
from mocc_gb300 import output as out_mod
from mocc_gb300 import workloads as W

QUAD = ("alpha", "theta", "omega_x", "omega_y", "omega_z", "weight")


def _inputs(ref_example, ref_xsl):
    return {"example_3x3": (ref_example["3x3"], ref_xsl), "lattice3": W.lattice_case(3, 8, 0.05, "double", seed=1000)}


def test_quadrature_and_group_bounds_match_oracle_tracer(ref_example, ref_xsl):
    for name, (xml, xsl) in _inputs(ref_example, ref_xsl).items():
        P, T = m.Problem(xml, xsl), oracle.Traced(xml, xsl)
        q = P.quadrature()
        npol, nazi = T.array("quad_n")
        assert (q["n_polar"], q["n_azimuthal"]) == (npol, nazi), name
        # a level-symmetric set keeps MOCC's -1 for both (the input has no
        # n_polar / n_azimuthal attributes)
        assert len(q["alpha"]) % 8 == 0
        if npol > 0:
            assert len(q["alpha"]) == 8 * npol * nazi
        for key, orc in zip(QUAD, ("quad_alpha", "quad_theta", "quad_ox", "quad_oy", "quad_oz", "quad_weight")):
            np.testing.assert_allclose(q[key], T.array(orc), rtol=0, atol=1e-14, err_msg=f"{name} {key}")
        assert np.array_equal(P.group_bounds(), T.array("group_bounds")), name
    # MOCC's C5G7 library header: 7 groups from 20 MeV down to 0.0635 eV
    b = m.Problem(ref_example["3x3"], ref_xsl).group_bounds()
    assert len(b) == 7 and b[0] == 2.0e7 and b[-1] == 0.0635


def test_dump_fsr_flux_option_is_read_from_the_sweeper_tag(ref_example, ref_xsl):
    xml = ref_example["3x3"]
    assert m.Problem(xml, ref_xsl).options["dump_fsr_flux"] == 0
    tagged = xml.replace("<sweeper ", '<sweeper dump_fsr_flux="true" ', 1)
    assert tagged != xml and m.Problem(tagged, ref_xsl).options["dump_fsr_flux"] == 1


class _FakeSweeper:
    def __init__(self, G, ny, nx, n_fsr, rng):
        self.n_group, self._ny, self._nx = G, ny, nx
        self._pin = rng.uniform(0.1, 2.0, size=(ny * nx, G))
        self._pin[0, :] = 0.0  # a pin without flux (counted out by Normalize)
        self._fsr = rng.uniform(0.1, 2.0, size=(n_fsr, G))
        self._pow = rng.uniform(0.5, 1.5, size=(ny, nx))

    def get_pin_flux_1g(self, g):
        return self._pin[:, g].copy()

    def pin_powers(self):
        return self._pow.copy()

    def flux(self):
        return self._fsr.copy()


class _FakeProblem:
    def __init__(self, ny, nx, n_fsr):
        self.sizes = {"nx": nx, "ny": ny, "nfsr": n_fsr}
        self.options = {"dump_fsr_flux": 0}

    def group_bounds(self):
        return np.array([2.0e7, 1.0e6, 0.625])

    def quadrature(self):
        return {"n_polar": 1, "n_azimuthal": 1, **{k: np.arange(8.0) for k in QUAD}}


class _FakeSolver:
    def __init__(self):
        rng = np.random.default_rng(5)
        self.sweeper, self.problem = _FakeSweeper(3, 2, 3, 10, rng), _FakeProblem(2, 3, 10)

    def history(self):
        return np.array([[1.1, 0.1, 0.2, 0.5], [1.05, 0.05, 0.01, 0.9]])


def test_output_layout_and_normalize_on_a_fake_solver():
    # the assembly of the datasets alone (no GPU): paths, shapes, MOCC's
    # Normalize over the whole [pin][group] pin flux, fsr_flux only when asked
    S = _FakeSolver()
    d = out_mod.eigen_output(S)
    assert not any(k.startswith("fsr_flux/") for k in d)
    assert [k for k in d if k.startswith("flux/")] == ["flux/001", "flux/002", "flux/003"]
    allf = np.concatenate([d[f"flux/{g:03d}"].ravel() for g in (1, 2, 3)])
    assert d["flux/001"].shape == (1, 2, 3)
    assert abs(allf.sum() - np.count_nonzero(allf > 0)) < 1e-12 * allf.size
    ratio = d["flux/002"].reshape(-1)[1:] / S.sweeper._pin[1:, 1]
    assert np.allclose(ratio, ratio[0])  # one common factor for all groups
    assert np.array_equal(d["convergence/k"], [1.1, 1.05])
    assert np.array_equal(d["convergence/iteration_time"], d["convergence/abscissae"])
    assert d["pin_powers"].shape == (1, 2, 3) and int(d["ng"]) == 3
    assert d["ang_quad/weight"].shape == (8,) and int(d["ang_quad/n_polar"]) == 1
    d2 = out_mod.eigen_output(S, dump_fsr_flux=True)
    assert d2["fsr_flux/002"].shape == (10, 1)
    assert np.array_equal(d2["fsr_flux/002"][:, 0], S.sweeper._fsr[:, 1])


def test_npz_round_trip(tmp_path):
    d = {"convergence/k": np.array([1.0, 0.9]), "ng": np.array(7, dtype=np.int32),
         "flux/001": np.ones((1, 2, 3))}
    p = tmp_path / "out.npz"
    out_mod.save_npz(str(p), d)
    back = out_mod.load_npz(str(p))
    assert set(back) == set(d)
    for k in d:
        assert back[k].shape == d[k].shape and np.array_equal(back[k], d[k])


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["example_3x3", "lattice3"])
def test_eigen_output_matches_oracle(case, ref_example, ref_xsl, tmp_path):
    xml, xsl = _inputs(ref_example, ref_xsl)[case]
    P = m.Problem(xml, xsl)
    E = m.EigenSolver(P, 0)
    r = E.solve()
    O = oracle.OracleSolver.from_xml(xml, xsl)
    ro = O.solve()
    assert r["converged"] and ro["converged"] and r["iterations"] == ro["iterations"]
    a, b = E.output(dump_fsr_flux=True), O.output()
    G = P.sizes["ngroup"]
    assert set(a) == set(b) | {f"fsr_flux/{g + 1:03d}" for g in range(G)}
    for k, v in b.items():
        assert a[k].shape == v.shape and a[k].dtype == v.dtype, k
    n = r["iterations"]
    assert a["convergence/k"].shape == (n,)
    np.testing.assert_allclose(a["convergence/k"], b["convergence/k"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(a["convergence/error_k"], b["convergence/error_k"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(a["convergence/error_psi"], b["convergence/error_psi"], rtol=0, atol=1e-9)
    t = a["convergence/iteration_time"]
    assert np.all(np.diff(t) >= 0.0) and np.array_equal(t, a["convergence/abscissae"])
    assert int(a["ng"]) == G and np.array_equal(a["eubounds"], b["eubounds"])
    for g in range(G):
        k = f"flux/{g + 1:03d}"
        np.testing.assert_allclose(a[k], b[k], rtol=1e-8, atol=0, err_msg=k)
        assert a[f"fsr_flux/{g + 1:03d}"].shape == (P.sizes["nfsr"], 1)
    # Normalize: the pin flux of all groups sums to its number of positive entries
    allf = np.concatenate([a[f"flux/{g + 1:03d}"].ravel() for g in range(G)])
    assert abs(allf.sum() - np.count_nonzero(allf > 0)) < 1e-9 * allf.size
    q = b["pin_powers"] > 0
    np.testing.assert_allclose(a["pin_powers"][q], b["pin_powers"][q], rtol=1e-8, atol=0)
    for key in ("n_polar", "n_azimuthal") + QUAD:
        np.testing.assert_allclose(a["ang_quad/" + key], b["ang_quad/" + key], rtol=0, atol=1e-14)
    p = tmp_path / "mocc_output.npz"
    out_mod.save_npz(str(p), a)
    back = out_mod.load_npz(str(p))
    assert set(back) == set(a) and all(np.array_equal(back[k], a[k]) for k in a)
