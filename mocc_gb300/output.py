"""MOCC's output datasets after an eigenvalue solve.

MOCC writes its results to an HDF5 file through ``EigenSolver::output``
(``src/solvers/eigen_solver.cpp:293-322``), which calls
``FixedSourceSolver::output`` (``src/solvers/fixed_source_solver.cpp:
119-129``), ``MoCSweeper::output`` (``src/sweepers/moc/moc_sweeper.cpp:
533-585``) and ``AngularQuadrature::output``
(``src/core/angular_quadrature.cpp:213-248``). ``eigen_output`` returns
the same datasets, under the same paths, with the same shapes and scaling,
as ``{path: numpy array}``:

* ``convergence/k``, ``error_k``, ``error_psi``: one entry per outer
  iteration; ``iteration_time`` and ``abscissae``: the time of each
  iteration (MOCC writes its iteration times under both names), here
  seconds since the solve began;
* ``ng`` and ``eubounds`` (the library's group upper bounds);
* ``flux/001`` .. ``flux/NNN``: the volume-averaged pin flux of each group,
  the whole [pin][group] array scaled as ``Normalize`` does (to sum to its
  number of positive entries), each group shaped (nz, ny, nx) = (1, ny, nx);
  ``fsr_flux/NNN`` of the FSR flux when ``dump_fsr_flux`` (MOCC's
  ``dump_fsr_flux`` option), shaped (n_fsr, 1);
* ``pin_powers``, shaped (1, ny, nx);
* ``ang_quad/n_polar``, ``n_azimuthal`` and every angle's ``alpha``,
  ``theta``, ``omega_x``, ``omega_y``, ``omega_z``, ``weight``.

No HDF5 library is installed where this package is built, so the container
is left to the caller: ``save_npz`` writes the datasets under their paths to
a NumPy archive, and any HDF5 writer can take the dict as it is (one dataset
per key; keys with a ``/`` lie in groups).
"""
from __future__ import annotations

import numpy as np


def eigen_output(solver, dump_fsr_flux: bool = False) -> dict:
    """Datasets of MOCC's output for ``solver`` (a solved
    ``mocc_gb300.EigenSolver``)."""
    S, P = solver.sweeper, solver.problem
    h = solver.history()
    if h.shape[0] == 0:
        raise ValueError("no eigenvalue solve has run on this solver")
    G, nx, ny = S.n_group, int(P.sizes["nx"]), int(P.sizes["ny"])
    # MoCSweeper::output: get_pin_flux(), then Normalize over all of it
    flux = np.stack([S.get_pin_flux_1g(g) for g in range(G)], axis=1)
    flux = flux * (np.count_nonzero(flux > 0.0) / flux.sum())
    out = {
        "convergence/k": h[:, 0].copy(),
        "convergence/error_k": h[:, 1].copy(),
        "convergence/error_psi": h[:, 2].copy(),
        "convergence/iteration_time": h[:, 3].copy(),
        "convergence/abscissae": h[:, 3].copy(),
        "ng": np.array(G, dtype=np.int32),
        "eubounds": P.group_bounds(),
    }
    if dump_fsr_flux:
        phi = S.flux()
        for g in range(G):
            out[f"fsr_flux/{g + 1:03d}"] = phi[:, g].reshape(-1, 1).copy()
    for g in range(G):
        out[f"flux/{g + 1:03d}"] = flux[:, g].reshape(1, ny, nx).copy()
    out["pin_powers"] = S.pin_powers().reshape(1, ny, nx)
    q = P.quadrature()
    out["ang_quad/n_polar"] = np.array(q["n_polar"], dtype=np.int32)
    out["ang_quad/n_azimuthal"] = np.array(q["n_azimuthal"], dtype=np.int32)
    for key in ("alpha", "theta", "omega_x", "omega_y", "omega_z", "weight"):
        out["ang_quad/" + key] = q[key]
    return out


def save_npz(path: str, datasets: dict) -> None:
    """Writes the datasets to a NumPy archive, one member per path."""
    np.savez(path, **datasets)


def load_npz(path: str) -> dict:
    with np.load(path) as z:
        return {k: z[k] for k in z.files}
