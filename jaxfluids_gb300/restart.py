"""Output and restart of the single-phase state in the reference's field layout.

The reference writes its output with h5py (io_utils/hdf5_writer.py:79-265)
and restarts from such a file (initialization/material_fields_initializer.py:
212-340, loader initialization/helper_functions.py:195-223).  h5py is
installed on neither machine of this build, so the same datasets go into a
numpy ``.npz`` archive instead, under the reference's dataset names:

* ``time``; ``domain/dim``, ``domain/active_axes_indices``,
  ``domain/split_factors``, ``domain/gridX|Y|Z`` (cell centres),
  ``domain/gridFX|FY|FZ`` (cell faces), ``domain/cellsizeX|Y|Z``;
  ``metadata/is_double_precision``, ``metadata/available_quantities/primitives``;
* ``primitives/density``, ``primitives/velocity``, ``primitives/pressure``,
  each the interior field transposed as the reference writes it
  (``buffer.T``: scalars ``[Nz, Ny, Nx]``, the velocity ``[Nz, Ny, Nx, 3]``).

A restart, as the reference's, reads the primitives and rebuilds the
conservatives from them (``create_material_fields``); the fused path then takes
the primitives for its first stage, so a restarted run continues exactly as a
run started from those primitives.
"""
from __future__ import annotations

from typing import Tuple

import numpy as np

from .config import CaseConfig


def _cell_faces(cfg: CaseConfig, axis: int) -> np.ndarray:
    lo, hi = cfg.ranges[axis]
    return np.linspace(lo, hi, cfg.cells[axis] + 1)


def write_fields(path: str, config: CaseConfig, primitives, time: float) -> str:
    """Write interior primitives [5, Nx, Ny, Nz] (numpy or torch) and the time."""
    P = primitives.detach().cpu().numpy() if hasattr(primitives, "detach") else np.asarray(primitives)
    P = np.asarray(P, dtype=np.float64).reshape((5,) + tuple(config.cells))
    out = {
        "time": np.float64(time),
        "domain/dim": np.int64(len(config.active)),
        "domain/active_axes_indices": np.array(config.active, dtype=np.int64),
        "domain/split_factors": np.ones(3, dtype=np.int64),
        "metadata/is_double_precision": np.bool_(True),
        "metadata/available_quantities/primitives": np.array(["density", "velocity", "pressure"]),
        "primitives/density": P[0].T,
        "primitives/velocity": P[1:4].T,
        "primitives/pressure": P[4].T,
    }
    for a, ax in enumerate("XYZ"):
        out[f"domain/grid{ax}"] = config.cell_centers(a)
        out[f"domain/gridF{ax}"] = _cell_faces(config, a)
        out[f"domain/cellsize{ax}"] = np.full(config.cells[a], config.cell_size(a) if config.cells[a] > 1 else
                                              config.ranges[a][1] - config.ranges[a][0])
    if not path.endswith(".npz"):
        path = path + ".npz"
    np.savez(path, **out)
    return path


def read_fields(path: str, config: CaseConfig = None) -> Tuple[np.ndarray, float]:
    """Interior primitives [5, Nx, Ny, Nz] and the time of a file written by
    write_fields (the inverse transposes of the reference's loader)."""
    with np.load(path) as z:
        rho = z["primitives/density"].T
        vel = np.moveaxis(z["primitives/velocity"], -1, -4)
        vel = np.swapaxes(vel, -1, -3)
        p = z["primitives/pressure"].T
        t = float(z["time"])
        cells = tuple(len(z[f"domain/grid{ax}"]) for ax in "XYZ")
    P = np.concatenate([rho[None], vel, p[None]], axis=0)
    if config is not None and tuple(config.cells) != cells:
        raise ValueError(f"restart file has {cells} cells, the case {config.cells}")
    return np.ascontiguousarray(P), t
