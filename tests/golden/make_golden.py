"""Regenerate the golden fixtures in this folder from the JAX-Fluids sources.

Run from the repository root with the reference checkout at REFERENCE
(default /root/reference); the outputs are committed, so the tests never read
the reference at run time.

* ``tut01_log.json``: per-step (time, dt, min density) printed by the
  reference's own run of notebooks/basics/101/01_tutorial (linear advection,
  50 cells, MINMOD + HLLC/Einfeldt, PRIMITIVE, periodic, RK3, CFL 0.9,
  JAX CPU backend), parsed from the notebook's stored output.
* ``tut02_grad.json``: the losses and parameters printed every 25 iterations of
  the gradient-descent run of notebooks/basics/101/02_tutorial (Sod, 100 cells,
  MINMOD-AD + Rusanov, fixed dt 1e-3, 200 steps, jax.value_and_grad through
  _feed_forward), with the first update's gradient.
* ``sod_exact.npz``: the reference's exact Riemann solver
  (src/jaxfluids_thirdparty/exact_riemann_solver) for Sod at t = 0.2 sampled
  on 4001 points of x in [0, 1] (W = rho, u, p rows).
"""
import json
import os
import re
import sys
import types

import numpy as np

REFERENCE = os.environ.get("REFERENCE", "/root/reference")
HERE = os.path.dirname(os.path.abspath(__file__))


def _notebook_text(path, cell):
    nb = json.load(open(path))
    outs = nb["cells"][cell].get("outputs", [])
    return "".join("".join(o.get("text", "")) for o in outs)


def tut01():
    txt = _notebook_text(os.path.join(REFERENCE, "notebooks/basics/101/01_tutorial/01_tutorial.ipynb"), 9)
    pat = re.compile(
        r"CURRENT TIME\s+=\s+([0-9.e+-]+).*?CURRENT DT\s+=\s+([0-9.e+-]+).*?CURRENT STEP\s+=\s+(\d+)"
        r".*?MIN DENSITY\s+=\s+([0-9.e+-]+)", re.S)
    rows = [(int(m.group(3)), float(m.group(1)), float(m.group(2)), float(m.group(4)))
            for m in pat.finditer(txt)]
    steps = [r[0] for r in rows]
    assert steps == list(range(len(rows))), "unexpected log structure"
    return {
        "source": "notebooks/basics/101/01_tutorial/01_tutorial.ipynb cell 9 output",
        "case": {"cells": 50, "range": [0.0, 1.0], "bc": "PERIODIC", "recon": "MINMOD",
                 "riemann": "HLLC", "signal_speed": "EINFELDT", "cfl": 0.9, "nh": 4,
                 "end_time": 2.0, "rho": "2 + sin(2 pi x)", "u": 1.0, "p": 1.0, "gamma": 1.4},
        "digits": {"time": 6, "dt": 6, "min_density": 5},
        "rows": [{"step": s, "time": t, "dt": d, "min_density": m} for s, t, d, m in rows],
    }


def tut02():
    path = os.path.join(REFERENCE, "notebooks/basics/101/02_tutorial/02_tutorial.ipynb")
    txt = _notebook_text(path, 7)
    first = txt.splitlines()[0]
    m = re.match(r"0000, ([0-9.e+-]+), \[(.*)\]", first)
    loss = float(m.group(1))
    params1 = [float(x) for x in m.group(2).split()]
    theta0 = [1.0, 1.0, 0.0, 0.0, 1.0, 1.0]
    lr = 0.2
    grad = [(a - b) / lr for a, b in zip(theta0, params1)]
    # every printed line: iteration, loss (3 digits) and the parameters after
    # that iteration's update (numpy's 8 decimals); plain gradient descent with
    # lr_schedule of cell 6 (0.2 below 50, 0.1 below 200, else 0.01)
    traj = []
    for line in txt.splitlines():
        mm = re.match(r"(\d{4}), ([0-9.e+-]+), \[(.*)\]", line.strip())
        if mm:
            traj.append({"itr": int(mm.group(1)), "loss": float(mm.group(2)),
                         "params": [float(x) for x in mm.group(3).split()]})
    return {
        "source": "notebooks/basics/101/02_tutorial/02_tutorial.ipynb cell 7 output",
        "case": {"cells": 100, "range": [0.0, 1.0], "bc": "ZEROGRADIENT", "recon": "MINMOD-AD",
                 "riemann": "RUSANOV", "signal_speed": "EINFELDT", "fixed_dt": 1e-3, "nh": 4,
                 "steps": 200, "end_time_ref": 0.2, "gamma": 1.4},
        "theta0": theta0, "lr": lr, "loss": loss, "loss_digits": 3,
        "params_after_first_update": params1, "params_decimals": 8, "grad": grad,
        "lr_schedule": [[50, 0.2], [200, 0.1], [None, 0.01]], "trajectory": traj,
    }


def sod_exact():
    sys.path.insert(0, os.path.join(REFERENCE, "src"))
    # the solver imports matplotlib at module level but only plots on request
    mpl = types.ModuleType("matplotlib")
    mpl.pyplot = types.ModuleType("matplotlib.pyplot")
    sys.modules.setdefault("matplotlib", mpl)
    sys.modules.setdefault("matplotlib.pyplot", mpl.pyplot)
    from jaxfluids_thirdparty.exact_riemann_solver.exact_riemann_solver import ExactRiemannSolver
    res = ExactRiemannSolver().solve([1.0, 0.0, 1.0], [0.125, 0.0, 0.1], gamma_L=1.4, gamma_R=1.4,
                                     Nx=4001, ts=0.2, xlims=(0.0, 1.0), x0=0.5)
    p_star, u_star, W, x = res
    return {"p_star": np.float64(p_star), "u_star": np.float64(u_star), "W": np.asarray(W), "x": np.asarray(x)}


def main():
    json.dump(tut01(), open(os.path.join(HERE, "tut01_log.json"), "w"), indent=1)
    json.dump(tut02(), open(os.path.join(HERE, "tut02_grad.json"), "w"), indent=1)
    arrays = sod_exact()
    np.savez(os.path.join(HERE, "sod_exact.npz"), **arrays)
    print({k: np.shape(v) for k, v in arrays.items()})


if __name__ == "__main__":
    main()
