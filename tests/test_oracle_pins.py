"""Pin the CPU oracle to numbers the reference itself produced.

The fixtures in tests/golden were extracted from the reference's stored
notebook outputs and from its exact Riemann solver (tests/golden/make_golden.py).
"""
import json
import math
import os

import numpy as np
import torch

from oracle import jf_oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_tutorial01_dt_and_min_density_log_matches_printed_digits():
    """240 logged steps of linear advection: time, dt and min density as printed."""
    g = json.load(open(os.path.join(GOLDEN, "tut01_log.json")))
    case = O.OracleCase(cells=(50, 1, 1), nh=4, recon="MINMOD", riemann="HLLC",
                        signal_speed="EINFELDT", cfl=0.9, bc={f: "PERIODIC" for f in O.FACES})
    x = case.cell_centers(0)
    rho = 2.0 + torch.sin(2 * math.pi * x)
    prims = torch.stack([rho, torch.ones_like(x), torch.ones_like(x)]).reshape(3, 50, 1, 1)
    U, P = O.initialize(prims, case)
    log = []
    O.simulate(U, P, case, end_time=2.0, log=log)
    assert len(log) == len(g["rows"])
    for (t, dt, m), r in zip(log, g["rows"]):
        assert "%.5e" % t == "%.5e" % r["time"]
        assert "%.5e" % dt == "%.5e" % r["dt"]
        assert "%.4e" % m == "%.4e" % r["min_density"]


def _tut02_case():
    return O.OracleCase(cells=(100, 1, 1), nh=4, recon="MINMOD-AD", riemann="RUSANOV",
                        signal_speed="EINFELDT", fixed_dt=1e-3,
                        bc={f: "ZEROGRADIENT" for f in O.FACES})


def test_tutorial02_gradient_matches_jax_grad_trace():
    """Loss and d loss / d theta through 200 RK3 steps match jax.value_and_grad."""
    g = json.load(open(os.path.join(GOLDEN, "tut02_grad.json")))
    case = _tut02_case()
    x = case.cell_centers(0)
    rho = torch.where(x <= 0.5, 1.0, 0.125)
    p = torch.where(x <= 0.5, 1.0, 0.1)
    U, P = O.initialize(torch.stack([rho, torch.zeros_like(x), p]).reshape(3, 100, 1, 1), case)
    U, P, t, steps = O.simulate(U, P, case, end_time=0.2)
    assert steps == 200
    rho_ref = P[case.interior()][0].reshape(-1).clone()

    theta = torch.tensor(g["theta0"], dtype=torch.float64, requires_grad=True)
    d0 = torch.where(x < 0.5, theta[0], theta[1])
    u0 = torch.where(x < 0.5, theta[2], theta[3])
    p0 = torch.where(x < 0.5, theta[4], theta[5])
    z = torch.zeros_like(u0)
    U, P = O.initialize(torch.stack([d0, u0, z, z, p0]).reshape(5, 100, 1, 1), case)
    dt = torch.tensor(1e-3, dtype=torch.float64)
    for _ in range(200):
        U, P = O.rk3_step(U, P, dt, case)
    loss = torch.mean((P[case.interior()][0].reshape(-1) - rho_ref) ** 2)
    loss.backward()
    assert "%.2e" % loss.item() == "%.2e" % g["loss"]
    new = theta.detach() - g["lr"] * theta.grad
    for a, b in zip(new.tolist(), g["params_after_first_update"]):
        assert abs(a - b) <= 0.6e-8


def test_sod_weno5z_hllc_close_to_exact_solution():
    """WENO5-Z + HLLC, 200 cells, CFL 0.5 to t = 0.2 vs the reference's exact solver."""
    ex = np.load(os.path.join(GOLDEN, "sod_exact.npz"))
    case = O.OracleCase(cells=(200, 1, 1), nh=3, recon="WENO5-Z", riemann="HLLC",
                        signal_speed="EINFELDT", cfl=0.5, bc={f: "ZEROGRADIENT" for f in O.FACES})
    x = case.cell_centers(0)
    rho = torch.where(x <= 0.5, 1.0, 0.125)
    p = torch.where(x <= 0.5, 1.0, 0.1)
    U, P = O.initialize(torch.stack([rho, torch.zeros_like(x), p]).reshape(3, 200, 1, 1), case)
    U, P, t, steps = O.simulate(U, P, case, end_time=0.2)
    Pi = P[case.interior()].reshape(5, -1).numpy()
    xe, W = ex["x"], ex["W"]
    for row, var in ((0, 0), (1, 1), (2, 4)):
        exact = np.interp(x.numpy(), xe, W[row])
        l1 = np.mean(np.abs(Pi[var] - exact))
        assert l1 < 6e-3, (var, l1)
    assert abs(t - 0.2) < 2e-3
