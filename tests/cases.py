"""Shared test cases: the same setup as an oracle case and as a CaseConfig."""
import math

import numpy as np
import torch

from oracle import jf_oracle as O


def both(cells, bc, **kw):
    """(OracleCase, CaseConfig) for the same setup."""
    from jaxfluids_gb300.config import CaseConfig
    bcd = {f: bc[f] if isinstance(bc, dict) else bc for f in O.FACES}
    okw = {k: v for k, v in kw.items() if k != "kappa"}
    if "kappa" in kw:
        okw["thermal_conductivity"] = kw["kappa"]
    oc = O.OracleCase(cells=cells, bc=bcd, **okw)
    fields = {k: v for k, v in kw.items() if k in (
        "ranges", "nh", "gamma", "R", "recon", "recon_var", "frozen_state", "riemann", "signal_speed",
        "cfl", "fixed_dt", "viscous", "heat", "mu", "bulk_viscosity", "prandtl", "kappa", "viscous_heat_production",
        "bc_values", "diss_recon", "diss_deriv_center", "diss_deriv_face", "convective",
        "interpolation_limiter", "limit_velocity", "gravity")}
    cc = CaseConfig(cells=cells, bc={f: bcd[f] for f in O.FACES}, **fields)
    # boundary callables, strings and bounding domains reach the oracle as the
    # values CaseConfig evaluated at the boundary cells
    oc.bc = {f: cc.bc.get(f, oc.bc[f]) for f in O.FACES}
    oc.bc_values = dict(cc.bc_values)
    oc.bc_time = {f: (lambda t, f=f: cc.bc_values_at(f, t)) for f in cc.time_varying_faces}
    return oc, cc


def sod_prims(n=200):
    x = (np.arange(n) + 0.5) / n
    rho = np.where(x <= 0.5, 1.0, 0.125)
    p = np.where(x <= 0.5, 1.0, 0.1)
    return torch.from_numpy(np.stack([rho, np.zeros(n), p]).reshape(3, n, 1, 1))


def quadrant_prims(nx, ny, seed=0):
    """2-D four-quadrant Riemann problem, states drawn from U ranges."""
    rng = np.random.default_rng(seed)
    st = np.stack([rng.uniform(0.1, 2, 4), rng.uniform(-1, 1, 4), rng.uniform(-1, 1, 4),
                   rng.uniform(0.1, 2, 4)])
    x = (np.arange(nx) + 0.5) / nx
    y = (np.arange(ny) + 0.5) / ny
    X, Y = np.meshgrid(x, y, indexing="ij")
    q = (X >= 0.5).astype(int) + 2 * (Y >= 0.5).astype(int)
    f = st[:, q]  # [4, nx, ny]
    return torch.from_numpy(np.stack([f[0], f[1], f[2], f[3]]).reshape(4, nx, ny, 1))


def tgv_prims(n, ma=0.1, gamma=1.4, lengths=(2 * math.pi,) * 3, dims=3):
    """Taylor-Green vortex initial condition on [0, 2 pi]^3 (or a 2-D slice)."""
    p0 = 1.0 / (gamma * ma * ma)
    axes = [(np.arange(n) + 0.5) * (lengths[i] / n) for i in range(3)]
    if dims == 2:
        axes[2] = np.array([0.0])
    X, Y, Z = np.meshgrid(*axes, indexing="ij")
    u = np.sin(X) * np.cos(Y) * np.cos(Z)
    v = -np.cos(X) * np.sin(Y) * np.cos(Z)
    w = np.zeros_like(X)
    p = p0 + (np.cos(2 * X) + np.cos(2 * Y)) * (np.cos(2 * Z) + 2.0) / 16.0
    rho = np.ones_like(X)
    return torch.from_numpy(np.stack([rho, u, v, w, p]))


def rel_err(a: torch.Tensor, b: torch.Tensor) -> float:
    """max over variables of ||a_v - b_v||_inf / ||b_v||_inf."""
    a = a.detach().cpu().reshape(a.shape[0], -1)
    b = b.detach().cpu().reshape(b.shape[0], -1)
    worst = 0.0
    for v in range(a.shape[0]):
        den = b[v].abs().max().item()
        num = (a[v] - b[v]).abs().max().item()
        worst = max(worst, num / den if den > 0 else num)
    return worst


def smooth_field(cells, seed, mean, amp):
    """Sum of random-phase cosines varying along every active axis (no flat
    directions, where WENO-Z's derivative is not numerically meaningful)."""
    rng = np.random.default_rng(seed)
    axes = [(np.arange(n) + 0.5) / n for n in cells]
    X = np.meshgrid(*axes, indexing="ij")
    f = np.full(X[0].shape, mean, dtype=np.float64)
    for _ in range(3):
        k = rng.integers(1, 3, size=3)
        ph = rng.uniform(0, 2 * np.pi, size=3)
        term = np.ones_like(f)
        for a in range(3):
            if cells[a] > 1:
                term = term * np.cos(2 * np.pi * k[a] * X[a] + ph[a])
        f = f + amp * rng.uniform(0.3, 1.0) * term
    return f


def generic_cons(cells, seed=0):
    P = np.stack([smooth_field(cells, seed, 1.0, 0.2), smooth_field(cells, seed + 1, 0.0, 0.3),
                  smooth_field(cells, seed + 2, 0.0, 0.3) if cells[1] > 1 else np.zeros(cells),
                  smooth_field(cells, seed + 3, 0.0, 0.3) if cells[2] > 1 else np.zeros(cells),
                  smooth_field(cells, seed + 4, 1.0, 0.2)])
    return O.cons_from_prims(torch.from_numpy(P), 1.4)


def reflect_xy(U: torch.Tensor) -> torch.Tensor:
    """Cells (i, j, k) -> (j, i, k) with the x and y velocity (or momentum)
    components swapped: the mirror image of a field in the plane x = y."""
    return U.transpose(1, 2)[[0, 2, 1, 3, 4]].contiguous()


def assert_conserved(U0: torch.Tensor, UK: torch.Tensor, tol: float = 1e-12) -> None:
    """Domain totals of mass, momentum and energy unchanged to `tol` relative to
    the total of |rho|, of |rho u_i| over all components, and of |E|."""
    t0 = U0.reshape(5, -1).sum(1)
    tk = UK.reshape(5, -1).sum(1)
    a0 = U0.reshape(5, -1).abs().sum(1)
    mom = a0[1] + a0[2] + a0[3]
    scale = [a0[0], mom, mom, mom, a0[4]]
    for v in range(5):
        assert abs((tk[v] - t0[v]).item()) <= tol * scale[v].item(), (v, tk[v].item(), t0[v].item())
