"""Hand-written adjoint vs the oracle's autograd (jax.grad conventions), the
reference's recorded jax.grad trace, finite differences, and checkpointing."""
import json
import math
import os

import numpy as np
import pytest
import torch

from oracle import jf_oracle as O
from tests.cases import both, generic_cons, quadrant_prims, rel_err, sod_prims, tgv_prims

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
TOL = 1e-11


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from jaxfluids_gb300 import build
    build.build()


def kh_cons(nx, ny, gamma=1.4, seed=7):
    rng = np.random.default_rng(seed)
    x = (np.arange(nx) + 0.5) / nx
    y = (np.arange(ny) + 0.5) / ny
    X, Y = np.meshgrid(x, y, indexing="ij")
    inner = np.abs(Y - 0.5) < 0.25
    rho = np.where(inner, 2.0, 1.0)
    u = np.where(inner, 0.5, -0.5)
    v = 0.01 * np.sin(4 * np.pi * X) + rng.normal(0, 1e-3, X.shape)
    p = np.full_like(X, 2.5)
    P = torch.from_numpy(np.stack([rho, u, v, np.zeros_like(rho), p]).reshape(5, nx, ny, 1))
    return O.cons_from_prims(P, gamma)


def smooth_kh_cons(nx, ny, gamma=1.4, seed=7):
    """Shear layer with tanh profiles: smooth, so finite differences are derivatives
    (WENO-Z is not differentiable at piecewise-constant data)."""
    rng = np.random.default_rng(seed)
    x = (np.arange(nx) + 0.5) / nx
    y = (np.arange(ny) + 0.5) / ny
    X, Y = np.meshgrid(x, y, indexing="ij")
    s = np.tanh((0.25 - np.abs(Y - 0.5)) / 0.08)
    rho = 1.5 + 0.5 * s
    u = 0.5 * s
    v = 0.01 * np.sin(4 * np.pi * X) + rng.normal(0, 1e-3, X.shape)
    p = 2.5 + 0.1 * np.cos(2 * np.pi * X)
    P = torch.from_numpy(np.stack([rho, u, v, np.zeros_like(rho), p]).reshape(5, nx, ny, 1))
    return O.cons_from_prims(P, gamma)


def square_wave_prims(n):
    """1-D periodic state of two constant parts, the faster one (|u| + c) over
    the periodic wrap: its flat faces, face -1/2 among them, all attain the
    Lax-Friedrichs speed."""
    x = (np.arange(n) + 0.5) / n
    fast = (x < 0.25) | (x >= 0.75)
    P = np.stack([np.where(fast, 1.0, 0.5), np.where(fast, 0.5, -0.2), np.zeros(n), np.zeros(n),
                  np.where(fast, 1.0, 0.4)])
    return torch.from_numpy(P.reshape(5, n, 1, 1))


def mirror_prims(n):
    """1-D periodic smooth state, mirror-symmetric about the domain centre with
    the velocity odd: a face state and its mirror image have bitwise equal
    Lax-Friedrichs speeds, so the maximum is attained by a left and a right
    state at once."""
    x = (np.arange(n // 2) + 0.5) / n
    rho = 1.0 + 0.2 * np.cos(2 * np.pi * x)
    u = 0.3 * np.sin(2 * np.pi * x)
    p = 1.0 + 0.1 * np.cos(2 * np.pi * x)
    P = np.zeros((5, n))
    P[0] = np.concatenate([rho, rho[::-1]])
    P[1] = np.concatenate([u, -u[::-1]])
    P[4] = np.concatenate([p, p[::-1]])
    return torch.from_numpy(P.reshape(5, n, 1, 1))


def _interior_cons(kind, cells, oc):
    if kind == "generic":
        return generic_cons(cells)
    if kind == "mirror":
        return O.cons_from_prims(mirror_prims(cells[0]), 1.4)
    if kind == "square":
        return O.cons_from_prims(square_wave_prims(cells[0]), 1.4)
    if kind == "kh":
        return kh_cons(cells[0], cells[1])
    if kind == "sod":
        U, P = O.initialize(sod_prims(cells[0]), oc)
        return U[oc.interior()].clone()
    if kind == "quad":
        U, P = O.initialize(quadrant_prims(cells[0], cells[1], seed=5), oc)
        return U[oc.interior()].clone()
    U, P = O.initialize(tgv_prims(max(cells))[:, :cells[0], :cells[1], :cells[2]].contiguous(), oc)
    g = torch.Generator().manual_seed(3)
    Ui = U[oc.interior()].clone()
    return Ui * (1 + 1e-3 * torch.rand(Ui.shape, generator=g, dtype=torch.float64))


# WENO-Z's Jacobian is only numerically meaningful where the data varies in
# every direction (flat data multiplies rounding noise by 1/eps = 1e30), so the
# WENO cases use smooth random-phase fields; the MINMOD-AD case keeps Sod.
VJP_CASES = [
    ("2d-weno-hllc", (40, 36, 1), "PERIODIC", {}, "generic"),
    ("2d-weno-rusanov-zg", (20, 36, 1), "ZEROGRADIENT", {"riemann": "RUSANOV"}, "generic"),
    ("sod-minmodad-rusanov", (40, 1, 1), "ZEROGRADIENT", {"nh": 4, "recon": "MINMOD-AD", "riemann": "RUSANOV"}, "sod"),
    ("2d-sym-hllc", (36, 20, 1), {"east": "SYMMETRY", "west": "SYMMETRY", "north": "PERIODIC", "south": "PERIODIC",
                                   "top": "PERIODIC", "bottom": "PERIODIC"}, {}, "generic"),
    ("3d-weno-hllc", (20, 12, 18), "PERIODIC", {}, "generic"),
    ("3d-minmodad-rusanov-zg", (12, 10, 20), "ZEROGRADIENT", {"nh": 4, "recon": "MINMOD-AD", "riemann": "RUSANOV"},
     "generic"),
    ("2d-char-roe-hllc", (40, 36, 1), "PERIODIC", {"recon_var": "CHAR-PRIMITIVE", "frozen_state": "ROE"}, "generic"),
    ("2d-char-arith-rusanov-zg", (20, 36, 1), "ZEROGRADIENT", {"recon_var": "CHAR-PRIMITIVE", "riemann": "RUSANOV"},
     "generic"),
    ("2d-char-roe-sym", (36, 20, 1), {"east": "SYMMETRY", "west": "SYMMETRY", "north": "ZEROGRADIENT",
                                       "south": "ZEROGRADIENT", "top": "PERIODIC", "bottom": "PERIODIC"},
     {"recon_var": "CHAR-PRIMITIVE", "frozen_state": "ROE"}, "generic"),
    ("3d-char-roe-hllc", (16, 12, 14), "PERIODIC", {"recon_var": "CHAR-PRIMITIVE", "frozen_state": "ROE"}, "generic"),
    ("2d-viscous-heat", (24, 20, 1), "PERIODIC", {"nh": 4, "viscous": True, "heat": True, "mu": 0.05,
                                                   "prandtl": 0.71}, "generic"),
    ("2d-heat-only", (20, 24, 1), "PERIODIC", {"nh": 4, "heat": True, "mu": 0.05, "prandtl": 0.71}, "generic"),
    ("3d-viscous-noheatprod", (12, 16, 10), "PERIODIC", {"nh": 4, "viscous": True, "mu": 0.02,
                                                          "viscous_heat_production": False}, "generic"),
    ("2d-weno5js-hll", (40, 36, 1), "PERIODIC", {"recon": "WENO5-JS", "riemann": "HLL"}, "generic"),
    ("2d-weno3js-hllc", (40, 36, 1), "PERIODIC", {"recon": "WENO3-JS"}, "generic"),
    ("2d-weno3z-rusanov-zg", (20, 36, 1), "ZEROGRADIENT", {"recon": "WENO3-Z", "riemann": "RUSANOV"}, "generic"),
    ("3d-weno5z-hll", (12, 14, 10), "PERIODIC", {"riemann": "HLL"}, "generic"),
    ("3d-char-roe-hll", (16, 12, 14), "PERIODIC", {"recon_var": "CHAR-PRIMITIVE", "frozen_state": "ROE",
                                                   "riemann": "HLL"}, "generic"),
    ("sod-minmodad-hll", (40, 1, 1), "ZEROGRADIENT", {"nh": 4, "recon": "MINMOD-AD", "riemann": "HLL"}, "sod"),
    # every signal-speed estimate of HLLC and HLL
    ("2d-weno-hllc-davis", (40, 36, 1), "PERIODIC", {"signal_speed": "DAVIS"}, "generic"),
    ("2d-weno-hllc-arith-zg", (24, 20, 1), "ZEROGRADIENT", {"signal_speed": "ARITHMETIC"}, "generic"),
    ("2d-weno-hllc-rusanov-speed", (40, 36, 1), "PERIODIC", {"signal_speed": "RUSANOV"}, "generic"),
    ("2d-weno-hllc-toro", (40, 36, 1), "PERIODIC", {"signal_speed": "TORO"}, "generic"),
    ("2d-weno-hll-toro", (32, 28, 1), "PERIODIC", {"riemann": "HLL", "signal_speed": "TORO"}, "generic"),
    ("3d-char-roe-hll-davis", (12, 10, 14), "PERIODIC", {"recon_var": "CHAR-PRIMITIVE", "frozen_state": "ROE",
                                                          "riemann": "HLL", "signal_speed": "DAVIS"}, "generic"),
    ("2d-cons-hllc-arith", (24, 20, 1), "PERIODIC", {"recon_var": "CONSERVATIVE", "signal_speed": "ARITHMETIC"},
     "generic"),
    # MINMOD: the limiter max(0, min(1, r)) clips on the smooth fields' steep
    # parts and passes r on their flat ones
    ("sod-minmod-hllc", (40, 1, 1), "ZEROGRADIENT", {"nh": 4, "recon": "MINMOD"}, "sod"),
    ("2d-minmod-hllc", (40, 36, 1), "PERIODIC", {"nh": 4, "recon": "MINMOD"}, "generic"),
    ("3d-minmod-lf-zg", (12, 10, 14), "ZEROGRADIENT", {"nh": 4, "recon": "MINMOD", "riemann": "LAX-FRIEDRICHS"},
     "generic"),
    ("2d-minmod-rusanov-viscous", (24, 20, 1), "PERIODIC", {"nh": 4, "recon": "MINMOD", "riemann": "RUSANOV",
                                                             "viscous": True, "heat": True, "mu": 0.02,
                                                             "prandtl": 0.71}, "generic"),
    # CONSERVATIVE: WENO5-Z on the conservatives
    ("2d-cons-hllc", (32, 28, 1), "PERIODIC", {"recon_var": "CONSERVATIVE"}, "generic"),
    ("3d-cons-hll-zg", (12, 14, 10), "ZEROGRADIENT", {"recon_var": "CONSERVATIVE", "riemann": "HLL"}, "generic"),
    ("1d-cons-rusanov", (60, 1, 1), "ZEROGRADIENT", {"recon_var": "CONSERVATIVE", "riemann": "RUSANOV"}, "generic"),
    # TENO5: the cutoff is piecewise constant; quadrant states make it cut
    ("2d-teno5-hllc-quad", (32, 28, 1), "ZEROGRADIENT", {"recon": "TENO5"}, "quad"),
    ("3d-teno5-rusanov-viscous", (12, 14, 10), "PERIODIC", {"nh": 4, "recon": "TENO5", "riemann": "RUSANOV",
                                                            "viscous": True, "mu": 0.02}, "generic"),
    ("3d-char-roe-viscous-heat", (16, 12, 14), "PERIODIC", {"nh": 4, "recon_var": "CHAR-PRIMITIVE",
                                                             "frozen_state": "ROE", "viscous": True, "heat": True,
                                                             "mu": 0.02, "prandtl": 0.71}, "generic"),
    # CHAR-CONSERVATIVE: the conservative eigen-transforms of the full frozen
    # state (ROE and ARITHMETIC)
    ("2d-charcons-roe-hllc", (32, 28, 1), "PERIODIC", {"recon_var": "CHAR-CONSERVATIVE", "frozen_state": "ROE"},
     "generic"),
    ("2d-charcons-arith-hll-zg", (24, 20, 1), "ZEROGRADIENT", {"recon_var": "CHAR-CONSERVATIVE", "riemann": "HLL"},
     "generic"),
    ("3d-charcons-roe-rusanov", (12, 10, 14), "PERIODIC", {"recon_var": "CHAR-CONSERVATIVE", "frozen_state": "ROE",
                                                           "riemann": "RUSANOV"}, "generic"),
    ("2d-charcons-roe-sym-viscous", (20, 24, 1), {"east": "SYMMETRY", "west": "SYMMETRY", "north": "PERIODIC",
                                                  "south": "PERIODIC", "top": "PERIODIC", "bottom": "PERIODIC"},
     {"nh": 4, "recon_var": "CHAR-CONSERVATIVE", "frozen_state": "ROE", "viscous": True, "mu": 0.02}, "generic"),
    # Lax-Friedrichs: one speed per axis, the maximum over every face state;
    # its cotangent goes to the states attaining it (the flat parts of Sod
    # and of the square wave: many ties on both sides, and face -1/2 of the
    # periodic axis counted twice, as the reference's face arrays hold it)
    ("2d-weno-lf", (40, 36, 1), "PERIODIC", {"riemann": "LAX-FRIEDRICHS"}, "generic"),
    ("3d-weno5js-lf-zg", (12, 14, 10), "ZEROGRADIENT", {"recon": "WENO5-JS", "riemann": "LAX-FRIEDRICHS"},
     "generic"),
    ("sod-minmodad-lf", (40, 1, 1), "ZEROGRADIENT", {"nh": 4, "recon": "MINMOD-AD", "riemann": "LAX-FRIEDRICHS"},
     "sod"),
    ("1d-minmodad-lf-periodic-ties", (48, 1, 1), "PERIODIC", {"nh": 4, "recon": "MINMOD-AD",
                                                              "riemann": "LAX-FRIEDRICHS"}, "square"),
    ("2d-weno3z-lf-sym", (36, 20, 1), {"east": "SYMMETRY", "west": "SYMMETRY", "north": "PERIODIC",
                                       "south": "PERIODIC", "top": "PERIODIC", "bottom": "PERIODIC"},
     {"recon": "WENO3-Z", "riemann": "LAX-FRIEDRICHS"}, "generic"),
    ("2d-teno5-lf-viscous", (20, 16, 1), "PERIODIC", {"nh": 4, "recon": "TENO5", "riemann": "LAX-FRIEDRICHS",
                                                      "viscous": True, "mu": 0.02}, "generic"),
    ("2d-char-roe-lf", (32, 28, 1), "PERIODIC", {"recon_var": "CHAR-PRIMITIVE", "frozen_state": "ROE",
                                                 "riemann": "LAX-FRIEDRICHS"}, "generic"),
    ("3d-cons-lf-zg", (12, 10, 14), "ZEROGRADIENT", {"recon_var": "CONSERVATIVE", "riemann": "LAX-FRIEDRICHS"},
     "generic"),
    ("2d-charcons-arith-lf-zg", (24, 20, 1), "ZEROGRADIENT", {"recon_var": "CHAR-CONSERVATIVE",
                                                              "riemann": "LAX-FRIEDRICHS"}, "generic"),
    # mirror-symmetric states: the speed attained by a left and a right state
    ("1d-weno-lf-mirror", (48, 1, 1), "PERIODIC", {"riemann": "LAX-FRIEDRICHS"}, "mirror"),
    ("1d-char-roe-lf-mirror", (48, 1, 1), "PERIODIC", {"recon_var": "CHAR-PRIMITIVE", "frozen_state": "ROE",
                                                       "riemann": "LAX-FRIEDRICHS"}, "mirror"),
    ("1d-cons-lf-mirror", (48, 1, 1), "PERIODIC", {"recon_var": "CONSERVATIVE", "riemann": "LAX-FRIEDRICHS"},
     "mirror"),
    ("1d-charcons-roe-lf-mirror", (48, 1, 1), "PERIODIC", {"recon_var": "CHAR-CONSERVATIVE", "frozen_state": "ROE",
                                                           "riemann": "LAX-FRIEDRICHS"}, "mirror"),
]


@pytest.mark.parametrize("name,cells,bc,kw,kind", VJP_CASES, ids=[c[0] for c in VJP_CASES])
def test_rhs_vjp_matches_oracle_autograd(name, cells, bc, kw, kind):
    from jaxfluids_gb300.adjoint import AdjointRK3
    oc, cc = both(cells, bc, **kw)
    Ui = _interior_cons(kind, cells, oc)
    w = torch.randn(Ui.shape, generator=torch.Generator().manual_seed(11), dtype=torch.float64)
    x = Ui.clone().requires_grad_(True)
    (O.rhs_of_interior_cons(x, oc) * w).sum().backward()
    adj = AdjointRK3(cc, dt=1e-3)
    g = adj.rhs_vjp(Ui.cuda().contiguous(), w.cuda().contiguous())
    assert rel_err(g, x.grad) <= TOL


@pytest.mark.parametrize("name,cells,bc,kw,kind", VJP_CASES, ids=[c[0] for c in VJP_CASES])
def test_step_vjp_matches_oracle_autograd(name, cells, bc, kw, kind):
    from jaxfluids_gb300.adjoint import AdjointRK3
    oc, cc = both(cells, bc, **kw)
    Ui = _interior_cons(kind, cells, oc)
    dt = 0.2 * float(O.compute_dt(O.buffers_from_interior_cons(Ui, oc)[1], oc))
    lam = torch.randn(Ui.shape, generator=torch.Generator().manual_seed(12), dtype=torch.float64)
    x = Ui.clone().requires_grad_(True)
    (O.rk3_step_interior(x, torch.tensor(dt, dtype=torch.float64), oc) * lam).sum().backward()
    adj = AdjointRK3(cc, dt=dt)
    g = adj.step_vjp(Ui.cuda().contiguous(), lam.cuda().contiguous())
    assert rel_err(g, x.grad) <= TOL


def test_checkpoint_schedules_agree_and_match_oracle():
    from jaxfluids_gb300.adjoint import AdjointRK3
    oc, cc = both((40, 36, 1), "PERIODIC")
    U0 = generic_cons((40, 36, 1))
    dt = 1e-3
    n = 12
    target = torch.randn(40, 36, 1, generator=torch.Generator().manual_seed(8), dtype=torch.float64)
    adj = AdjointRK3(cc, dt=dt)
    tg = target.cuda()
    grads = []
    for sched, kw in (("uniform", {"every": n}), ("uniform", {"every": 4}),
                      ("uniform", {"every": 5, "keep_stages": False}), ("binomial", {"slots": 2}),
                      ("binomial", {"slots": 2, "leaf": 4}), ("binomial", {"slots": 0, "leaf": 3}),
                      ("binomial", {"slots": 0}), ("stored", {})):
        UN, g = adj.gradient(U0.cuda(), n, lambda U: torch.stack([U[0] - tg] + [torch.zeros_like(tg)] * 4),
                             schedule=sched, **kw)
        grads.append(g)
    for g in grads[1:]:
        assert rel_err(g, grads[0]) <= 1e-12
    x = U0.clone().requires_grad_(True)
    U = x
    for _ in range(n):
        U = O.rk3_step_interior(U, torch.tensor(dt, dtype=torch.float64), oc)
    (0.5 * ((U[0] - target) ** 2).sum()).backward()
    assert rel_err(grads[0], x.grad) <= 1e-10


def test_tutorial02_gradient_trace_on_gpu():
    """jax.value_and_grad through 200 fixed-dt steps (MINMOD-AD + Rusanov), printed by the reference."""
    from jaxfluids_gb300 import FusedRK3
    from jaxfluids_gb300.adjoint import AdjointRK3, RK3Trajectory
    g = json.load(open(os.path.join(GOLDEN, "tut02_grad.json")))
    oc, cc = both((100, 1, 1), "ZEROGRADIENT", nh=4, recon="MINMOD-AD", riemann="RUSANOV", fixed_dt=1e-3)
    U, P = O.initialize(sod_prims(100), oc)
    f = FusedRK3(cc)
    f.set_state(U[oc.interior()].contiguous().cuda())
    f.advance(200)
    rho_ref = f.primitives()[0].reshape(-1)
    x = oc.cell_centers(0).cuda()
    theta = torch.tensor(g["theta0"], dtype=torch.float64, device="cuda", requires_grad=True)
    d0 = torch.where(x < 0.5, theta[0], theta[1])
    u0 = torch.where(x < 0.5, theta[2], theta[3])
    p0 = torch.where(x < 0.5, theta[4], theta[5])
    z = torch.zeros_like(u0)
    P0 = torch.stack([d0, u0, z, z, p0]).reshape(5, 100, 1, 1)
    U0 = O.cons_from_prims(P0, 1.4)
    adj = AdjointRK3(cc, dt=1e-3)
    UN = RK3Trajectory.apply(U0, adj, 200, "uniform", 50)
    loss = torch.mean((UN[0].reshape(-1) - rho_ref) ** 2)
    loss.backward()
    assert "%.2e" % loss.item() == "%.2e" % g["loss"]
    new = (theta.detach() - g["lr"] * theta.grad).tolist()
    for a, b in zip(new, g["params_after_first_update"]):
        assert abs(a - b) <= 0.6e-8


def test_tutorial02_optimisation_trajectory_on_gpu():
    """The reference's whole gradient-descent run (976 iterations, each a
    jax.value_and_grad through 200 fixed-dt steps), printed every 25
    iterations to 3 digits (loss) and 8 decimals (parameters), replayed with
    the hand-written adjoint."""
    from jaxfluids_gb300 import FusedRK3
    from jaxfluids_gb300.adjoint import AdjointRK3, RK3Trajectory
    g = json.load(open(os.path.join(GOLDEN, "tut02_grad.json")))
    oc, cc = both((100, 1, 1), "ZEROGRADIENT", nh=4, recon="MINMOD-AD", riemann="RUSANOV", fixed_dt=1e-3)
    U, P = O.initialize(sod_prims(100), oc)
    f = FusedRK3(cc)
    f.set_state(U[oc.interior()].contiguous().cuda())
    f.advance(200)
    rho_ref = f.primitives()[0].reshape(-1)
    x = oc.cell_centers(0).cuda()
    adj = AdjointRK3(cc, dt=1e-3)
    printed = {row["itr"]: row for row in g["trajectory"]}
    theta = torch.tensor(g["theta0"], dtype=torch.float64, device="cuda")
    for itr in range(max(printed) + 1):
        th = theta.clone().requires_grad_(True)
        d0 = torch.where(x < 0.5, th[0], th[1])
        u0 = torch.where(x < 0.5, th[2], th[3])
        p0 = torch.where(x < 0.5, th[4], th[5])
        z = torch.zeros_like(u0)
        U0 = O.cons_from_prims(torch.stack([d0, u0, z, z, p0]).reshape(5, 100, 1, 1), 1.4)
        # one stored-stage leaf over the whole 200-step trajectory
        UN = RK3Trajectory.apply(U0, adj, 200, "binomial", 50, 0, 200)
        loss = torch.mean((UN[0].reshape(-1) - rho_ref) ** 2)
        loss.backward()
        lr = next(v for lim, v in g["lr_schedule"] if lim is None or itr < lim)
        theta = theta - lr * th.grad
        if itr in printed:
            row = printed[itr]
            assert "%.2e" % loss.item() == "%.2e" % row["loss"], itr
            for a, b in zip(theta.tolist(), row["params"]):
                assert abs(a - b) <= 0.6e-8, (itr, theta.tolist(), row["params"])


def test_gradient_matches_central_differences():
    from jaxfluids_gb300.adjoint import AdjointRK3
    oc, cc = both((40, 36, 1), "PERIODIC")
    U0 = generic_cons((40, 36, 1)).cuda()
    target = generic_cons((40, 36, 1), seed=8)[0].cuda()
    n, dt = 20, 2e-3
    adj = AdjointRK3(cc, dt=dt)
    loss = lambda U: 0.5 * ((U[0] - target) ** 2).sum().item()
    UN, grad = adj.gradient(U0, n, lambda U: torch.stack([U[0] - target] + [torch.zeros_like(target)] * 4),
                            schedule="uniform", every=5)
    gen = torch.Generator(device="cuda").manual_seed(4)
    for _ in range(3):
        d = torch.randn(U0.shape, generator=gen, dtype=torch.float64, device="cuda") * U0.abs()
        d[3] = 0.0  # the inactive z momentum stays identically zero
        h = 1e-6
        fd = (loss(adj.advance(U0 + h * d, n)) - loss(adj.advance(U0 - h * d, n))) / (2 * h)
        an = (grad * d).sum().item()
        # HLLC's contact sign, the Einfeldt min/max and WENO-Z's |b0 - b2| are
        # kinks; over 20 steps some sit inside the +-h stencil, so central
        # differences agree with the adjoint to ~1e-3, not to rounding.
        assert abs(fd - an) <= 2e-3 * max(abs(an), 1e-12)
