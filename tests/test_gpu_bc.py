"""WALL, DIRICHLET and NEUMANN boundaries (halos/outer/material.py:473-866) and
the edge halos of the dissipative fluxes (:289-379), with CENTRAL4 and CENTRAL2
dissipative stencils, on the CUDA path against
the oracle: right-hand side bitwise, halo buffers bitwise, RK3 steps through
the drop-in and fused paths, and the adjoint (viscous and inviscid)."""
import math

import pytest
import torch

from oracle import jf_oracle as O
from tests.cases import both, generic_cons, quadrant_prims, rel_err, sod_prims, tgv_prims

pytestmark = pytest.mark.gpu

RHS_TOL = 1e-12
STEP_TOL = 1e-10


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from jaxfluids_gb300 import build
    build.build()


def _faces(x=None, y=None, z=None):
    bc = {}
    for (lo, hi), t in ((("west", "east"), x), (("south", "north"), y), (("bottom", "top"), z)):
        if t is None:
            t = ("PERIODIC", "PERIODIC")
        bc[lo], bc[hi] = t
    return bc


IN_STATE = (1.2, 0.3, 0.1, 0.0, 1.1)
# double Mach reflection: post-shock state of the Mach 10 shock
POST_SHOCK = (8.0, 7.144709581221618, -4.125, 0.0, 116.5)
GRAD = (0.1, -0.2, 0.05, 0.0, 0.3)
VISC = {"nh": 4, "viscous": True, "heat": True, "mu": 0.02, "prandtl": 0.71}

# (name, cells, bc, bc_values, scheme keywords, initial condition)
BC_CASES = [
    ("1d-dirichlet-neumann", (100, 1, 1), _faces(x=("DIRICHLET", "NEUMANN")),
     {"west": (1.0, 0.0, 0.0, 0.0, 1.0), "east": GRAD}, {}, "sod"),
    ("2d-dirichlet-neumann-wall", (40, 32, 1), _faces(x=("DIRICHLET", "NEUMANN"), y=("WALL", "WALL")),
     {"west": IN_STATE, "east": GRAD, "south": (0.0, 0.0, 0.0), "north": (0.4, 0.0, 0.0)}, {}, "quad"),
    ("2d-wall-sym-minmod-rusanov", (36, 28, 1), _faces(x=("WALL", "WALL"), y=("SYMMETRY", "SYMMETRY")),
     {"west": (0.0, 0.2, 0.0), "east": (0.0, -0.1, 0.0)}, {"nh": 4, "recon": "MINMOD", "riemann": "RUSANOV"},
     "quad"),
    ("2d-char-roe-dirichlet-wall", (32, 36, 1), _faces(x=("NEUMANN", "DIRICHLET"), y=("WALL", "ZEROGRADIENT")),
     {"west": GRAD, "east": IN_STATE, "south": (0.1, 0.0, 0.0)},
     {"recon_var": "CHAR-PRIMITIVE", "frozen_state": "ROE"}, "quad"),
    ("2d-cavity-viscous-heat", (32, 32, 1), _faces(x=("WALL", "WALL"), y=("WALL", "WALL")),
     {"west": (0.0, 0.0, 0.0), "east": (0.0, 0.0, 0.0), "south": (0.0, 0.0, 0.0), "north": (0.5, 0.0, 0.0)},
     dict(VISC), "quad"),
    ("3d-viscous-periodic-wall-zg", (16, 12, 14), _faces(y=("WALL", "WALL"), z=("ZEROGRADIENT", "ZEROGRADIENT")),
     {"south": (0.0, 0.0, 0.0), "north": (0.3, 0.0, 0.1)}, dict(VISC), "tgv"),
    ("3d-char-roe-viscous-sym-neumann-dirichlet-wall", (12, 14, 16),
     _faces(x=("SYMMETRY", "SYMMETRY"), y=("NEUMANN", "DIRICHLET"), z=("WALL", "WALL")),
     {"south": GRAD, "north": (1.0, 0.1, 0.0, 0.05, 72.0), "bottom": (0.0, 0.0, 0.0), "top": (0.2, -0.1, 0.0)},
     dict(VISC, recon_var="CHAR-PRIMITIVE", frozen_state="ROE", mu=1.0 / 1600), "tgv"),
    ("3d-viscous-noheatprod-wall-neumann", (14, 12, 12),
     _faces(x=("WALL", "NEUMANN"), y=("ZEROGRADIENT", "WALL"), z=("SYMMETRY", "SYMMETRY")),
     {"west": (0.0, 0.1, 0.0), "east": GRAD, "north": (0.2, 0.0, 0.0)},
     dict(VISC, viscous_heat_production=False), "tgv"),
    # CENTRAL2 dissipative stencils (reconstruction, centre and face derivative)
    ("2d-cavity-viscous-heat-central2", (30, 26, 1), _faces(x=("WALL", "WALL"), y=("WALL", "WALL")),
     {"west": (0.0, 0.0, 0.0), "east": (0.0, 0.0, 0.0), "south": (0.0, 0.0, 0.0), "north": (0.5, 0.0, 0.0)},
     dict(VISC, nh=3, diss_recon="CENTRAL2", diss_deriv_center="CENTRAL2", diss_deriv_face="CENTRAL2"), "quad"),
    ("3d-viscous-mixed-stencils-wall-neumann", (14, 12, 10),
     _faces(y=("WALL", "NEUMANN"), z=("ZEROGRADIENT", "SYMMETRY")),
     {"south": (0.2, 0.0, -0.1), "north": GRAD},
     dict(VISC, nh=3, diss_recon="CENTRAL2", diss_deriv_center="CENTRAL4", diss_deriv_face="CENTRAL2"), "tgv"),
    ("3d-char-roe-viscous-c4recon-c2deriv", (12, 12, 12), _faces(x=("WALL", "DIRICHLET")),
     {"west": (0.0, 0.0, 0.1), "east": (1.0, 0.1, 0.0, 0.05, 72.0)},
     dict(VISC, recon_var="CHAR-PRIMITIVE", frozen_state="ROE", diss_recon="CENTRAL4", diss_deriv_center="CENTRAL2",
          diss_deriv_face="CENTRAL4"), "tgv"),
    # dissipative fluxes beside the other reconstructions (lid-driven cavity:
    # WENO5-JS + HLLC + CENTRAL4 viscous, no heat production)
    ("2d-cavity-weno5js-viscous", (28, 30, 1), _faces(x=("WALL", "WALL"), y=("WALL", "WALL")),
     {"west": (0.0, 0.0, 0.0), "east": (0.0, 0.0, 0.0), "south": (0.0, 0.0, 0.0), "north": (0.5, 0.0, 0.0)},
     dict(nh=4, recon="WENO5-JS", viscous=True, mu=0.01, viscous_heat_production=False), "quad"),
    ("3d-weno3z-rusanov-viscous-heat", (12, 10, 14), _faces(y=("WALL", "ZEROGRADIENT")),
     {"south": (0.1, 0.0, 0.0)}, dict(VISC, recon="WENO3-Z", riemann="RUSANOV"), "tgv"),
    ("2d-minmod-ad-hll-viscous-heat-c2", (26, 24, 1), _faces(x=("DIRICHLET", "NEUMANN"), y=("SYMMETRY", "WALL")),
     {"west": IN_STATE, "east": GRAD, "north": (0.2, 0.0, 0.0)},
     dict(VISC, nh=3, recon="MINMOD-AD", riemann="HLL", diss_recon="CENTRAL2", diss_deriv_center="CENTRAL2",
          diss_deriv_face="CENTRAL2"), "quad"),
    # no convective flux (active_physics.is_convective_flux = false): Couette
    # flow, and heat conduction alone with a constant CUSTOM conductivity
    ("2d-couette-viscous-only", (16, 24, 1), _faces(y=("WALL", "WALL")),
     {"south": (0.0, 0.0, 0.0), "north": (0.1, 0.0, 0.0)},
     dict(nh=4, recon="WENO5-JS", viscous=True, mu=0.1, convective=False), "quad"),
    ("1d-heat-only-dirichlet", (64, 1, 1), _faces(x=("DIRICHLET", "DIRICHLET")),
     {"west": (1.0, 0.0, 0.0, 0.0, 1.0), "east": (0.5, 0.0, 0.0, 0.0, 1.0)},
     dict(nh=4, recon="WENO5-JS", heat=True, kappa=0.1, convective=False), "sod"),
    ("3d-heat-viscous-only-c2", (10, 12, 8), _faces(x=("DIRICHLET", "WALL"), z=("NEUMANN", "ZEROGRADIENT")),
     {"west": (1.0, 0.0, 0.1, 0.0, 1.2), "east": (0.0, 0.1, 0.0), "bottom": GRAD},
     dict(VISC, nh=3, convective=False, diss_recon="CENTRAL2", diss_deriv_center="CENTRAL2",
          diss_deriv_face="CENTRAL4"), "tgv"),
    # boundary values varying along a face (callables of the boundary
    # coordinates) and faces of several types (bounding_domain masks)
    ("2d-heat-equation-sine-dirichlet", (24, 20, 1), _faces(x=("DIRICHLET", "DIRICHLET"), y=("DIRICHLET", "DIRICHLET")),
     {"west": (1.0, 0.0, 0.0, 0.0, 1.0), "east": (1.0, 0.0, 0.0, 0.0, 1.0), "south": (1.0, 0.0, 0.0, 0.0, 1.0),
      "north": (1.0, 0.0, 0.0, 0.0, "lambda x,t: 1.0 + jnp.sin(jnp.pi * x)")},
     dict(nh=4, recon="WENO5-JS", heat=True, kappa=0.1, convective=False), "quad"),
    ("2d-double-mach-mixed-south", (48, 12, 1),
     _faces(x=("DIRICHLET", "ZEROGRADIENT"),
            y=([("DIRICHLET", POST_SHOCK, "lambda x: x < 1.0 / 6.0"),
                ("SYMMETRY", None, "lambda x: x >= 1.0 / 6.0")], "ZEROGRADIENT")),
     {"west": POST_SHOCK}, dict(ranges=((0.0, 4.0), (0.0, 1.0), (0.0, 1.0)), interpolation_limiter=True), "dmr"),
    ("3d-viscous-mixed-wall-neumann-fields", (12, 10, 8),
     _faces(y=([("WALL", ("lambda x,z,t: 0.1 * jnp.sin(2 * jnp.pi * x)", 0.0, "lambda x,z,t: 0.05 * z"),
                 "lambda x,z: x < 0.5"),
                ("NEUMANN", GRAD, "lambda x,z: x >= 0.5")], ("WALL")),
            z=("DIRICHLET", "ZEROGRADIENT")),
     {"north": ("lambda x,z,t: 0.2 + 0.05 * z", 0.0, 0.0),
      "bottom": ("lambda x,y,t: 1.0 + 0.1 * x * y", 0.05, 0.0, 0.0, 1.1)}, dict(VISC), "tgv"),
    ("2d-char-roe-neumann-wall-fields", (30, 28, 1),
     _faces(x=("SYMMETRY", "NEUMANN"), y=("ZEROGRADIENT", "WALL")),
     {"east": (0.0, "lambda y,t: 0.2 * y", 0.0, 0.0, "lambda y,t: -0.1 + 0.3 * y * y"),
      "north": ("lambda x,t: 0.3 * x * (1.0 - x)", 0.0, 0.0)},
     {"recon_var": "CHAR-PRIMITIVE", "frozen_state": "ROE"}, "quad"),
    # conservative reconstructions: halo conservatives are those of the halo
    # primitives (material.py:248-250)
    ("2d-charcons-roe-wall-dirichlet-limiter", (32, 30, 1), _faces(x=("WALL", "DIRICHLET"), y=("SYMMETRY", "NEUMANN")),
     {"west": (0.0, 0.1, 0.0), "east": IN_STATE, "north": GRAD},
     dict(recon_var="CHAR-CONSERVATIVE", frozen_state="ROE", interpolation_limiter=True), "quad"),
    ("3d-cons-viscous-wall", (12, 10, 14), _faces(y=("WALL", "WALL")), {"south": (0.0, 0.0, 0.0), "north": (0.2, 0.0, 0.0)},
     dict(VISC, recon_var="CONSERVATIVE"), "tgv"),
    # gravity (active_physics.is_volume_force): Rayleigh-Taylor-like walls of
    # fixed states, and a 3-D viscous case with every component
    ("2d-rayleigh-taylor-gravity", (16, 40, 1), _faces(x=("SYMMETRY", "SYMMETRY"), y=("DIRICHLET", "DIRICHLET")),
     {"south": (2.0, 0.0, 0.0, 0.0, 1.0), "north": (1.0, 0.0, 0.0, 0.0, 2.5)},
     dict(gravity=(0.0, 1.0, 0.0), ranges=((0.0, 0.25), (0.0, 1.0), (0.0, 1.0))), "quad"),
    ("3d-viscous-gravity-wall", (10, 12, 8), _faces(y=("WALL", "WALL")),
     {"south": (0.0, 0.0, 0.0), "north": (0.1, 0.0, 0.0)}, dict(VISC, gravity=(0.3, -0.5, 0.2)), "tgv"),
]


def _dmr_prims(cells, ranges=((0.0, 4.0), (0.0, 1.0))):
    """Mach 10 shock at 60 degrees through x = 1/6 (the double Mach
    reflection's initial condition)."""
    x = [torch.linspace(lo + (hi - lo) / n / 2, hi - (hi - lo) / n / 2, n, dtype=torch.float64)
         for (lo, hi), n in zip(ranges, cells[:2])]
    X, Y = torch.meshgrid(x[0], x[1], indexing="ij")
    post = Y > math.sqrt(3.0) * (X - 1.0 / 6.0)
    P = torch.zeros(5, cells[0], cells[1], 1, dtype=torch.float64)
    for v, (a, b) in enumerate(zip(POST_SHOCK, (1.4, 0.0, 0.0, 0.0, 1.0))):
        P[v, :, :, 0] = torch.where(post, torch.full_like(X, a), torch.full_like(X, b))
    return P


def _prims(kind, cells):
    if kind == "dmr":
        return _dmr_prims(cells)
    if kind == "sod":
        return sod_prims(cells[0])
    if kind == "quad":
        return quadrant_prims(cells[0], cells[1], seed=cells[0] + 1)
    n = max(cells)
    full = tgv_prims(n)
    return full[:, :cells[0], :cells[1], :cells[2]].contiguous()


def _case(name):
    for c in BC_CASES:
        if c[0] == name:
            return c
    raise KeyError(name)


IDS = [c[0] for c in BC_CASES]


@pytest.mark.parametrize("name", IDS)
def test_bc_rhs_bitwise(name):
    from jaxfluids_gb300 import SimulationManager
    _, cells, bc, vals, kw, kind = _case(name)
    oc, cc = both(cells, bc, bc_values=vals, **kw)
    U, P = O.initialize(_prims(kind, cells), oc)
    ref = O.compute_rhs(U, P, oc)
    sim = SimulationManager(cc)
    rhs = sim.space_solver.compute_rhs(U.cuda(), P.cuda(), None, 0.0, 0.0)[0].euler_buffers.conservatives
    assert rel_err(rhs, ref) <= RHS_TOL
    assert torch.equal(rhs.cpu(), ref)


@pytest.mark.parametrize("name", IDS)
def test_bc_halo_fill_bitwise(name):
    """Face halos of every face (and edge halos of the dissipative cases)."""
    from jaxfluids_gb300 import SimulationManager
    _, cells, bc, vals, kw, kind = _case(name)
    oc, cc = both(cells, bc, bc_values=vals, **kw)
    prims = _prims(kind, cells)
    U, P = O.initialize(prims, oc)
    Ug, Pg = SimulationManager(cc).initialize(prims.cuda())
    assert torch.equal(Pg.cpu(), P)
    assert torch.equal(Ug.cpu(), U)


@pytest.mark.parametrize("fused", [False, True], ids=["drop-in", "fused"])
@pytest.mark.parametrize("name", IDS)
def test_bc_steps(name, fused):
    from jaxfluids_gb300 import FusedRK3, SimulationManager
    _, cells, bc, vals, kw, kind = _case(name)
    oc, cc = both(cells, bc, bc_values=vals, **kw)
    U, P = O.initialize(_prims(kind, cells), oc)
    steps = 5
    Ur, Pr = U, P
    for _ in range(steps):
        Ur, Pr = O.rk3_step(Ur, Pr, O.compute_dt(Pr, oc), oc)
    inner = oc.interior()
    if fused:
        f = FusedRK3(cc)
        f.set_state(U[inner].contiguous().cuda())
        f.advance(steps)
        out = f.cons
    else:
        sim = SimulationManager(cc)
        Ug, Pg = U.cuda(), P.cuda()
        for _ in range(steps):
            Ug, Pg = sim.do_integration_step(Ug, Pg, sim.compute_time_step_size(Pg))
        out = Ug[inner]
    assert rel_err(out, Ur[inner]) <= STEP_TOL


ADJ_CASES = IDS


@pytest.mark.parametrize("name", ADJ_CASES)
def test_bc_rhs_vjp_matches_oracle_autograd(name):
    from jaxfluids_gb300.adjoint import AdjointRK3
    _, cells, bc, vals, kw, kind = _case(name)
    oc, cc = both(cells, bc, bc_values=vals, **kw)
    # smooth random-phase fields: WENO-Z's derivative amplifies rounding by
    # up to 1/eps where stencils are flat, e.g. zero-gradient halos of a
    # piecewise-constant state, so the comparison uses fields with none
    Ui = generic_cons(cells, seed=3)
    w = torch.randn(Ui.shape, generator=torch.Generator().manual_seed(22), dtype=torch.float64)
    x = Ui.clone().requires_grad_(True)
    (O.rhs_of_interior_cons(x, oc) * w).sum().backward()
    adj = AdjointRK3(cc, dt=1e-3)
    gv = adj.rhs_vjp(Ui.cuda().contiguous(), w.cuda().contiguous())
    assert rel_err(gv, x.grad) <= 1e-11


@pytest.mark.parametrize("name", ["2d-cavity-viscous-heat", "3d-char-roe-viscous-sym-neumann-dirichlet-wall",
                                  "2d-cavity-viscous-heat-central2", "3d-viscous-mixed-stencils-wall-neumann",
                                  "2d-cavity-weno5js-viscous", "2d-couette-viscous-only",
                                  "3d-heat-viscous-only-c2", "2d-heat-equation-sine-dirichlet",
                                  "3d-viscous-mixed-wall-neumann-fields", "2d-rayleigh-taylor-gravity",
                                  "3d-viscous-gravity-wall", "3d-cons-viscous-wall"])
def test_bc_step_vjp_matches_oracle_autograd(name):
    from jaxfluids_gb300.adjoint import AdjointRK3
    _, cells, bc, vals, kw, kind = _case(name)
    oc, cc = both(cells, bc, bc_values=vals, **kw)
    Ui = generic_cons(cells, seed=4)
    dt = 0.2 * float(O.compute_dt(O.buffers_from_interior_cons(Ui, oc)[1], oc))
    lam = torch.randn(Ui.shape, generator=torch.Generator().manual_seed(23), dtype=torch.float64)
    if cells[2] == 1:
        lam[3] = 0.0
    x = Ui.clone().requires_grad_(True)
    (O.rk3_step_interior(x, torch.tensor(dt, dtype=torch.float64), oc) * lam).sum().backward()
    adj = AdjointRK3(cc, dt=dt)
    g = adj.step_vjp(Ui.cuda().contiguous(), lam.cuda().contiguous())
    assert rel_err(g, x.grad) <= 1e-11


def test_time_varying_boundary_values_drop_in_steps():
    """DIRICHLET and WALL values that are functions of time, filled at each
    stage's time t + dt (1, 1/2, 1) (simulation_manager.py:855-857), through
    the drop-in stage loop; 4 steps against the oracle."""
    from jaxfluids_gb300 import SimulationManager
    cells = (32, 28, 1)
    bc = _faces(x=("DIRICHLET", "ZEROGRADIENT"), y=("WALL", "WALL"))
    vals = {"west": (1.2, "lambda y,t: 0.3 + 2.0 * t * y", 0.0, 0.0, "lambda y,t: 1.1 + 5.0 * t"),
            "south": (0.0, 0.0, 0.0), "north": ("lambda x,t: 0.4 * jnp.sin(20.0 * t) * x", 0.0, 0.0)}
    oc, cc = both(cells, bc, bc_values=vals, nh=4, viscous=True, heat=True, mu=0.02, prandtl=0.71)
    assert cc.time_varying_faces == ["north", "west"]
    U, P = O.initialize(_prims("quad", cells), oc)
    sim = SimulationManager(cc)
    Ug, Pg = sim.initialize(_prims("quad", cells).cuda())
    assert torch.equal(Pg.cpu(), P)
    t = 0.0
    for _ in range(4):
        dt = O.compute_dt(P, oc)
        U, P = O.rk3_step(U, P, dt, oc, t)
        Ug, Pg = sim.do_integration_step(Ug, Pg, dt.cuda(), t)
        t += float(dt)
    assert rel_err(Ug[oc.interior()], U[oc.interior()]) <= STEP_TOL
    assert torch.equal(Pg.cpu()[oc.interior()], P[oc.interior()])
