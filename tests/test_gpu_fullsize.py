"""The headline workloads at their full sizes, checked through properties that
hold at any size (tests/test_gpu_headline.py compares the same sizes with the
oracle directly):

* 3-D inviscid Taylor-Green vortex, 128^3 periodic (WENO5-Z + HLLC, RK3 at CFL
  0.5) and 3-D viscous Taylor-Green vortex, 256^3 periodic (WENO5-Z on the
  ROE characteristic variables + HLLC + CENTRAL4 viscous and heat fluxes, Re
  1600, Pr 0.71): the reflection x <-> y (cells (i, j, k) -> (j, i, k), u <->
  v) commutes with the fused steps, and the periodic finite-volume update
  conserves mass, momentum and energy to rounding;
* the same TGV 128^3 through the reference-facing drop-in (halo buffers,
  SimulationManager.do_integration_step) equals the fused path bitwise;
* 2-D four-quadrant Riemann problems with the batch's grid sides
  {64, 128, 192, 256, 384, 512}: the batched steps equal single-case steps;
* adjoint of the 2-D Kelvin-Helmholtz case at 512^2: the gradient is linear
  in the final-state cotangent and does not depend on the checkpoint schedule;
* 1-D Sod, 200 cells, to t = 0.2 (176 steps): the CUDA path against the
  oracle step for step.
"""
import math

import numpy as np
import pytest
import torch

from oracle import jf_oracle as O
from tests.cases import assert_conserved, both, quadrant_prims, reflect_xy, rel_err, sod_prims, tgv_prims

pytestmark = pytest.mark.gpu

# RK3 steps of the same data in another cell order: the per-cell arithmetic is
# the same up to the order of commutative additions, so the states agree to
# rounding (equal in practice); 1e-12 relative per variable.
REFLECT_TOL = 1e-12
# change of a domain total over the steps, relative to the total of |U|
CONSERVE_TOL = 1e-12


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from jaxfluids_gb300 import build
    build.build()


def _tgv_cons(n, device="cuda"):
    return O.cons_from_prims(tgv_prims(n), 1.4).to(device)


def _reflection_and_conservation(cells, steps, **kw):
    from jaxfluids_gb300 import FusedRK3
    assert cells[0] == cells[1]
    _, cc = both(cells, "PERIODIC", ranges=((0, 2 * math.pi),) * 3, **kw)
    U0 = _tgv_cons(cells[0])
    a = FusedRK3(cc)
    a.set_state(U0)
    a.advance(steps)
    b = FusedRK3(cc)
    b.set_state(reflect_xy(U0))
    b.advance(steps)
    torch.cuda.synchronize()
    assert torch.isfinite(a.cons).all()
    for x, y in ((a.t.item(), b.t.item()), (a.dt.item(), b.dt.item())):
        assert abs(x - y) <= 1e-14 * abs(x)
    assert rel_err(reflect_xy(a.cons), b.cons) <= REFLECT_TOL
    assert_conserved(U0, a.cons, CONSERVE_TOL)
    return a


def test_tgv128_reflection_and_conservation():
    a = _reflection_and_conservation((128, 128, 128), 20)
    assert a.t.item() > 0


def test_viscous_tgv256_char_roe_reflection_and_conservation():
    _reflection_and_conservation((256, 256, 256), 3, nh=4, recon_var="CHAR-PRIMITIVE", frozen_state="ROE",
                                 viscous=True, heat=True, mu=1.0 / 1600, prandtl=0.71)


def test_tgv128_dropin_equals_fused():
    """Two steps through the halo-buffer drop-in (the reference's
    SimulationManager.do_integration_step interface) and through the fused
    path, both starting from the initial primitives as the reference does:
    equal bitwise (and within 1e-10 relative per variable, the bound after
    steps), time steps and time equal."""
    from jaxfluids_gb300 import FusedRK3, SimulationManager
    cells = (128, 128, 128)
    oc, cc = both(cells, "PERIODIC", ranges=((0, 2 * math.pi),) * 3)
    U, P = O.initialize(tgv_prims(128), oc)
    inner = oc.interior()
    f = FusedRK3(cc)
    f.set_state(U[inner].contiguous().cuda(), prims=P[inner].contiguous().cuda())
    f.advance(2)
    sim = SimulationManager(cc)
    Ug, Pg = U.cuda(), P.cuda()
    t = 0.0
    for _ in range(2):
        dt = sim.compute_time_step_size(Pg)
        Ug, Pg = sim.do_integration_step(Ug, Pg, dt)
        t += float(dt)
    torch.cuda.synchronize()
    assert rel_err(Ug[inner], f.cons) <= 1e-10
    assert torch.equal(Ug[inner], f.cons)
    assert t == f.t.item()


# the batch workload's grid sides, each once on x and once on y
BATCH_SIDES = [(512, 64), (384, 192), (256, 256), (128, 512), (64, 384), (192, 128)]


def test_batch_full_sides_equal_single_cases():
    from jaxfluids_gb300 import BatchedRK3, CaseConfig, FusedRK3
    cfgs = [CaseConfig(cells=(a, b, 1), bc={f: "ZEROGRADIENT" for f in ("east", "west", "north", "south")})
            for a, b in BATCH_SIDES]
    states = []
    for i, (a, b) in enumerate(BATCH_SIDES):
        q = quadrant_prims(a, b, seed=500 + i)
        states.append(O.cons_from_prims(torch.stack([q[0], q[1], q[2], torch.zeros_like(q[0]), q[3]]), 1.4).cuda())
    batch = BatchedRK3(cfgs)
    batch.set_states(states)
    batch.advance(5)
    for i, c in enumerate(cfgs):
        f = FusedRK3(c)
        f.set_state(states[i])
        f.advance(5)
        torch.cuda.synchronize()
        assert torch.equal(batch.case_view(i), f.cons), BATCH_SIDES[i]
        assert batch.dt[i].item() == f.dt.item() and batch.t[i].item() == f.t.item()


def _kh_cons(n, seed):
    """2-D Kelvin-Helmholtz on [0, 1]^2: rho = 2, u = 0.5 for |y - 0.5| < 0.25,
    else rho = 1, u = -0.5; p = 2.5; v = 0.01 sin(4 pi x) + N(0, 1e-3)."""
    rng = np.random.default_rng(seed)
    x = (np.arange(n) + 0.5) / n
    X, Y = np.meshgrid(x, x, indexing="ij")
    inner = np.abs(Y - 0.5) < 0.25
    rho = np.where(inner, 2.0, 1.0)
    u = np.where(inner, 0.5, -0.5)
    v = 0.01 * np.sin(4 * np.pi * X) + rng.normal(0.0, 1e-3, X.shape)
    P = np.stack([rho, u, v, np.zeros_like(rho), np.full_like(X, 2.5)]).reshape(5, n, n, 1)
    return O.cons_from_prims(torch.from_numpy(P), 1.4)


def test_kh512_gradient_linear_and_schedule_independent():
    from jaxfluids_gb300 import CaseConfig, FusedRK3
    from jaxfluids_gb300.adjoint import AdjointRK3
    n, steps = 512, 20
    cfg = CaseConfig(cells=(n, n, 1), bc={f: "PERIODIC" for f in ("east", "west", "north", "south")}, cfl=0.5)
    U0 = _kh_cons(n, 7).cuda()
    f = FusedRK3(cfg)
    f.set_state(U0)
    adj = AdjointRK3(cfg, float(f.dt))
    gen = torch.Generator(device="cuda").manual_seed(11)
    W1 = torch.randn(U0.shape, generator=gen, dtype=torch.float64, device="cuda")
    W2 = torch.randn(U0.shape, generator=gen, dtype=torch.float64, device="cuda")
    W1[3] = 0.0
    W2[3] = 0.0
    a, b = 0.75, -1.25
    _, g1 = adj.gradient(U0, steps, lambda U: W1, schedule="uniform", every=5)
    _, g2 = adj.gradient(U0, steps, lambda U: W2, schedule="uniform", every=5)
    UN, g12 = adj.gradient(U0, steps, lambda U: a * W1 + b * W2, schedule="uniform", every=5)
    assert torch.isfinite(g12).all()
    assert rel_err(g12, a * g1 + b * g2) <= 1e-11
    for sched, kw in (("binomial", {"slots": 2}), ("uniform", {"every": steps, "keep_stages": False})):
        UNs, gs = adj.gradient(U0, steps, lambda U: W1, schedule=sched, **kw)
        assert torch.equal(UNs, UN)
        assert rel_err(gs, g1) <= 1e-12
    assert_conserved(U0, UN, CONSERVE_TOL)


def test_sod200_to_end_time_matches_oracle():
    """1-D Sod, 200 cells, WENO5-Z + HLLC, CFL 0.5, zero-gradient: every RK3
    step until t >= 0.2 against the oracle (1e-10 relative at the end)."""
    from jaxfluids_gb300 import FusedRK3
    oc, cc = both((200, 1, 1), "ZEROGRADIENT", cfl=0.5)
    U, P = O.initialize(sod_prims(200), oc)
    Ur, Pr, t, steps = U, P, 0.0, 0
    while t < 0.2:
        dt = O.compute_dt(Pr, oc)
        Ur, Pr = O.rk3_step(Ur, Pr, dt, oc)
        t += dt.item()
        steps += 1
    inner = oc.interior()
    f = FusedRK3(cc)
    f.set_state(U[inner].contiguous().cuda(), prims=P[inner].contiguous().cuda())
    f.advance(steps)
    torch.cuda.synchronize()
    assert steps == 176  # the reference's own run of this case (tests/golden/ref/sod.npz)
    assert rel_err(f.cons, Ur[inner]) <= 1e-10
    assert torch.equal(f.cons.cpu(), Ur[inner])
    assert f.t.item() == t
