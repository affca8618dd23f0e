"""The headline workloads at their stated sizes against the oracle.

* TGV 128^3 (WENO5-Z + HLLC, PRIMITIVE, periodic): one right-hand side through
  the drop-in path (<= 1e-12 relative) and 20 fused CFL steps (<= 1e-10),
  every time step equal; and all 500 steps of the stated run against the
  oracle's C restatement.
* Viscous TGV 256^3 (Re 1600, Pr 0.71, WENO5-Z on Roe-characteristic variables
  + HLLC + CENTRAL4 viscous and heat fluxes): one right-hand side and one fused
  step against the torch oracle, 30 CFL steps against the oracle's C
  restatement, and the adjoint of the final kinetic energy with respect to the
  initial velocity (binomial checkpoints, 20 steps) against central
  differences.
* Kelvin-Helmholtz 512^2 (periodic, noise from default_rng(7)): the
  right-hand-side VJP against the oracle's autograd (<= 1e-11) and a 5-step
  fixed-dt gradient of 1/2 ||rho(T) - rho_target||^2 with respect to the
  initial v field, the workload's control (<= 1e-10).  The gradient with
  respect to rho, rho u and E is rounding-dominated on this piecewise-constant
  initial state (WENO-Z's weights on nearly flat stencils): a one-ulp change
  of the initial rho v moves the oracle's own gradient by 1.5e-3 (max norm)
  there, while its v-field gradient moves by 1.4e-11; that part is held to
  1e-2.  The forward run as stated (1000 fixed-dt steps) against the oracle's
  C restatement, bitwise.
* The same Kelvin-Helmholtz gradient as stated (1000 steps, uniform
  checkpoints every 50) against central differences in 16 random directions
  at h = 1e-6 relative.
* The batched path on four quadrant problems with sides 64, 128, 192 and 512
  (states from default_rng(1000 + i)), 10 steps, against the oracle case by
  case, and 300 steps (the batched configuration's) against the oracle's C
  restatement.

The kernels follow the reference's operation order, so the forward results are
also asserted bitwise equal.  The oracle runs on the host's cores: these tests
take a few minutes; the 256^3 one needs about 45 GB of host memory and is
skipped on a host with less available.
"""
import math

import numpy as np
import pytest
import torch

from oracle import jf_oracle as O
from tests.cases import both, quadrant_prims, rel_err, tgv_prims

pytestmark = pytest.mark.gpu
TWO_PI = ((0.0, 2 * math.pi),) * 3


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from jaxfluids_gb300 import build
    build.build()
    torch.set_num_threads(max(1, __import__("os").cpu_count() or 1))


def _available_host_bytes():
    try:
        for line in open("/proc/meminfo"):
            if line.startswith("MemAvailable:"):
                return int(line.split()[1]) * 1024
    except OSError:
        pass
    return 0


def _rhs_and_steps(oc, cc, prims, steps):
    from jaxfluids_gb300 import FusedRK3, SimulationManager
    U, P = O.initialize(prims, oc)
    ref_rhs = O.compute_rhs(U, P, oc)
    sim = SimulationManager(cc)
    rhs = sim.space_solver.compute_rhs(U.cuda(), P.cuda(), None, 0.0, 0.0)[0].euler_buffers.conservatives.cpu()
    del sim
    assert rel_err(rhs, ref_rhs) <= 1e-12
    assert torch.equal(rhs, ref_rhs)
    del rhs, ref_rhs
    inner = oc.interior()
    f = FusedRK3(cc)
    f.set_state(U[inner].contiguous().cuda(), prims=P[inner].contiguous().cuda())
    dts_gpu = [float(f.dt)]
    for _ in range(steps):
        f.advance(1)
        dts_gpu.append(float(f.dt))
    dt = O.compute_dt(P, oc)
    dts = [float(dt)]
    for _ in range(steps):
        U, P = O.rk3_step(U, P, dt, oc)
        dt = O.compute_dt(P, oc)
        dts.append(float(dt))
    cons = f.cons.cpu()
    assert dts_gpu == dts
    assert rel_err(cons, U[inner]) <= 1e-10
    assert torch.equal(cons, U[inner])


def test_tgv_128_rhs_and_20_steps():
    oc, cc = both((128, 128, 128), "PERIODIC", ranges=TWO_PI)
    _rhs_and_steps(oc, cc, tgv_prims(128), 20)


def test_tgv_128_all_500_steps_against_the_c_restatement():
    """The inviscid TGV as stated: 128^3, 500 CFL steps, every step's time step
    from the state at its start, against the oracle's plain-C restatement
    (bitwise equal to the torch oracle, tests/test_oracle_c.py; OpenMP on the
    host's cores, about two minutes on 16 cores): the final conservatives and
    time bitwise equal."""
    import ctypes
    import __graft_entry__
    from jaxfluids_gb300 import FusedRK3
    so = __graft_entry__.build_oracle_c()
    if not so:
        pytest.skip("no C compiler for the oracle's C restatement")
    f_c = ctypes.CDLL(so).jf_rk3_steps
    f_c.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.c_int,
                    ctypes.POINTER(ctypes.c_double), ctypes.c_double, ctypes.c_double, ctypes.c_double,
                    ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.c_int,
                    ctypes.POINTER(ctypes.c_double)]
    f_c.restype = ctypes.c_int
    n, steps = 128, 500
    oc, cc = both((n, n, n), "PERIODIC", ranges=TWO_PI)
    P0 = tgv_prims(n).contiguous()
    U0 = O.cons_from_prims(P0, oc.gamma).contiguous()
    f = FusedRK3(cc)
    f.set_state(U0.cuda(), prims=P0.cuda())
    f.advance(steps)
    U = U0.numpy().copy()
    P = P0.numpy().copy()
    dx = 2 * math.pi / n
    t = ctypes.c_double(0.0)
    assert f_c(U.ctypes.data, P.ctypes.data, (ctypes.c_int * 3)(n, n, n), 3,
               (ctypes.c_double * 3)(1.0 / dx, 1.0 / dx, 1.0 / dx), dx, oc.cfl, oc.gamma, O.STENCIL_EPS, 0, 0,
               (ctypes.c_int * 6)(0, 0, 0, 0, 0, 0), steps, ctypes.byref(t)) == 0
    cons = f.cons.cpu()
    assert float(f.t) == t.value
    assert rel_err(cons, torch.from_numpy(U)) <= 1e-10
    assert torch.equal(cons, torch.from_numpy(U))


def test_viscous_tgv_256_char_roe_rhs_and_one_step():
    if _available_host_bytes() < 120e9:
        pytest.skip("the oracle's 256^3 viscous step needs about 45 GB of host memory")
    oc, cc = both((256, 256, 256), "PERIODIC", ranges=TWO_PI, nh=4, recon_var="CHAR-PRIMITIVE",
                  frozen_state="ROE", viscous=True, heat=True, mu=1.0 / 1600, prandtl=0.71)
    _rhs_and_steps(oc, cc, tgv_prims(256), 1)


def test_viscous_tgv_256_30_steps_against_the_c_restatement():
    """The viscous TGV at its stated size (256^3, Re 1600, Pr 0.71, CHAR-ROE
    WENO5-Z + HLLC + CENTRAL4 viscous and heat fluxes, CFL 0.5 with the
    viscous and heat limits): 30 steps of the fused path against the oracle's
    C restatement (bitwise equal to the torch oracle, tests/test_oracle_c.py;
    OpenMP on the host's cores, a few minutes): final conservatives and time
    bitwise equal."""
    import ctypes
    import __graft_entry__
    from jaxfluids_gb300 import FusedRK3
    so = __graft_entry__.build_oracle_c()
    if not so:
        pytest.skip("no C compiler for the oracle's C restatement")
    f_c = ctypes.CDLL(so).jf_rk3_steps_visc
    f_c.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.c_int,
                    ctypes.POINTER(ctypes.c_double), ctypes.c_double, ctypes.c_double, ctypes.c_double,
                    ctypes.c_double, ctypes.c_int, ctypes.c_int] + [ctypes.c_double] * 5 + [ctypes.c_int] * 4 + \
        [ctypes.POINTER(ctypes.c_double)]
    f_c.restype = ctypes.c_int
    n, steps = 256, 30
    oc, cc = both((n, n, n), "PERIODIC", ranges=TWO_PI, nh=4, recon_var="CHAR-PRIMITIVE",
                  frozen_state="ROE", viscous=True, heat=True, mu=1.0 / 1600, prandtl=0.71)
    P0 = tgv_prims(n).contiguous()
    U0 = O.cons_from_prims(P0, oc.gamma).contiguous()
    f = FusedRK3(cc)
    f.set_state(U0.cuda(), prims=P0.cuda())
    f.advance(steps)
    cons = f.cons.cpu()
    t_gpu = float(f.t)
    del f
    U = U0.numpy().copy()
    P = P0.numpy().copy()
    dx = 2 * math.pi / n
    t = ctypes.c_double(0.0)
    assert f_c(U.ctypes.data, P.ctypes.data, (ctypes.c_int * 3)(n, n, n), oc.nh,
               (ctypes.c_double * 3)(1.0 / dx, 1.0 / dx, 1.0 / dx), dx, oc.cfl, oc.gamma, O.STENCIL_EPS, 2, 0,
               oc.mu, oc.bulk_viscosity, oc.kappa(), oc.cp(), oc.R, 1, 1, 1, steps, ctypes.byref(t)) == 0
    assert t_gpu == t.value
    assert rel_err(cons, torch.from_numpy(U)) <= 1e-10
    assert torch.equal(cons, torch.from_numpy(U))


def _kh_cons(n, seed):
    rng = np.random.default_rng(seed)
    x = (np.arange(n) + 0.5) / n
    X, Y = np.meshgrid(x, x, indexing="ij")
    inner = np.abs(Y - 0.5) < 0.25
    P = np.stack([np.where(inner, 2.0, 1.0), np.where(inner, 0.5, -0.5),
                  0.01 * np.sin(4 * np.pi * X) + rng.normal(0.0, 1e-3, X.shape), np.zeros_like(X),
                  np.full_like(X, 2.5)]).reshape(5, n, n, 1)
    return O.cons_from_prims(torch.from_numpy(P), 1.4)


def test_kh_512_rhs_vjp_and_5_step_gradient():
    from jaxfluids_gb300.adjoint import AdjointRK3
    n = 512
    oc, cc = both((n, n, 1), "PERIODIC")
    U0 = _kh_cons(n, 7)
    target = _kh_cons(n, 8)[0]
    dt = float(O.compute_dt(O.buffers_from_interior_cons(U0, oc)[1], oc))
    adj = AdjointRK3(cc, dt=dt)
    # right-hand-side VJP
    w = torch.randn(U0.shape, generator=torch.Generator().manual_seed(11), dtype=torch.float64)
    x = U0.clone().requires_grad_(True)
    (O.rhs_of_interior_cons(x, oc) * w).sum().backward()
    g = adj.rhs_vjp(U0.cuda().contiguous(), w.cuda().contiguous())
    assert rel_err(g, x.grad) <= 1e-11
    # 5-step fixed-dt gradient of 1/2 ||rho(T) - target||^2
    steps = 5
    tg = target.cuda()
    UN, grad = adj.gradient(U0.cuda(), steps, lambda U: torch.stack([U[0] - tg] + [torch.zeros_like(tg)] * 4),
                            schedule="uniform", every=2)
    x = U0.clone().requires_grad_(True)
    U = x
    for _ in range(steps):
        U = O.rk3_step_interior(U, torch.tensor(dt, dtype=torch.float64), oc)
    (0.5 * ((U[0] - target) ** 2).sum()).backward()
    assert torch.equal(UN.cpu(), U.detach())
    # d loss / d v0 = (d loss / d rho v) rho + (d loss / d E) rho v, with U = cons(P)
    dv_gpu = grad[2].cpu() * U0[0] + grad[4].cpu() * U0[2]
    dv_ref = x.grad[2] * U0[0] + x.grad[4] * U0[2]
    assert rel_err(dv_gpu[None], dv_ref[None]) <= 1e-10
    assert rel_err(grad, x.grad) <= 1e-2


def test_kh_512_adjoint_1000_steps_against_central_differences():
    """The Kelvin-Helmholtz adjoint as stated: 512^2, 1000 fixed-dt steps
    (dt the CFL 0.5 step of the initial state), uniform checkpoints every 50
    steps, loss 1/2 ||rho(T) - rho_target||^2 with the target the forward run
    from the noise of default_rng(8); its gradient with respect to the
    initial v field against central differences in 16 random directions d
    (v0 +- h d, h = 1e-6 relative: d = N(0, 1) |v0|).

    The loss is not differentiable everywhere: this initial state's density,
    x velocity and pressure are piecewise constant, and WENO-Z's |b0 - b2|,
    HLLC's contact sign and the Einfeldt speeds' min / max meet their kinks
    exactly on flat stencils, where jax.grad's conventions pick one branch
    while a central difference averages both.  The differences therefore agree
    with the adjoint to ~1e-3 of each directional derivative (measured on a
    GB300: median 1.2e-3 at h = 1e-6, the same at h = 1e-7 and 1e-8, so not a
    truncation error), and to within 1e-5 of the Cauchy-Schwarz bound
    ||grad|| ||d|| in every direction (measured at most 5.3e-6)."""
    from jaxfluids_gb300 import FusedRK3
    from jaxfluids_gb300.adjoint import AdjointRK3
    n, steps, every = 512, 1000, 50
    _, cc = both((n, n, 1), "PERIODIC")
    dev = torch.device("cuda", 0)
    gamma = 1.4

    def prims(seed):
        return O.prims_from_cons(_kh_cons(n, seed), gamma).to(dev)

    def cons(P):
        return O.cons_from_prims(P, gamma)

    P0 = prims(7)
    U0 = cons(P0)
    f = FusedRK3(cc, dev)
    f.set_state(U0)
    dt = float(f.dt)
    del f
    adj = AdjointRK3(cc, dt, dev)
    target = adj.advance(cons(prims(8)), steps)[0]

    def loss(U):
        return 0.5 * ((U[0] - target) ** 2).sum().item()

    UN, grad = adj.gradient(U0, steps, lambda U: torch.stack([U[0] - target] + [torch.zeros_like(target)] * 4),
                            schedule="uniform", every=every)
    dv = grad[2] * U0[0] + grad[4] * U0[2]
    gen = torch.Generator(device=dev).manual_seed(16)
    h = 1e-6
    rel, cs = [], []
    for _ in range(16):
        d = torch.randn(P0[2].shape, generator=gen, dtype=torch.float64, device=dev) * P0[2].abs()
        Pp, Pm = P0.clone(), P0.clone()
        Pp[2] += h * d
        Pm[2] -= h * d
        fd = (loss(adj.advance(cons(Pp), steps)) - loss(adj.advance(cons(Pm), steps))) / (2 * h)
        an = (dv * d).sum().item()
        rel.append(abs(fd - an) / abs(an))
        cs.append(abs(fd - an) / float(dv.norm() * d.norm()))
    assert max(cs) <= 1e-5, cs
    assert sorted(rel)[len(rel) // 2] <= 1e-2, rel


def test_viscous_tgv_256_adjoint_against_central_differences():
    """The viscous TGV adjoint at its stated size and form (256^3, Re 1600,
    Pr 0.71, CHAR-ROE WENO5-Z + HLLC + CENTRAL4 viscous and heat fluxes,
    fixed dt = the CFL 0.5 step of the initial state, binomial checkpoints):
    the gradient of the final kinetic energy with respect to the initial
    velocity (density and pressure held) over 20 steps, against central
    differences in 4 random directions (u0 +- h d, h = 1e-6, d = N(0, 1) per
    cell and component).  The state is smooth, so the loss is differentiable
    and the two agree to a small fraction of each directional derivative
    (measured on a GB300: at most 6.2e-6, the rounding of the 1.7e7-cell
    kinetic-energy sums over 2 h; bound 1e-4)."""
    from jaxfluids_gb300 import FusedRK3
    from jaxfluids_gb300.adjoint import AdjointRK3
    n, steps = 256, 20
    _, cc = both((n, n, n), "PERIODIC", ranges=TWO_PI, nh=4, recon_var="CHAR-PRIMITIVE",
                 frozen_state="ROE", viscous=True, heat=True, mu=1.0 / 1600, prandtl=0.71)
    dev = torch.device("cuda", 0)
    gamma = 1.4
    P0 = tgv_prims(n).to(dev)
    U0 = O.cons_from_prims(P0, gamma)
    f = FusedRK3(cc, dev)
    f.set_state(U0)
    dt = float(f.dt)
    del f
    adj = AdjointRK3(cc, dt, dev)

    def ke(U):
        return float((0.5 * (U[1:4] ** 2).sum(0) / U[0]).sum())

    def ke_grad(U):
        # dKE/d(rho u_i) = u_i, dKE/drho = -|u|^2 / 2
        u = U[1:4] / U[0]
        return torch.cat([(-0.5 * (u * u).sum(0))[None], u, torch.zeros_like(U[:1])])

    _, grad = adj.gradient(U0, steps, ke_grad, schedule="binomial", slots=2, leaf=5)
    # chain to the velocity at fixed rho and p: d(rho u_i)/du_i = rho, dE/du_i = rho u_i
    gu = torch.stack([grad[1 + i] * U0[0] + grad[4] * U0[1 + i] for i in range(3)])
    del grad
    gen = torch.Generator(device=dev).manual_seed(5)
    h = 1e-6
    rel = []
    for _ in range(4):
        d = torch.randn(gu.shape, generator=gen, dtype=torch.float64, device=dev)
        d[2] = 0.0  # w stays zero: the 3-D TGV's initial w
        Pp, Pm = P0.clone(), P0.clone()
        Pp[1:4] += h * d
        Pm[1:4] -= h * d
        fd = (ke(adj.advance(O.cons_from_prims(Pp, gamma), steps)) -
              ke(adj.advance(O.cons_from_prims(Pm, gamma), steps))) / (2 * h)
        an = float((gu * d).sum())
        rel.append(abs(fd - an) / abs(an))
    print("viscous TGV 256^3 adjoint vs central differences, relative:", rel)
    assert max(rel) <= 1e-4, rel


def test_kh_512_1000_fixed_dt_steps_against_the_c_restatement():
    """The Kelvin-Helmholtz forward run as stated (512^2, 1000 steps at the
    fixed CFL 0.5 time step of the initial state, feed-forward semantics)
    through the adjoint's forward path, against the oracle's C restatement:
    the final state bitwise equal."""
    import ctypes
    import __graft_entry__
    from jaxfluids_gb300.adjoint import AdjointRK3
    so = __graft_entry__.build_oracle_c()
    if not so:
        pytest.skip("no C compiler for the oracle's C restatement")
    f_c = ctypes.CDLL(so).jf_rk3_steps_fixed_dt
    f_c.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.c_int,
                    ctypes.POINTER(ctypes.c_double), ctypes.c_double, ctypes.c_double, ctypes.c_double,
                    ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.c_int,
                    ctypes.POINTER(ctypes.c_double)]
    f_c.restype = ctypes.c_int
    n, steps = 512, 1000
    oc, cc = both((n, n, 1), "PERIODIC")
    U0 = _kh_cons(n, 7)
    dt = float(O.compute_dt(O.buffers_from_interior_cons(U0, oc)[1], oc))
    UN = AdjointRK3(cc, dt=dt).advance(U0.cuda(), steps).cpu()
    U = U0.numpy().copy()
    P = O.prims_from_cons(U0, oc.gamma).numpy().copy()
    t = ctypes.c_double(0.0)
    assert f_c(U.ctypes.data, P.ctypes.data, (ctypes.c_int * 3)(n, n, 1), oc.nh,
               (ctypes.c_double * 3)(float(n), float(n), 0.0), dt, oc.gamma, O.STENCIL_EPS, 0, 0,
               (ctypes.c_int * 6)(0, 0, 0, 0, 0, 0), steps, ctypes.byref(t)) == 0
    assert torch.equal(UN, torch.from_numpy(U))


def test_batch_with_a_512_case_against_the_oracle():
    from jaxfluids_gb300 import BatchedRK3, CaseConfig
    sides = (64, 128, 192, 512)
    zg = {f: "ZEROGRADIENT" for f in ("east", "west", "north", "south")}
    cfgs = [CaseConfig(cells=(s, s, 1), bc=dict(zg)) for s in sides]
    states, refs = [], []
    steps = 10
    for i, s in enumerate(sides):
        oc, _ = both((s, s, 1), "ZEROGRADIENT")
        q = quadrant_prims(s, s, seed=1000 + i)
        U, P = O.initialize(q, oc)
        Ui = U[oc.interior()].contiguous()
        states.append(Ui)
        # the batch takes conservatives: its first stage reads their
        # primitives, so the oracle starts from those too
        U, P = O.buffers_from_interior_cons(Ui, oc)
        Ur, _, _, k = O.simulate(U, P, oc, end_step=steps)
        assert k == steps
        refs.append(Ur[oc.interior()])
    batch = BatchedRK3(cfgs)
    batch.set_states([u.cuda() for u in states])
    batch.advance(steps)
    torch.cuda.synchronize()
    for i in range(len(sides)):
        got = batch.case_view(i).cpu()
        assert rel_err(got, refs[i]) <= 1e-10, sides[i]
        assert torch.equal(got, refs[i]), sides[i]


def test_batch_300_steps_against_the_c_restatement():
    """The batched configuration's step count (300 CFL steps per case, each case
    its own time step) on cases of sides 64, 128, 192 and 512 (states from
    default_rng(1000 + i)), against the oracle's plain-C restatement (OpenMP)
    started from the same conservatives' primitives: every case bitwise."""
    import ctypes
    import __graft_entry__
    from jaxfluids_gb300 import BatchedRK3, CaseConfig
    so = __graft_entry__.build_oracle_c()
    if not so:
        pytest.skip("no C compiler for the oracle's C restatement")
    f_c = ctypes.CDLL(so).jf_rk3_steps
    f_c.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.c_int,
                    ctypes.POINTER(ctypes.c_double), ctypes.c_double, ctypes.c_double, ctypes.c_double,
                    ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.c_int,
                    ctypes.POINTER(ctypes.c_double)]
    f_c.restype = ctypes.c_int
    sides, steps = (64, 128, 192, 512), 300
    zg = {f: "ZEROGRADIENT" for f in ("east", "west", "north", "south")}
    cfgs = [CaseConfig(cells=(s, s, 1), bc=dict(zg)) for s in sides]
    states = []
    for i, s in enumerate(sides):
        oc, _ = both((s, s, 1), "ZEROGRADIENT")
        U, _ = O.initialize(quadrant_prims(s, s, seed=1000 + i), oc)
        states.append(U[oc.interior()].contiguous())
    batch = BatchedRK3(cfgs)
    batch.set_states([u.cuda() for u in states])
    batch.advance(steps)
    torch.cuda.synchronize()
    for i, s in enumerate(sides):
        oc, _ = both((s, s, 1), "ZEROGRADIENT")
        U = states[i].numpy().copy()
        # the batch's first stage reads the primitives of its conservatives
        P = O.prims_from_cons(states[i], oc.gamma).numpy().copy()
        dx = 1.0 / s
        t = ctypes.c_double(0.0)
        assert f_c(U.ctypes.data, P.ctypes.data, (ctypes.c_int * 3)(s, s, 1), oc.nh,
                   (ctypes.c_double * 3)(1.0 / dx, 1.0 / dx, 0.0), dx, oc.cfl, oc.gamma, O.STENCIL_EPS, 0, 0,
                   (ctypes.c_int * 6)(1, 1, 1, 1, 1, 1), steps, ctypes.byref(t)) == 0
        got = batch.case_view(i).cpu()
        assert batch.t[i].item() == t.value, s
        assert torch.equal(got, torch.from_numpy(U)), s

