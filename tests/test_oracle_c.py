"""Two independent CPU restatements of the reference agree bitwise: the plain-C
right-hand side (oracle/jf_rhs.c: WENO5-Z on primitives or on their
characteristic variables with the ARITHMETIC or ROE frozen state, HLLC with
Einfeldt speeds, HLL or Rusanov) against the torch oracle, on periodic, zero-gradient and symmetry
halos in 1-D to 3-D, each side filling its own halos from the same interior;
and with CENTRAL4 viscous and heat fluxes on periodic boxes, the right-hand
side and RK3 steps under each of the three time-step limits.
Built here with the system C compiler, contraction off."""
import ctypes
import os

import numpy as np
import pytest
import torch

from oracle import jf_oracle as O
from tests.cases import both, quadrant_prims, sod_prims, tgv_prims

BC = {"PERIODIC": 0, "ZEROGRADIENT": 1, "SYMMETRY": 2}
FACE_ORDER = ("west", "east", "south", "north", "bottom", "top")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def crhs():
    import __graft_entry__
    so = __graft_entry__.build_oracle_c()  # oracle/_build/jf_rhs.so, rebuilt when the source is newer
    if not so:
        pytest.skip("no C compiler")
    lib = ctypes.CDLL(so)
    f = lib.jf_rhs_weno5z
    f.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                  ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


@pytest.fixture(scope="module")
def halos(crhs):
    import __graft_entry__
    f = ctypes.CDLL(__graft_entry__.build_oracle_c()).jf_fill_face_halos
    f.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    f.restype = ctypes.c_int
    return f


CASES = [
    ("sod-1d", (120, 1, 1), "ZEROGRADIENT", "sod"),
    ("quad-2d-sym", (36, 28, 1), {"east": "ZEROGRADIENT", "west": "ZEROGRADIENT", "north": "SYMMETRY",
                                  "south": "SYMMETRY", "top": "PERIODIC", "bottom": "PERIODIC"}, "quad"),
    ("tgv-3d", (16, 12, 14), "PERIODIC", "tgv"),
]


MODES = {0: {}, 1: dict(recon_var="CHAR-PRIMITIVE", frozen_state="ARITHMETIC"),
         2: dict(recon_var="CHAR-PRIMITIVE", frozen_state="ROE")}


RIEMANN = {0: "HLLC", 1: "RUSANOV", 2: "HLL"}


@pytest.mark.parametrize("riemann", list(RIEMANN), ids=[v.lower() for v in RIEMANN.values()])
@pytest.mark.parametrize("mode", list(MODES), ids=["primitive", "char-arithmetic", "char-roe"])
@pytest.mark.parametrize("name,cells,bc,kind", CASES, ids=[c[0] for c in CASES])
def test_c_restatement_matches_torch_oracle(crhs, halos, name, cells, bc, kind, mode, riemann):
    oc, _ = both(cells, bc, riemann=RIEMANN[riemann], **MODES[mode])
    if kind == "sod":
        prims = sod_prims(cells[0])
    elif kind == "quad":
        prims = quadrant_prims(cells[0], cells[1], seed=4)
    else:
        prims = tgv_prims(max(cells))[:, :cells[0], :cells[1], :cells[2]].contiguous()
    U, P = O.initialize(prims, oc)
    ref = O.compute_rhs(U, P, oc)
    # the C side fills its own face halos from the interior
    Pn = np.zeros(P.shape, dtype=np.float64)
    Pn[(slice(None),) + oc.interior()[1:]] = P[oc.interior()].numpy()
    codes = (ctypes.c_int * 6)(*[BC[oc.bc[f]] for f in FACE_ORDER])
    assert halos(Pn.ctypes.data, (ctypes.c_int * 3)(*cells), oc.nh, codes) == 0
    for a in range(3):
        if cells[a] > 1:
            face_rows = [slice(None)] + [slice(None) if b == a else oc.interior()[b + 1] for b in range(3)]
            assert np.array_equal(Pn[tuple(face_rows)], P[tuple(face_rows)].numpy()), a
    out = np.empty(ref.shape, dtype=np.float64)
    n = (ctypes.c_int * 3)(*cells)
    odx = (ctypes.c_double * 3)(*[oc.one_cell_size(a) if cells[a] > 1 else 0.0 for a in range(3)])
    assert crhs(Pn.ctypes.data, n, oc.nh, odx, oc.gamma, O.STENCIL_EPS, mode, riemann, out.ctypes.data) == 0
    assert torch.equal(torch.from_numpy(out), ref)


def test_oracle_sqrt_is_correctly_rounded():
    """The oracle's square root rounds like jnp.sqrt, libm and CUDA, whatever
    the host's torch build does, and keeps torch's derivative."""
    import math
    x = torch.from_numpy(np.random.default_rng(3).uniform(0.01, 10.0, 20000))
    assert torch.equal(O.sqrt(x), torch.from_numpy(np.sqrt(x.numpy())))
    assert [O.sqrt(torch.tensor(v, dtype=torch.float64)).item() for v in (2.0, 0.125, 1.12)] == \
        [math.sqrt(v) for v in (2.0, 0.125, 1.12)]
    xg = x[:64].clone().requires_grad_(True)
    O.sqrt(xg).sum().backward()
    assert torch.allclose(xg.grad, 0.5 / torch.from_numpy(np.sqrt(x[:64].numpy())), rtol=1e-15, atol=0)


def test_oracle_takes_every_root_from_its_own_sqrt():
    src = open(os.path.join(ROOT, "oracle", "jf_oracle.py")).read()
    code = "\n".join(line.split("#")[0] for line in src.splitlines())
    assert "torch.sqrt(" not in code and ".sqrt()" not in code and "** 0.5" not in code


STEP_SCHEMES = [(0, 0), (1, 1), (2, 2)]  # (reconstruction mode, Riemann solver)


@pytest.mark.parametrize("mode,riemann", STEP_SCHEMES, ids=["primitive-hllc", "char-arithmetic-rusanov",
                                                            "char-roe-hll"])
@pytest.mark.parametrize("name,cells,bc,kind", CASES, ids=[c[0] for c in CASES])
def test_c_rk3_steps_match_torch_oracle(crhs, name, cells, bc, kind, mode, riemann):
    """CFL time step, three stages, primitives and halos after every stage:
    the states and the time agree bitwise after the steps."""
    import __graft_entry__
    lib = ctypes.CDLL(__graft_entry__.build_oracle_c())
    f = lib.jf_rk3_steps
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.c_int,
                  ctypes.POINTER(ctypes.c_double), ctypes.c_double, ctypes.c_double, ctypes.c_double,
                  ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.c_int,
                  ctypes.POINTER(ctypes.c_double)]
    f.restype = ctypes.c_int
    oc, _ = both(cells, bc, riemann=RIEMANN[riemann], **MODES[mode])
    if kind == "sod":
        prims, steps = sod_prims(cells[0]), 12
    elif kind == "quad":
        prims, steps = quadrant_prims(cells[0], cells[1], seed=4), 4
    else:
        prims, steps = tgv_prims(max(cells))[:, :cells[0], :cells[1], :cells[2]].contiguous(), 3
    U, P = O.initialize(prims, oc)
    inner = oc.interior()
    Uc = np.ascontiguousarray(U[inner].numpy())
    Pc = np.ascontiguousarray(P[inner].numpy())
    t = 0.0
    for _ in range(steps):
        dt = O.compute_dt(P, oc)
        U, P = O.rk3_step(U, P, dt, oc)
        t += dt.item()
    tc = ctypes.c_double(0.0)
    odx = (ctypes.c_double * 3)(*[oc.one_cell_size(a) if cells[a] > 1 else 0.0 for a in range(3)])
    codes = (ctypes.c_int * 6)(*[BC[oc.bc[f_]] for f_ in FACE_ORDER])
    assert f(Uc.ctypes.data, Pc.ctypes.data, (ctypes.c_int * 3)(*cells), oc.nh, odx, oc.min_cell_size, oc.cfl,
             oc.gamma, O.STENCIL_EPS, mode, riemann, codes, steps, ctypes.byref(tc)) == 0
    assert tc.value == t
    assert torch.equal(torch.from_numpy(Uc), U[inner])
    assert torch.equal(torch.from_numpy(Pc), P[inner])


def test_oracle_rdiv_rounds_once():
    x = torch.from_numpy(np.random.default_rng(5).uniform(0.01, 10.0, 20000))
    for a in (0.1, 3.0 / 14.0, 1.0 / 120.0):
        assert torch.equal(O.rdiv(a, x), torch.from_numpy(a / x.numpy()))


def test_c_and_torch_oracles_agree_on_sod_200_to_end_time(crhs):
    """The 1-D Sod workload at its full size (200 cells, WENO5-Z + HLLC, CFL
    0.5, zero-gradient) to t = 0.2: both restatements step to the same state
    and time, bitwise."""
    import __graft_entry__
    f = ctypes.CDLL(__graft_entry__.build_oracle_c()).jf_rk3_steps
    f.restype = ctypes.c_int
    cells = (200, 1, 1)
    oc, _ = both(cells, "ZEROGRADIENT", cfl=0.5)
    U, P = O.initialize(sod_prims(200), oc)
    inner = oc.interior()
    Uc = np.ascontiguousarray(U[inner].numpy())
    Pc = np.ascontiguousarray(P[inner].numpy())
    t, steps = 0.0, 0
    while t < 0.2:
        dt = O.compute_dt(P, oc)
        U, P = O.rk3_step(U, P, dt, oc)
        t += dt.item()
        steps += 1
    tc = ctypes.c_double(0.0)
    odx = (ctypes.c_double * 3)(oc.one_cell_size(0), 0.0, 0.0)
    codes = (ctypes.c_int * 6)(*[BC["ZEROGRADIENT"]] * 6)
    assert f(ctypes.c_void_p(Uc.ctypes.data), ctypes.c_void_p(Pc.ctypes.data), (ctypes.c_int * 3)(*cells),
             ctypes.c_int(oc.nh), odx, ctypes.c_double(oc.min_cell_size), ctypes.c_double(oc.cfl),
             ctypes.c_double(oc.gamma), ctypes.c_double(O.STENCIL_EPS), ctypes.c_int(0), ctypes.c_int(0), codes,
             ctypes.c_int(steps), ctypes.byref(tc)) == 0
    assert steps > 50 and tc.value == t
    assert torch.equal(torch.from_numpy(Uc), U[inner])


VISC_CASES = [("tgv-3d", (12, 10, 8)), ("tgv-2d", (16, 12, 1))]
DISS = {"visc-heat": dict(viscous=True, heat=True), "visc": dict(viscous=True, heat=False),
        "heat": dict(viscous=False, heat=True),
        "visc-heat-noproduction": dict(viscous=True, heat=True, viscous_heat_production=False)}


def _visc_args(oc):
    return (oc.mu, oc.bulk_viscosity, oc.kappa(), oc.cp(), oc.R, int(oc.viscous), int(oc.heat),
            int(oc.viscous_heat_production))


def _rough_tgv(cells, seed):
    prims = tgv_prims(max(cells))[:, :cells[0], :cells[1], :cells[2]].contiguous().clone()
    rng = np.random.default_rng(seed)
    # relative noise: density and pressure stay positive
    return prims * (1.0 + torch.from_numpy(0.05 * rng.uniform(-1.0, 1.0, prims.shape)))


@pytest.mark.parametrize("riemann", list(RIEMANN), ids=[v.lower() for v in RIEMANN.values()])
@pytest.mark.parametrize("diss", list(DISS))
@pytest.mark.parametrize("mode", [0, 1, 2], ids=["primitive", "char-arithmetic", "char-roe"])
@pytest.mark.parametrize("name,cells", VISC_CASES, ids=[c[0] for c in VISC_CASES])
def test_c_viscous_rhs_matches_torch_oracle(name, cells, mode, diss, riemann):
    """CENTRAL4 viscous and heat fluxes on a periodic box, added to the
    WENO5-Z (primitive or characteristic) + HLLC / Rusanov / HLL flux of every
    face: the C right-hand side equals the torch oracle's bitwise."""
    import __graft_entry__
    f = ctypes.CDLL(__graft_entry__.build_oracle_c()).jf_rhs_weno5z_visc
    f.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                  ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int] + [ctypes.c_double] * 5 + \
        [ctypes.c_int] * 3 + [ctypes.c_void_p]
    f.restype = ctypes.c_int
    oc, _ = both(cells, "PERIODIC", nh=4, riemann=RIEMANN[riemann], mu=0.01, bulk_viscosity=0.003, prandtl=0.72,
                 **MODES[mode], **DISS[diss])
    U, P = O.initialize(_rough_tgv(cells, 7), oc)
    ref = O.compute_rhs(U, P, oc)
    Pn = np.ascontiguousarray(P.numpy())
    out = np.empty(ref.shape, dtype=np.float64)
    odx = (ctypes.c_double * 3)(*[oc.one_cell_size(a) if cells[a] > 1 else 0.0 for a in range(3)])
    assert f(Pn.ctypes.data, (ctypes.c_int * 3)(*cells), oc.nh, odx, oc.gamma, O.STENCIL_EPS, mode, riemann,
             *_visc_args(oc), out.ctypes.data) == 0
    assert torch.equal(torch.from_numpy(out), ref)


@pytest.mark.parametrize("limit,mu,heat", [("heat", 0.5, True), ("viscous", 1.0, False), ("cfl", 0.05, True)])
@pytest.mark.parametrize("mode", [0, 2], ids=["primitive", "char-roe"])
def test_c_viscous_rk3_steps_match_torch_oracle(mode, limit, mu, heat):
    """CFL, viscous and heat time-step limits (mu chosen so that `limit`
    decides dt), three stages: the C steps equal the torch oracle's bitwise
    (states and time)."""
    import __graft_entry__
    f = ctypes.CDLL(__graft_entry__.build_oracle_c()).jf_rk3_steps_visc
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.c_int,
                  ctypes.POINTER(ctypes.c_double), ctypes.c_double, ctypes.c_double, ctypes.c_double,
                  ctypes.c_double, ctypes.c_int, ctypes.c_int] + [ctypes.c_double] * 5 + [ctypes.c_int] * 4 + \
        [ctypes.POINTER(ctypes.c_double)]
    f.restype = ctypes.c_int
    cells = (12, 10, 8)
    oc, _ = both(cells, "PERIODIC", nh=4, riemann="HLLC", mu=mu, prandtl=0.72, viscous=True, heat=heat, cfl=0.5,
                 **MODES[mode])
    U, P = O.initialize(_rough_tgv(cells, 11), oc)
    Pi = P[oc.interior()]
    c = O.speed_of_sound(Pi[4], Pi[0], oc.gamma)
    dts = {"cfl": O.rdiv(oc.min_cell_size, (sum(torch.abs(Pi[i + 1]) + c for i in range(3))).max() + O.EPS),
           "viscous": O.rdiv(3.0 / 14.0 * oc.min_cell_size ** 2, O.rdiv(oc.mu, Pi[0]).max() + O.EPS)}
    if heat:
        dts["heat"] = O.rdiv(0.1 * oc.min_cell_size ** 2, O.rdiv(oc.kappa(), Pi[0] * oc.cp()).max() + O.EPS)
    assert min(dts, key=lambda k: dts[k].item()) == limit
    inner = oc.interior()
    Uc = np.ascontiguousarray(U[inner].numpy())
    Pc = np.ascontiguousarray(P[inner].numpy())
    t, steps = 0.0, 3
    for _ in range(steps):
        dt = O.compute_dt(P, oc)
        U, P = O.rk3_step(U, P, dt, oc)
        t += dt.item()
    tc = ctypes.c_double(0.0)
    odx = (ctypes.c_double * 3)(*[oc.one_cell_size(a) for a in range(3)])
    assert f(Uc.ctypes.data, Pc.ctypes.data, (ctypes.c_int * 3)(*cells), oc.nh, odx, oc.min_cell_size, oc.cfl,
             oc.gamma, O.STENCIL_EPS, mode, 0, *_visc_args(oc), steps, ctypes.byref(tc)) == 0
    assert tc.value == t
    assert torch.equal(torch.from_numpy(Uc), U[inner])
    assert torch.equal(torch.from_numpy(Pc), P[inner])
