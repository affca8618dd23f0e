"""Single-stage entry points and the solver handle against the fused step:
three gbf_rk3_stage calls equal one gbf_rk3_advance step bitwise, the stage
VJPs compose to the step VJP, and gbf_create / gbf_solver_advance equal the
fused path."""
import ctypes
import math

import pytest
import torch

from oracle import jf_oracle as O
from tests.cases import both, quadrant_prims, rel_err, tgv_prims

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from jaxfluids_gb300 import build
    build.build()


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


CASES = [
    ("tgv-3d", (16, 16, 16), "PERIODIC", {"ranges": ((0, 2 * math.pi),) * 3}, "tgv"),
    ("quad-2d-walls-char-roe-viscous", (24, 20, 1),
     {"east": "WALL", "west": "WALL", "north": "WALL", "south": "WALL", "top": "PERIODIC", "bottom": "PERIODIC"},
     {"nh": 4, "recon_var": "CHAR-PRIMITIVE", "frozen_state": "ROE", "viscous": True, "heat": True, "mu": 0.02,
      "prandtl": 0.71, "bc_values": {"east": (0.0, 0.0, 0.0), "west": (0.0, 0.0, 0.0), "north": (0.3, 0.0, 0.0),
                                     "south": (0.0, 0.0, 0.0)}}, "quad"),
]


def _state(cells, kind, oc):
    if kind == "tgv":
        prims = tgv_prims(max(cells))[:, :cells[0], :cells[1], :cells[2]].contiguous()
    else:
        prims = quadrant_prims(cells[0], cells[1], seed=4)
    U, P = O.initialize(prims, oc)
    return U[oc.interior()].contiguous().cuda()


@pytest.mark.parametrize("name,cells,bc,kw,kind", CASES, ids=[c[0] for c in CASES])
def test_three_stages_equal_one_fused_step(name, cells, bc, kw, kind):
    from jaxfluids_gb300 import FusedRK3, _lib
    lib = _lib.load()
    oc, cc = both(cells, bc, **kw)
    U0 = _state(cells, kind, oc)
    f = FusedRK3(cc)
    f.set_state(U0)
    dt_state = f.dt_state.clone()
    f.advance(2)
    ref = f.cons.clone()
    c = cc.to_c()
    U = U0.clone()
    A, B = torch.empty_like(U), torch.empty_like(U)
    ws = torch.empty(int(lib.gbf_rk3_workspace_bytes(ctypes.byref(c))) // 8, dtype=torch.float64, device="cuda")
    for _ in range(2):
        for stage, (k, n, out) in enumerate(((U, U, A), (A, U, B), (B, U, U))):
            st = lib.gbf_rk3_stage(ctypes.byref(c), stage, _ptr(k), _ptr(n), _ptr(out), _ptr(dt_state), _ptr(ws),
                                   None, _stream())
            assert st == _lib.GBF_OK, st
    torch.cuda.synchronize()
    assert torch.equal(U, ref)
    assert torch.equal(dt_state[:2], f.dt_state[:2])


def test_stage_vjps_compose_to_the_step_vjp():
    from jaxfluids_gb300 import _lib
    from jaxfluids_gb300.adjoint import AdjointRK3
    lib = _lib.load()
    oc, cc = both((40, 36, 1), "PERIODIC", recon_var="CHAR-PRIMITIVE", frozen_state="ROE")
    U0 = _state((40, 36, 1), "quad", oc)
    dt = 1e-3
    adj = AdjointRK3(cc, dt=dt)
    _, store = adj.forward_stored(U0, 1)
    Un, U1, U2 = store[0]
    lam = torch.randn(U0.shape, generator=torch.Generator(device="cuda").manual_seed(5), dtype=torch.float64,
                      device="cuda")
    ref = adj.step_vjp_stages(Un, U1, U2, lam)
    c = cc.to_c()
    ws = adj.ws
    lam_n = torch.zeros_like(lam)
    lam2, lam1, lam0 = torch.empty_like(lam), torch.empty_like(lam), torch.empty_like(lam)
    for stage, (Uk, lin, lout) in ((2, (U2, lam, lam2)), (1, (U1, lam2, lam1)), (0, (Un, lam1, lam0))):
        st = lib.gbf_rk3_stage_vjp(ctypes.byref(c), stage, _ptr(Uk), _ptr(adj.dt_dev), _ptr(lin), _ptr(lout),
                                   _ptr(lam_n), _ptr(ws), None, _stream())
        assert st == _lib.GBF_OK, st
    total = lam0 + lam_n
    assert rel_err(total, ref) <= 1e-13


def test_solver_handle_equals_the_fused_path():
    from jaxfluids_gb300 import FusedRK3, _lib
    lib = _lib.load()
    oc, cc = both((16, 16, 16), "PERIODIC", ranges=((0, 2 * math.pi),) * 3)
    U0 = _state((16, 16, 16), "tgv", oc)
    f = FusedRK3(cc)
    f.set_state(U0)
    f.advance(3)
    c = cc.to_c()
    h = ctypes.c_void_p()
    assert lib.gbf_create(ctypes.byref(c), None, ctypes.byref(h)) == _lib.GBF_OK
    try:
        U = U0.clone()
        assert lib.gbf_solver_init(h, _ptr(U), ctypes.c_double(0.0), _stream()) == _lib.GBF_OK
        assert lib.gbf_solver_advance(h, _ptr(U), 3, _stream()) == _lib.GBF_OK
        dt_t = (ctypes.c_double * 2)()
        assert lib.gbf_solver_time(h, dt_t, _stream()) == _lib.GBF_OK
        assert torch.equal(U, f.cons)
        assert dt_t[0] == f.dt.item() and dt_t[1] == f.t.item()
    finally:
        assert lib.gbf_destroy(h) == _lib.GBF_OK


def test_captured_steps_equal_launched_steps():
    from jaxfluids_gb300 import FusedRK3
    oc, cc = both((64, 1, 1), "ZEROGRADIENT")
    from tests.cases import sod_prims
    U, P = O.initialize(sod_prims(64), oc)
    U0 = U[oc.interior()].contiguous().cuda()
    a, b = FusedRK3(cc), FusedRK3(cc)
    a.set_state(U0)
    b.set_state(U0)
    g = b.capture(5)
    assert torch.equal(b.cons, U0)  # capturing does not advance the state
    for _ in range(3):
        a.advance(5)
        g.replay()
    torch.cuda.synchronize()
    assert torch.equal(a.cons, b.cons)
    assert torch.equal(a.dt_state[:2], b.dt_state[:2])


def test_state_health_counts_planted_faults():
    from jaxfluids_gb300 import FusedRK3
    oc, cc = both((32, 24, 1), "ZEROGRADIENT")
    U0 = _state((32, 24, 1), "quad", oc)
    f = FusedRK3(cc)
    f.set_state(U0)
    assert f.state_health() == {"nonfinite": 0, "rho_nonpositive": 0, "p_nonpositive": 0}
    bad = U0.clone()
    bad[4, 3, 5, 0] = float("nan")                       # non-finite energy
    bad[:, 10, 2, 0] = torch.tensor([-1.0, 0.0, 0.0, 0.0, 1.0], dtype=torch.float64)   # rho < 0, p > 0
    bad[:, 20, 7, 0] = torch.tensor([1.0, 0.0, 0.0, 0.0, -1.0], dtype=torch.float64)   # p < 0
    f.cons.copy_(bad)
    assert f.state_health() == {"nonfinite": 1, "rho_nonpositive": 1, "p_nonpositive": 1}
