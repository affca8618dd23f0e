"""The interpolation limiter (conservatives.positivity.is_interpolation_limiter,
solvers/positivity/limiter_interpolation.py:82-210) on the CUDA path against
the oracle: the right-hand side bitwise where the limiter replaces face states,
and its reverse (the replaced primitives' cotangents go to the cell beside the
face) against the oracle's autograd, on primitive, characteristic,
conservative and characteristic-conservative reconstructions."""
import math

import pytest
import torch

from oracle import jf_oracle as O
from tests.cases import both, rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from jaxfluids_gb300 import build
    build.build()


def _dip_prims(n=48):
    """Smooth periodic state with a pressure dip to 4e-11: the reconstructed
    pressure at the dip's faces drops below the limiter's 1e-10."""
    x = (torch.arange(n, dtype=torch.float64) + 0.5) / n
    rho = 1.0 + 0.2 * torch.sin(2 * math.pi * x + 0.3)
    u = 0.3 * torch.sin(2 * math.pi * x + 1.1)
    p = 0.5 + 0.3 * torch.sin(2 * math.pi * x + 2.0)
    p[19] = 0.02
    p[20] = 4e-11
    return torch.stack([rho, u, p]).reshape(3, n, 1, 1)


CHAR = {"CHAR-ARITHMETIC": dict(recon_var="CHAR-PRIMITIVE", frozen_state="ARITHMETIC"),
        "CHAR-ROE": dict(recon_var="CHAR-PRIMITIVE", frozen_state="ROE"),
        "CONSERVATIVE": dict(recon_var="CONSERVATIVE"),
        "CHARCONS-ROE": dict(recon_var="CHAR-CONSERVATIVE", frozen_state="ROE")}
CASES = [(r, s, lv) for r in ("WENO5-Z", "WENO5-JS", "WENO3-Z", "MINMOD-AD") + tuple(CHAR)
         for s in ("HLLC", "RUSANOV") for lv in (False, True)]


def _ids(c):
    return f"{c[0]}-{c[1]}" + ("-limit-velocity" if c[2] else "")


def _face_pressures(P, oc, j):
    """Reconstructed face pressures of side j along x, before the limiter
    (the oracle's primitive or characteristic reconstruction)."""
    if oc.recon_var == "PRIMITIVE":
        return O.reconstruct_xi(P, oc, 0, j)[4]
    order = (0, 1, 2, 3, 4) if j == 0 else (5, 4, 3, 2, 1)
    if oc.recon_var in ("CONSERVATIVE", "CHAR-CONSERVATIVE"):
        U = O.cons_from_prims(P, oc.gamma)
        if oc.recon_var == "CONSERVATIVE":
            Uj = O.reconstruct_xi(U, oc, 0, j)
        else:
            Rm, Lm = O.eigvecs_conservatives(P, oc, 0)
            win = [U[O._stencil_slice(oc, 0, k)] for k in range(-3, 3)]
            chars = [O._matvec5(Lm, [w[v] for v in range(5)]) for w in win]
            ch = [O.weno5z_stencil(*[chars[k][v] for k in order]) for v in range(5)]
            Uj = torch.stack(O._matvec5(Rm, ch), 0)
        return O.prims_from_cons(Uj, oc.gamma)[4]
    rho_a, c, cc = O.frozen_state(P, oc, 0)
    win = [P[O._stencil_slice(oc, 0, k)] for k in range(-3, 3)]
    chars = [O.chars_from_prims([w[v] for v in range(5)], rho_a, c, cc, 0) for w in win]
    ch = [O.weno5z_stencil(*[chars[k][v] for k in order]) for v in range(5)]
    return O.prims_from_chars(ch, rho_a, c, cc, 0)[4]


@pytest.mark.parametrize("recon,riemann,limit_velocity", CASES, ids=[_ids(c) for c in CASES])
def test_limiter_rhs_bitwise_and_vjp(recon, riemann, limit_velocity):
    from jaxfluids_gb300 import SimulationManager
    from jaxfluids_gb300.adjoint import AdjointRK3
    n = 48
    kw = CHAR.get(recon, {"recon": recon})
    oc, cc = both((n, 1, 1), {f: "PERIODIC" for f in O.FACES}, riemann=riemann,
                  interpolation_limiter=True, limit_velocity=limit_velocity, **kw)
    U, P = O.initialize(_dip_prims(n), oc)
    limited = sum(int((_face_pressures(P, oc, j) < O.LIMITER_EPS_PRESSURE).sum()) for j in (0, 1))
    assert limited > 0, "the case must exercise the limiter"
    ref = O.compute_rhs(U, P, oc)
    sim = SimulationManager(cc)
    rhs = sim.space_solver.compute_rhs(U.cuda(), P.cuda(), None, 0.0, 0.0)[0].euler_buffers.conservatives
    assert torch.equal(rhs.cpu(), ref)
    Ui = U[oc.interior()].contiguous()
    w = torch.randn(Ui.shape, generator=torch.Generator().manual_seed(5), dtype=torch.float64)
    x = Ui.clone().requires_grad_(True)
    (O.rhs_of_interior_cons(x, oc) * w).sum().backward()
    gv = AdjointRK3(cc, dt=1e-4).rhs_vjp(Ui.cuda(), w.cuda().contiguous())
    assert rel_err(gv, x.grad) <= 1e-11


def test_limiter_fused_steps():
    from jaxfluids_gb300 import FusedRK3
    n = 48
    oc, cc = both((n, 1, 1), {f: "PERIODIC" for f in O.FACES}, interpolation_limiter=True)
    U, P = O.initialize(_dip_prims(n), oc)
    Ur, Pr = U, P
    for _ in range(4):
        Ur, Pr = O.rk3_step(Ur, Pr, O.compute_dt(Pr, oc), oc)
    f = FusedRK3(cc)
    f.set_state(U[oc.interior()].contiguous().cuda())
    f.advance(4)
    assert rel_err(f.cons, Ur[oc.interior()]) <= 1e-10
