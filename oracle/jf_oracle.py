"""CPU restatement of JAX-Fluids' single-phase finite-volume right-hand side.

TEST INFRASTRUCTURE ONLY -- this module is the oracle the CUDA kernels are
checked against.  The product package never imports it.

The reference (JAX-Fluids 0.2.x, ``src/jaxfluids``) is written in
``jax.numpy``; JAX is not available where this oracle runs, so every function
below restates the reference op for op in ``torch`` on the CPU in float64.
torch's elementwise CPU kernels round after every operation, like the
reference's un-fused ``jnp`` graph, and torch autograd follows the same
conventions as ``jax.grad`` at the non-smooth points used here
(``where`` selects, ``abs'(0) = 0``, ``maximum``/``minimum`` split ties
evenly), so ``torch.autograd`` on this oracle stands in for ``jax.grad``
through ``SimulationManager._feed_forward``.

Each function cites the reference file:line it follows (paths relative to
``src/jaxfluids``).  Parity pins (``tests/golden``): the per-step dt and
minimum-density log of ``notebooks/basics/101/01_tutorial`` (HLLC + MINMOD,
periodic, CFL 0.9), the loss/gradient trace of
``notebooks/basics/101/02_tutorial`` (Rusanov + MINMOD-AD, zero-gradient,
fixed dt, through ``jax.grad``) and the reference's own exact Riemann solver
for Sod at t = 0.2 (physics tolerance).  WENO5-Z, CHAR-PRIMITIVE and the
viscous flux have no numeric pin in the reference; they are pinned by
line-by-line citation and by the physics checks in ``tests/``.

Buffers follow the reference layout: ``[5, Nx+2nh, Ny+2nh, Nz+2nh]`` with an
inactive axis of size 1 and no halo; primitives are (rho, u, v, w, p) and
conservatives (rho, rho u, rho v, rho w, E).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Callable, Dict, List, Optional, Tuple

import numpy as np
import torch

Tensor = torch.Tensor


class _Sqrt(torch.autograd.Function):
    """Correctly rounded square root with torch's own derivative.

    jnp.sqrt (XLA), libm and CUDA's double sqrt round correctly; torch.sqrt
    in float64 does not on every CPU build (an x86 build with MKL is one ulp
    off for about 1% of inputs, sqrt(2.0) among them), so the oracle takes
    numpy's, which does.  The derivative is torch's: grad / (2 sqrt(x)).
    """

    @staticmethod
    def forward(ctx, x):
        out = torch.from_numpy(np.asarray(np.sqrt(x.detach().numpy())))
        ctx.save_for_backward(out)
        return out

    @staticmethod
    def backward(ctx, grad):
        (out,) = ctx.saved_tensors
        return grad / (2 * out)


def sqrt(x: Tensor) -> Tensor:
    return _Sqrt.apply(x)


def rdiv(a: float, t: Tensor) -> Tensor:
    """a / t rounded once, as jnp's true_divide of a Python scalar by an array.
    torch evaluates ``float / tensor`` as ``float * (1 / tensor)``, two
    roundings, which differs for about a quarter of the inputs unless the
    numerator is a power of two (``1.0 / x``, ``0.5 / x`` stay exact)."""
    return torch.full_like(t, a) / t


# precision.py:50 (jnp.finfo(float64).eps) and :53 (spatial stencil eps)
EPS = 2.220446049250313e-16
STENCIL_EPS = 1e-30

FACES = ("east", "west", "north", "south", "top", "bottom")
FACE_AXIS = {"east": 0, "west": 0, "north": 1, "south": 1, "top": 2, "bottom": 2}
AXIS_FACES = {0: ("west", "east"), 1: ("south", "north"), 2: ("bottom", "top")}


@dataclass
class OracleCase:
    """The subset of case_setup / numerical_setup the path reads."""
    cells: Tuple[int, int, int]
    ranges: Tuple[Tuple[float, float], ...] = ((0.0, 1.0), (0.0, 1.0), (0.0, 1.0))
    nh: int = 3
    gamma: float = 1.4
    R: float = 1.0
    bc: Dict[str, str] = field(default_factory=dict)
    recon: str = "WENO5-Z"                 # WENO5-Z | WENO5-JS | TENO5 | WENO3-JS | WENO3-Z | MINMOD | MINMOD-AD
    recon_var: str = "PRIMITIVE"           # PRIMITIVE | CHAR-PRIMITIVE | CONSERVATIVE | CHAR-CONSERVATIVE
    frozen_state: str = "ARITHMETIC"       # ARITHMETIC | ROE
    riemann: str = "HLLC"                  # HLLC | HLL | RUSANOV | LAX-FRIEDRICHS
    signal_speed: str = "EINFELDT"
    cfl: float = 0.5
    fixed_dt: Optional[float] = None
    viscous: bool = False
    heat: bool = False
    mu: float = 0.0
    bulk_viscosity: float = 0.0
    prandtl: Optional[float] = None
    viscous_heat_production: bool = True
    # constant boundary values per face: WALL (u, v, w) wall velocity
    # (wall_velocity_callable), DIRICHLET (rho, u, v, w, p)
    # (primitives_callable), NEUMANN (rho, u, v, w, p) normal derivatives
    bc_values: Dict[str, Tuple[float, ...]] = field(default_factory=dict)
    # dissipative_fluxes stencils: CENTRAL4 | CENTRAL2
    diss_recon: str = "CENTRAL4"
    diss_deriv_center: str = "CENTRAL4"
    diss_deriv_face: str = "CENTRAL4"
    # active_physics.is_convective_flux
    convective: bool = True
    # thermal_conductivity CUSTOM value (None: PRANDTL model from prandtl)
    thermal_conductivity: Optional[float] = None
    # conservatives.positivity.{is_interpolation_limiter, limit_velocity}
    interpolation_limiter: bool = False
    limit_velocity: bool = False
    # forcings.gravity with active_physics.is_volume_force
    gravity: Optional[Tuple[float, float, float]] = None
    # boundary values varying in time: face -> function of t giving the
    # values [k, boundary cells] at t (replaces bc_values[face])
    bc_time: Dict[str, Callable] = field(default_factory=dict)

    # ---- domain information (domain/domain_information.py:80-206) ----
    @property
    def active(self) -> List[int]:
        return [i for i in range(3) if self.cells[i] > 1]

    @property
    def dim(self) -> int:
        return len(self.active)

    def cell_size(self, axis: int) -> float:
        # domain/mesh_creation/homogenous.py:13
        lo, hi = self.ranges[axis]
        return (hi - lo) / self.cells[axis]

    def one_cell_size(self, axis: int) -> float:
        # domain/domain_information.py:290
        return 1.0 / self.cell_size(axis)

    @property
    def min_cell_size(self) -> float:
        # domain/domain_information.py:698-701
        return min(self.cell_size(i) for i in self.active)

    def cell_centers(self, axis: int) -> Tensor:
        # domain/mesh_creation/homogenous.py:14 (np.linspace)
        import numpy as np
        lo, hi = self.ranges[axis]
        d = self.cell_size(axis)
        return torch.from_numpy(np.linspace(lo + d / 2, hi - d / 2, self.cells[axis]))

    def buffer_shape(self) -> Tuple[int, int, int, int]:
        # initialization/helper_functions.py:49
        return (5,) + tuple(n + 2 * self.nh if n > 1 else 1 for n in self.cells)

    def inner(self, axis: int) -> slice:
        return slice(self.nh, -self.nh) if self.cells[axis] > 1 else slice(None)

    def interior(self) -> Tuple[slice, ...]:
        return (slice(None),) + tuple(self.inner(i) for i in range(3))

    def cp(self) -> float:
        # materials/single_materials/ideal_gas.py:32
        return self.gamma / (self.gamma - 1.0) * self.R

    def kappa(self) -> float:
        # CUSTOM constant value, else the PRANDTL model
        # (materials/single_materials/material.py:115-116): cp mu / Pr
        if self.thermal_conductivity is not None:
            return self.thermal_conductivity
        return self.cp() * self.mu / self.prandtl


def _axis_slice(case: OracleCase, axis: int, s: slice) -> Tuple[slice, ...]:
    sl = [slice(None)] + [case.inner(i) for i in range(3)]
    sl[axis + 1] = s
    return tuple(sl)


def _stencil_slice(case: OracleCase, axis: int, k: int, at_center: int = 0) -> Tuple[slice, ...]:
    # stencils/spatial_stencil.py:96-110 (nlo = n + k, nhi = -n + k + 1 - at_cell_center)
    n = case.nh
    nlo = n + k
    nhi = -n + k + 1 - at_center
    assert nlo >= 0 and nhi <= 0
    return _axis_slice(case, axis, slice(nlo, nhi if nhi != 0 else None))


class _JaxAbs(torch.autograd.Function):
    """|x| with jax's derivative convention: d|x|/dx = +1 at x = 0
    (jax.lax abs JVP, select(x >= 0, g, -g)); torch's own abs gives 0 there."""

    @staticmethod
    def forward(ctx, x):
        ctx.save_for_backward(x)
        return torch.abs(x)

    @staticmethod
    def backward(ctx, g):
        (x,) = ctx.saved_tensors
        return torch.where(x >= 0, g, -g)


def jabs(x: Tensor) -> Tensor:
    return _JaxAbs.apply(x)


# ---------------------------------------------------------------------------
# Ideal-gas EOS and equation layout
# ---------------------------------------------------------------------------

def speed_of_sound(p: Tensor, rho: Tensor, gamma: float) -> Tensor:
    # materials/single_materials/ideal_gas.py:69-71
    return sqrt(gamma * p / rho)


def cons_from_prims(P: Tensor, gamma: float) -> Tensor:
    # equation_manager.py:93-101, ideal_gas.py:85-88 (e = p / (rho (gamma-1)))
    rho = P[0]
    vel = P[1:4]
    e = P[4] / (rho * (gamma - 1.0))
    mom = rho * vel
    sq = vel * vel
    E = rho * (0.5 * (sq[0] + sq[1] + sq[2]) + e)
    return torch.stack([rho, mom[0], mom[1], mom[2], E], dim=0)


def prims_from_cons(U: Tensor, gamma: float) -> Tensor:
    # equation_manager.py:164-171, ideal_gas.py:73-75 (p = (gamma-1) e rho)
    rho = U[0]
    one_rho = 1.0 / rho
    vel = U[1:4] * one_rho
    sq = vel * vel
    e = U[4] * one_rho - 0.5 * (sq[0] + sq[1] + sq[2])
    p = (gamma - 1.0) * e * rho
    return torch.stack([rho, vel[0], vel[1], vel[2], p], dim=0)


def fluxes_xi(P: Tensor, U: Tensor, axis: int) -> Tensor:
    # equation_manager.py:237-252
    rho_ui = U[axis + 1]
    f1 = U[axis + 1] * P[1]
    f2 = U[axis + 1] * P[2]
    f3 = U[axis + 1] * P[3]
    ui_Ep = P[axis + 1] * (U[4] + P[4])
    f = [rho_ui, f1, f2, f3, ui_Ep]
    f[axis + 1] = f[axis + 1] + P[4]
    return torch.stack(f, dim=0)


# ---------------------------------------------------------------------------
# Cell-face reconstruction
# ---------------------------------------------------------------------------

_WENO_DR = (1 / 10, 6 / 10, 3 / 10)                      # weno5_base.py:24
_WENO_CR = ((1 / 3, -7 / 6, 11 / 6),                      # weno5_base.py:25-27
            (-1 / 6, 5 / 6, 1 / 3),
            (1 / 3, 5 / 6, -1 / 6))


def weno5z_stencil(u0: Tensor, u1: Tensor, u2: Tensor, u3: Tensor, u4: Tensor,
                   eps: float = STENCIL_EPS) -> Tensor:
    """WENO5-Z on the five values (u_imm, u_im, u_i, u_ip, u_ipp).

    shock_capturing/weno/weno5_z.py:24-58, weno5_base.py:34-51.
    """
    b0 = 13.0 / 12.0 * torch.square(u0 - 2 * u1 + u2) + 1.0 / 4.0 * torch.square(u0 - 4 * u1 + 3 * u2)
    b1 = 13.0 / 12.0 * torch.square(u1 - 2 * u2 + u3) + 1.0 / 4.0 * torch.square(u1 - u3)
    b2 = 13.0 / 12.0 * torch.square(u2 - 2 * u3 + u4) + 1.0 / 4.0 * torch.square(3 * u2 - 4 * u3 + u4)
    tau5 = jabs(b0 - b2)
    a0 = _WENO_DR[0] * (1.0 + tau5 / (b0 + eps))
    a1 = _WENO_DR[1] * (1.0 + tau5 / (b1 + eps))
    a2 = _WENO_DR[2] * (1.0 + tau5 / (b2 + eps))
    one_a = 1.0 / (a0 + a1 + a2)
    w0 = a0 * one_a
    w1 = a1 * one_a
    w2 = a2 * one_a
    c = _WENO_CR
    p0 = c[0][0] * u0 + c[0][1] * u1 + c[0][2] * u2
    p1 = c[1][0] * u1 + c[1][1] * u2 + c[1][2] * u3
    p2 = c[2][0] * u2 + c[2][1] * u3 + c[2][2] * u4
    return w0 * p0 + w1 * p1 + w2 * p2


def _weno5_smoothness(u0, u1, u2, u3, u4):
    # weno5_base.py:34-41
    b0 = 13.0 / 12.0 * torch.square(u0 - 2 * u1 + u2) + 1.0 / 4.0 * torch.square(u0 - 4 * u1 + 3 * u2)
    b1 = 13.0 / 12.0 * torch.square(u1 - 2 * u2 + u3) + 1.0 / 4.0 * torch.square(u1 - u3)
    b2 = 13.0 / 12.0 * torch.square(u2 - 2 * u3 + u4) + 1.0 / 4.0 * torch.square(3 * u2 - 4 * u3 + u4)
    return b0, b1, b2


def weno5js_stencil(u0: Tensor, u1: Tensor, u2: Tensor, u3: Tensor, u4: Tensor,
                    eps: float = STENCIL_EPS) -> Tensor:
    """WENO5-JS (shock_capturing/weno/weno5_js.py:33-70, weno5_base.py:34-51)."""
    b0, b1, b2 = _weno5_smoothness(u0, u1, u2, u3, u4)
    a0 = _WENO_DR[0] * (1.0 / (b0 * b0 + eps))
    a1 = _WENO_DR[1] * (1.0 / (b1 * b1 + eps))
    a2 = _WENO_DR[2] * (1.0 / (b2 * b2 + eps))
    one_a = 1.0 / (a0 + a1 + a2)
    c = _WENO_CR
    p0 = c[0][0] * u0 + c[0][1] * u1 + c[0][2] * u2
    p1 = c[1][0] * u1 + c[1][1] * u2 + c[1][2] * u3
    p2 = c[2][0] * u2 + c[2][1] * u3 + c[2][2] * u4
    return (a0 * one_a) * p0 + (a1 * one_a) * p1 + (a2 * one_a) * p2


_TENO5_DR = (0.05, 0.55, 0.40)                # teno5.py: coefficients for spectral properties
_TENO5_CT = 1e-5                               # teno5.py: cutoff


def teno5_stencil(u0: Tensor, u1: Tensor, u2: Tensor, u3: Tensor, u4: Tensor,
                  eps: float = STENCIL_EPS) -> Tensor:
    """TENO5 (shock_capturing/teno/teno5.py, Fu et al. 2016): gamma_k = (C +
    tau5 / (beta_k + eps))^q with C = 1, q = 6 (jnp.power with an integer
    exponent: lax.integer_pow's square-and-multiply, x^2 (x^2 x^2)); stencils
    with gamma_k / sum gamma < CT are cut; the kept d_k normalised by their sum
    + eps weight the WENO5 polynomials."""
    b0, b1, b2 = _weno5_smoothness(u0, u1, u2, u3, u4)
    tau5 = torch.abs(b0 - b2)

    def gamma(b):
        x = 1.0 + tau5 / (b + eps)
        x2 = x * x
        return x2 * (x2 * x2)
    g0, g1, g2 = gamma(b0), gamma(b1), gamma(b2)
    one_gamma_sum = 1.0 / (g0 + g1 + g2)
    def keep(g):
        # jnp.where(chi < CT, 0, 1): no derivative
        return torch.where(g * one_gamma_sum < _TENO5_CT, torch.zeros_like(g), torch.ones_like(g)).detach()
    w0 = _TENO5_DR[0] * keep(g0)
    w1 = _TENO5_DR[1] * keep(g1)
    w2 = _TENO5_DR[2] * keep(g2)
    one_dk = 1.0 / (w0 + w1 + w2 + eps)
    c = _WENO_CR
    p0 = c[0][0] * u0 + c[0][1] * u1 + c[0][2] * u2
    p1 = c[1][0] * u1 + c[1][1] * u2 + c[1][2] * u3
    p2 = c[2][0] * u2 + c[2][1] * u3 + c[2][2] * u4
    return (w0 * one_dk) * p0 + (w1 * one_dk) * p1 + (w2 * one_dk) * p2


_WENO3_DR = (1 / 3, 2 / 3)                    # weno3_base.py:24
_WENO3_CR = ((-0.5, 1.5), (0.5, 0.5))          # weno3_base.py:25


def weno3_stencil(u0: Tensor, u1: Tensor, u2: Tensor, z: bool, eps: float = STENCIL_EPS) -> Tensor:
    """WENO3-JS (weno/weno3_js.py:22-45) and WENO3-Z (weno/weno3_z.py:24-46) on
    (u_im, u_i, u_ip), weno3_base.py:31-44."""
    b0 = torch.square(u1 - u0)
    b1 = torch.square(u2 - u1)
    if z:
        tau3 = jabs(b0 - b1)
        a0 = _WENO3_DR[0] * (1.0 + tau3 / (b0 + eps))
        a1 = _WENO3_DR[1] * (1.0 + tau3 / (b1 + eps))
    else:
        a0 = _WENO3_DR[0] * (1.0 / (b0 * b0 + eps))
        a1 = _WENO3_DR[1] * (1.0 / (b1 * b1 + eps))
    one_a = 1.0 / (a0 + a1)
    p0 = _WENO3_CR[0][0] * u0 + _WENO3_CR[0][1] * u1
    p1 = _WENO3_CR[1][0] * u1 + _WENO3_CR[1][1] * u2
    return (a0 * one_a) * p0 + (a1 * one_a) * p1


def _recon_offsets(recon: str, j: int) -> Tuple[int, ...]:
    if recon in ("WENO3-JS", "WENO3-Z"):
        # weno3_base.py:29 array_slices([range(-2, 1, 1), range(1, -2, -1)])
        return (-2, -1, 0) if j == 0 else (1, 0, -1)
    if recon in ("WENO5-Z", "WENO5-JS", "TENO5"):
        # weno5_base.py:30 array_slices([range(-3, 2, 1), range(2, -3, -1)])
        return (-3, -2, -1, 0, 1) if j == 0 else (2, 1, 0, -1, -2)
    if recon in ("MINMOD", "MINMOD-AD"):
        # muscl3.py:33, minmod_ad.py:32
        return (-2, -1, 0) if j == 0 else (1, 0, -1)
    raise NotImplementedError(recon)


def recon_stencil(recon: str, j: int, vals: List[Tensor], eps: float = STENCIL_EPS) -> Tensor:
    """Face value from the stencil values ordered as the reference's slices."""
    if recon == "WENO5-Z":
        return weno5z_stencil(*vals, eps=eps)
    if recon == "WENO5-JS":
        return weno5js_stencil(*vals, eps=eps)
    if recon == "TENO5":
        return teno5_stencil(*vals, eps=eps)
    if recon in ("WENO3-JS", "WENO3-Z"):
        return weno3_stencil(*vals, z=(recon == "WENO3-Z"), eps=eps)
    b0, b1, b2 = vals
    if recon == "MINMOD":
        # muscl3.py:53-75, limiter.py:9-10
        eps_ad = 1e-10
        if j == 0:
            dc = b2 - b1
            du = b1 - b0
        else:
            dc = b1 - b2
            du = b0 - b1
        r = torch.where(du >= eps, dc / (du + eps_ad), (dc + eps) / (du + eps))
        lim = torch.maximum(torch.zeros_like(r), torch.minimum(torch.ones_like(r), r))
        if j == 0:
            return b1 + 0.5 * lim * du
        return b1 - 0.5 * lim * du
    if recon == "MINMOD-AD":
        # muscl/minmod_ad.py:45-66
        eps_ad = 1e-100
        if j == 0:
            dc = b2 - b1
            du = b1 - b0
        else:
            dc = b1 - b2
            du = b0 - b1
        r = torch.where(du >= eps, dc / (du + eps_ad), (dc + eps) / (du + eps))
        return torch.where(r < 0, b1, torch.where(r < 1, 0.5 * (b1 + b2), 1.5 * b1 - 0.5 * b0))
    raise NotImplementedError(recon)


def reconstruct_xi(buf: Tensor, case: OracleCase, axis: int, j: int) -> Tensor:
    """SpatialReconstruction.reconstruct_xi on a halo buffer -> face values [.., N+1, ..]."""
    vals = [buf[_stencil_slice(case, axis, k)] for k in _recon_offsets(case.recon, j)]
    return recon_stencil(case.recon, j, vals)


# ---------------------------------------------------------------------------
# Characteristic decomposition (CHAR-PRIMITIVE)
# ---------------------------------------------------------------------------

# equation_information.py:110 and eigendecomposition.py:67-71
VEL_MINORS = ((2, 3), (3, 1), (1, 2))
VEL_ID_EIGS = ((2, 3), (3, 2), (2, 3))


def frozen_state(P: Tensor, case: OracleCase, axis: int) -> Tuple[Tensor, Tensor, Tensor]:
    """Eigendecomposition.compute_frozen_state, single phase (eigendecomposition.py:120-281).

    Returns the frozen density, speed of sound and its square at every face
    (the only parts the primitive characteristic transforms use).
    """
    g = case.gamma
    L = P[_stencil_slice(case, axis, -1)]   # slice_LR[axis][0]: nh-1 : -nh
    R = P[_stencil_slice(case, axis, 0)]    # slice_LR[axis][1]: nh : -nh+1
    if case.frozen_state == "ARITHMETIC":
        pa = 0.5 * (L + R)
        c = sqrt(g * pa[4] / pa[0])
        return pa[0], c, c * c
    if case.frozen_state == "ROE":
        rho_a = sqrt(L[0] * R[0])
        sL, sR = sqrt(L[0]), sqrt(R[0])
        rho_div = 1.0 / (sL + sR)
        psi_a = (sL * (L[4] / L[0]) + sR * (R[4] / R[0])) * rho_div
        gr_a = (sL * (g - 1) + sR * (g - 1)) * rho_div
        d = R[1:4] - L[1:4]
        d2 = d * d
        sqvd = d2[0] + d2[1] + d2[2]
        p_over_rho = (sL * L[4] / L[0] + sR * R[4] / R[0]) * rho_div \
            + 0.5 * rho_a * rho_div * rho_div * sqvd
        cc = psi_a + gr_a * p_over_rho
        return rho_a, sqrt(cc), cc
    raise NotImplementedError(case.frozen_state)


def _total_enthalpy(p: Tensor, rho: Tensor, u: Tensor, g: float) -> Tensor:
    # ideal_gas.py:90-110: (p / (gamma - 1) + 0.5 rho (u^2 + v^2 + w^2) + p) / rho
    E = p / (g - 1) + 0.5 * rho * (u[0] * u[0] + u[1] * u[1] + u[2] * u[2])
    return (E + p) / rho


def frozen_state_full(P: Tensor, case: OracleCase, axis: int):
    """compute_frozen_state (eigendecomposition.py:120-281), single phase, with
    every output the conservative eigenvectors use: averaged primitives (ROE:
    compute_roe_cons :283-294 with the density sqrt(rho_L rho_R)), total
    enthalpy, Grueneisen coefficient (gamma - 1 for the ideal gas), speed of
    sound, its square, and the squared averaged velocity."""
    g = case.gamma
    L = P[_stencil_slice(case, axis, -1)]
    R = P[_stencil_slice(case, axis, 0)]
    if case.frozen_state == "ARITHMETIC":
        pa = 0.5 * (L + R)
        gr = (g - 1) * torch.ones_like(pa[0])
        H = _total_enthalpy(pa[4], pa[0], pa[1:4], g)
        c = sqrt(g * pa[4] / pa[0])
        cc = c * c
    elif case.frozen_state == "ROE":
        sL, sR = sqrt(L[0]), sqrt(R[0])
        pa = (sL * L + sR * R) / (sL + sR)
        pa = torch.cat([sqrt(L[0] * R[0]).unsqueeze(0), pa[1:]], 0)
        rho_div = 1.0 / (sL + sR)
        H = (sL * _total_enthalpy(L[4], L[0], L[1:4], g) + sR * _total_enthalpy(R[4], R[0], R[1:4], g)) * rho_div
        psi_a = (sL * (L[4] / L[0]) + sR * (R[4] / R[0])) * rho_div
        gr = (sL * (g - 1) + sR * (g - 1)) * rho_div
        d = R[1:4] - L[1:4]
        d2 = d * d
        sqvd = d2[0] + d2[1] + d2[2]
        p_over_rho = (sL * L[4] / L[0] + sR * R[4] / R[0]) * rho_div \
            + 0.5 * pa[0] * rho_div * rho_div * sqvd
        cc = psi_a + gr * p_over_rho
        c = sqrt(cc)
    else:
        raise NotImplementedError(case.frozen_state)
    u2 = pa[1:4] * pa[1:4]
    vsq = u2[0] + u2[1] + u2[2]
    return pa, H, gr, c, cc, vsq


def eigvecs_conservatives(P: Tensor, case: OracleCase, axis: int):
    """eigendecomposition_conservatives (eigendecomposition.py:576-662), single
    phase (Fedkiw et al. 1999): right and left eigenvectors of the
    conservative flux Jacobian at every face, as 5 x 5 nested lists."""
    pa, H, gr, c, cc, vsq = frozen_state_full(P, case, axis)
    one_cc = 1.0 / cc
    one_rho = 1.0 / pa[0]
    n = axis + 1
    m0, m1 = VEL_MINORS[axis]
    z = torch.zeros_like(pa[0])
    Rm = [[z] * 5 for _ in range(5)]
    Lm = [[z] * 5 for _ in range(5)]
    one = torch.ones_like(pa[0])
    Rm[0][0], Rm[n][0], Rm[m0][0], Rm[m1][0], Rm[4][0] = one, pa[n] - c, pa[m0], pa[m1], H - pa[n] * c
    Rm[0][n], Rm[1][n], Rm[2][n], Rm[3][n] = gr, gr * pa[1], gr * pa[2], gr * pa[3]
    Rm[4][n] = gr * H - cc
    Rm[m0][m0], Rm[4][m0] = -pa[0], -pa[0] * pa[m0]
    Rm[m1][m1], Rm[4][m1] = pa[0], pa[0] * pa[m1]
    Rm[0][4], Rm[n][4], Rm[m0][4], Rm[m1][4], Rm[4][4] = one, pa[n] + c, pa[m0], pa[m1], H + pa[n] * c
    h = 0.5 * one_cc
    Lm[0][0] = h * (gr * vsq - gr * H + (pa[n] + c) * c)
    Lm[0][n] = h * (-pa[n] * gr - c)
    Lm[0][m0] = h * (-pa[m0] * gr)
    Lm[0][m1] = h * (-pa[m1] * gr)
    Lm[0][4] = h * gr
    Lm[n][0] = one_cc * (H - vsq)
    Lm[n][1], Lm[n][2], Lm[n][3] = pa[1] * one_cc, pa[2] * one_cc, pa[3] * one_cc
    Lm[n][4] = -one_cc
    Lm[m0][0], Lm[m0][m0] = pa[m0] * one_rho, -one_rho
    Lm[m1][0], Lm[m1][m1] = -pa[m1] * one_rho, one_rho
    Lm[4][0] = h * (gr * vsq - gr * H - (pa[n] - c) * c)
    Lm[4][n] = h * (-pa[n] * gr + c)
    Lm[4][m0] = h * (-pa[m0] * gr)
    Lm[4][m1] = h * (-pa[m1] * gr)
    Lm[4][4] = h * gr
    return Rm, Lm


def _matvec5(M, x: List[Tensor]) -> List[Tensor]:
    # jnp.einsum("ij...,j...->i...") as a sum over j in index order
    return [M[i][0] * x[0] + M[i][1] * x[1] + M[i][2] * x[2] + M[i][3] * x[3] + M[i][4] * x[4]
            for i in range(5)]


def chars_from_prims(x: List[Tensor], rho_a, c, cc, axis: int) -> List[Tensor]:
    """get_characteristics_from_primitives, single phase (eigendecomposition.py:402-433)."""
    n = axis + 1
    m0, m1 = VEL_MINORS[axis]
    e0, e1 = VEL_ID_EIGS[axis]
    out = [None] * 5
    out[0] = -0.5 / c * x[n] + 0.5 / (cc * rho_a) * x[4]
    out[1] = x[0] - 1.0 / cc * x[4]
    out[e0] = x[m0]
    out[e1] = x[m1]
    out[4] = 0.5 / c * x[n] + 0.5 / (cc * rho_a) * x[4]
    return out


def prims_from_chars(x: List[Tensor], rho_a, c, cc, axis: int) -> List[Tensor]:
    """get_primitives_from_characteristics, single phase (eigendecomposition.py:499-523)."""
    n = axis + 1
    m0, m1 = VEL_MINORS[axis]
    e0, e1 = VEL_ID_EIGS[axis]
    out = [None] * 5
    out[0] = rho_a * (x[0] + x[4]) + x[1]
    out[n] = c * (-x[0] + x[4])
    out[m0] = x[e0]
    out[m1] = x[e1]
    out[4] = cc * rho_a * (x[0] + x[4])
    return out


# ---------------------------------------------------------------------------
# Riemann solvers
# ---------------------------------------------------------------------------

def signal_speeds(name: str, uL, uR, aL, aR, rhoL, rhoR, pL, pR, gamma):
    # solvers/riemann_solvers/signal_speeds.py
    if name == "EINFELDT":              # :109-133
        sL = sqrt(rhoL)
        sR = sqrt(rhoR)
        od = 1.0 / (sL + sR)
        eta2 = 0.5 * sL * sR * od * od
        ubar = (sL * uL + sR * uR) * od
        dbar = sqrt((sL * aL * aL + sR * aR * aR) * od + eta2 * torch.square(uR - uL))
        return torch.minimum(ubar - dbar, uL - aL), torch.maximum(ubar + dbar, uR + aR)
    if name == "DAVIS":                 # :51-69
        return torch.minimum(uL - aL, uR - aR), torch.maximum(uL + aL, uR + aR)
    if name == "ARITHMETIC":            # :10-29
        um = 0.5 * (uL + uR)
        am = 0.5 * (aL + aR)
        return torch.minimum(um - am, uL - aL), torch.maximum(um + am, uR + aR)
    if name == "RUSANOV":               # :31-49
        sp = torch.maximum(jabs(uL) + aL, jabs(uR) + aR)
        return -sp, sp
    if name == "TORO":                  # :135-157, :201-231
        rho_bar = 0.5 * (rhoL + rhoR)
        a_bar = 0.5 * (aL + aR)
        p_pvrs = 0.5 * (pL + pR) - 0.5 * (uR - uL) * rho_bar * a_bar
        p_star = torch.maximum(torch.zeros_like(p_pvrs), p_pvrs)
        g_ = (gamma + 1) * 0.5 / gamma
        qL = 1.0 * (p_star <= pL) + sqrt(1 + g_ * (p_star / pL - 1)) * (p_star > pL)
        qR = 1.0 * (p_star <= pR) + sqrt(1 + g_ * (p_star / pR - 1)) * (p_star > pR)
        return uL - aL * qL, uR + aR * qR
    raise NotImplementedError(name)


def compute_sstar(uL, uR, pL, pR, rhoL, rhoR, SL, SR):
    # signal_speeds.py:159-199
    rdL = rhoL * (SL - uL)
    rdR = rhoR * (SR - uR)
    return ((pR - pL) + (uL * rdL - uR * rdR)) / (rdL - rdR)


def _hllc_star_flux(P, U, S, Sstar, axis, side):
    # HLLC.py:41-78
    n = axis + 1
    pre = (S - P[n]) / (S - Sstar) * P[0]
    e_term = pre * (U[4] / U[0] + (Sstar - P[n]) * (Sstar + P[4] / P[0] / (S - P[n])))
    us = [pre, pre, pre, pre, e_term]
    us[n] = us[n] * Sstar
    for t in (1, 2, 3):
        if t != n:
            us[t] = us[t] * P[t]
    us = torch.stack(us, dim=0)
    F = fluxes_xi(P, U, axis)
    if side == "L":
        wave = torch.minimum(S, torch.zeros_like(S))
    else:
        wave = torch.maximum(S, torch.zeros_like(S))
    return F + wave * (us - U)


def riemann(PL, PR, UL, UR, case: OracleCase, axis: int) -> Tensor:
    g = case.gamma
    n = axis + 1
    cL = speed_of_sound(PL[4], PL[0], g)
    cR = speed_of_sound(PR[4], PR[0], g)
    if case.riemann == "HLLC":
        # HLLC.py:80-126
        SL, SR = signal_speeds(case.signal_speed, PL[n], PR[n], cL, cR, PL[0], PR[0], PL[4], PR[4], g)
        Ss = compute_sstar(PL[n], PR[n], PL[4], PR[4], PL[0], PR[0], SL, SR)
        FL = _hllc_star_flux(PL, UL, SL, Ss, axis, "L")
        FR = _hllc_star_flux(PR, UR, SR, Ss, axis, "R")
        sg = torch.sign(Ss)
        return 0.5 * (1 + sg) * FL + 0.5 * (1 - sg) * FR
    if case.riemann == "HLL":
        # HLL.py:28-58 (eps = precision epsilon, riemann_solver.py:28)
        SLs, SRs = signal_speeds(case.signal_speed, PL[n], PR[n], cL, cR, PL[0], PR[0], PL[4], PR[4], g)
        SL = torch.minimum(SLs, torch.zeros_like(SLs))
        SR = torch.maximum(SRs, torch.zeros_like(SRs))
        FL = fluxes_xi(PL, UL, axis)
        FR = fluxes_xi(PR, UR, axis)
        return (SR * FL - SL * FR + SL * SR * (UR - UL)) / (SR - SL + EPS)
    if case.riemann == "RUSANOV":
        # Rusanov.py:25-47
        alpha = torch.maximum(jabs(PL[n]) + cL, jabs(PR[n]) + cR)
        FL = fluxes_xi(PL, UL, axis)
        FR = fluxes_xi(PR, UR, axis)
        return 0.5 * (FL + FR) - 0.5 * alpha * (UR - UL)
    if case.riemann == "LAX-FRIEDRICHS":
        # LaxFriedrichs.py:25-47: one alpha for the axis, the maxima over every face
        alpha = torch.maximum(torch.max(jabs(PL[n]) + cL), torch.max(jabs(PR[n]) + cR))
        FL = fluxes_xi(PL, UL, axis)
        FR = fluxes_xi(PR, UR, axis)
        return 0.5 * (FL + FR) - 0.5 * alpha * (UR - UL)
    raise NotImplementedError(case.riemann)


def convective_flux_xi(P: Tensor, case: OracleCase, axis: int, U: Optional[Tensor] = None) -> Tensor:
    """HighOrderGodunov.compute_flux_xi (high_order_godunov.py:117-231, :233-418)."""
    g = case.gamma
    UL = UR = None
    if case.recon_var == "PRIMITIVE":
        PL = reconstruct_xi(P, case, axis, 0)
        PR = reconstruct_xi(P, case, axis, 1)
    elif case.recon_var == "CHAR-PRIMITIVE":
        # high_order_godunov.py:298-316: window of the 6 cells around each face
        # (eigendecomposition.py:75-118), WENO on each characteristic variable
        # with the window slices (spatial_reconstruction.py:21-44), back-transform
        if case.recon != "WENO5-Z":
            raise NotImplementedError("CHAR-PRIMITIVE is restated for WENO5-Z")
        rho_a, c, cc = frozen_state(P, case, axis)
        win = [P[_stencil_slice(case, axis, k)] for k in range(-3, 3)]   # window cells 0..5
        chars = [chars_from_prims([w[v] for v in range(5)], rho_a, c, cc, axis) for w in win]
        cL = [weno5z_stencil(*[chars[k][v] for k in (0, 1, 2, 3, 4)]) for v in range(5)]
        cR = [weno5z_stencil(*[chars[k][v] for k in (5, 4, 3, 2, 1)]) for v in range(5)]
        PL = torch.stack(prims_from_chars(cL, rho_a, c, cc, axis), 0)
        PR = torch.stack(prims_from_chars(cR, rho_a, c, cc, axis), 0)
    elif case.recon_var == "CONSERVATIVE":
        # high_order_godunov.py:282-296: reconstruct the conservatives
        if case.recon != "WENO5-Z":
            raise NotImplementedError("CONSERVATIVE is restated for WENO5-Z")
        UL = reconstruct_xi(U, case, axis, 0)
        UR = reconstruct_xi(U, case, axis, 1)
        PL, PR = prims_from_cons(UL, g), prims_from_cons(UR, g)
    elif case.recon_var == "CHAR-CONSERVATIVE":
        # high_order_godunov.py:404-416: window of conservatives to
        # characteristics with the face's left eigenvectors, WENO on each,
        # back with the right eigenvectors
        if case.recon != "WENO5-Z":
            raise NotImplementedError("CHAR-CONSERVATIVE is restated for WENO5-Z")
        Rm, Lm = eigvecs_conservatives(P, case, axis)
        win = [U[_stencil_slice(case, axis, k)] for k in range(-3, 3)]
        chars = [_matvec5(Lm, [w[v] for v in range(5)]) for w in win]
        cL = [weno5z_stencil(*[chars[k][v] for k in (0, 1, 2, 3, 4)]) for v in range(5)]
        cR = [weno5z_stencil(*[chars[k][v] for k in (5, 4, 3, 2, 1)]) for v in range(5)]
        UL = torch.stack(_matvec5(Rm, cL), 0)
        UR = torch.stack(_matvec5(Rm, cR), 0)
        PL, PR = prims_from_cons(UL, g), prims_from_cons(UR, g)
    else:
        raise NotImplementedError(case.recon_var)
    if case.interpolation_limiter:
        # high_order_godunov.py:163-175; the limiter returns the conservatives
        # of its primitives (limiter_interpolation.py:206)
        PL = limit_interpolation(P, PL, case, axis, 0)
        PR = limit_interpolation(P, PR, case, axis, 1)
        UL = UR = None
    if UL is None:
        UL = cons_from_prims(PL, g)
        UR = cons_from_prims(PR, g)
    return riemann(PL, PR, UL, UR, case, axis)


# precision.py:54 (double precision): interpolation limiter epsilons
LIMITER_EPS_DENSITY = 1e-12
LIMITER_EPS_PRESSURE = 1e-10


def limit_interpolation(P: Tensor, Pj: Tensor, case: OracleCase, axis: int, j: int) -> Tensor:
    """PositivityLimiterInterpolation.limit_interpolation_xi, SINGLE-PHASE
    (limiter_interpolation.py:82-125, :170-188, apply_limiter :66-74): where
    the reconstructed density is below eps, then where the pressure (+ the
    ideal gas' zero background pressure) is below eps, the first-order value
    (WENO1, weno1_js.py: the cell left of the face for j = 0, right for
    j = 1) replaces density and pressure, or every primitive with
    limit_velocity, as x (1 - mask) + x1 mask."""
    w1 = P[_stencil_slice(case, axis, -1 if j == 0 else 0)]
    ids = list(range(5)) if case.limit_velocity else [0, 4]
    for check in range(2):
        if check == 0:
            mask = (Pj[0] < LIMITER_EPS_DENSITY).to(P.dtype)
        else:
            mask = (Pj[4] + 0.0 < LIMITER_EPS_PRESSURE).to(P.dtype)
        rows = [Pj[v] * (1 - mask) + w1[v] * mask if v in ids else Pj[v] for v in range(5)]
        Pj = torch.stack(rows, 0)
    return Pj


# ---------------------------------------------------------------------------
# Viscous flux (CENTRAL4), source_term_solver.py
# ---------------------------------------------------------------------------

# jnp.array([...]) / c coefficient arrays of the CENTRAL4 stencils
_C12 = (1.0 / 12.0, 8.0 / 12.0)      # derivative/deriv_center_4.py:35
_C24 = (1.0 / 24.0, 27.0 / 24.0)     # derivative/deriv_face_4.py:35
_C16 = (-1.0 / 16.0, 9.0 / 16.0)     # reconstruction/central/central_4.py:37


def _ring_slices(case: OracleCase, n: int, axis: int, lo: int, hi: Optional[int]) -> Tuple[slice, ...]:
    sl = [slice(None)] + [slice(n, -n) if case.cells[a] > 1 else slice(None) for a in range(3)]
    sl[axis + 1] = slice(lo, hi)
    return tuple(sl)


def _recon_halos(case: OracleCase) -> int:
    # required_halos of the reconstruction stencil (central_4.py / central_2.py)
    return 2 if case.diss_recon == "CENTRAL4" else 1


def _deriv_center_ring(buf: Tensor, case: OracleCase, axis_i: int) -> Tensor:
    """Centre derivative with offset (deriv_center_4.py:37-49, deriv_center_2.py:33-44).

    Built with offset = the reconstruction stencil's required halos
    (source_term_solver.py:63-71): the result covers the interior plus a ring
    of that many cells on every active axis.
    """
    n = case.nh - _recon_halos(case)

    def sl(k):
        hi = -n + k   # nhi = -n + k + 1 - at_cell_center
        return _ring_slices(case, n, axis_i, n + k, hi if hi != 0 else None)
    if case.diss_deriv_center == "CENTRAL2":
        # 1.0 / dxi * coeffs[0] * (u[i+1] - u[i-1]), coeffs = (1/2,)
        return 1.0 / case.cell_size(axis_i) * 0.5 * (buf[sl(1)] - buf[sl(-1)])
    return 1.0 / case.cell_size(axis_i) * (_C12[0] * (buf[sl(-2)] - buf[sl(2)]) + _C12[1] * (buf[sl(1)] - buf[sl(-1)]))


def _recon4_from_ring(ring: Tensor, case: OracleCase, axis_j: int) -> Tensor:
    """Reconstruction stencil built with nh = its halo width on the ring array
    (central_4.py:39-50, central_2.py:30-41)."""
    n = _recon_halos(case)

    def sl(k):
        hi = -n + k + 1
        return _ring_slices(case, n, axis_j, n + k, hi if hi != 0 else None)
    if case.diss_recon == "CENTRAL2":
        return 0.5 * (ring[sl(-1)] + ring[sl(0)])
    return _C16[0] * (ring[sl(-2)] + ring[sl(1)]) + _C16[1] * (ring[sl(-1)] + ring[sl(0)])


def _recon4(buf: Tensor, case: OracleCase, axis: int) -> Tensor:
    # reconstruct_stencil_ui (central_4.py:39-50, central_2.py:30-41) on the halo buffer
    if case.diss_recon == "CENTRAL2":
        s = [buf[_stencil_slice(case, axis, k)] for k in (-1, 0)]
        return 0.5 * (s[0] + s[1])
    s = [buf[_stencil_slice(case, axis, k)] for k in (-2, -1, 0, 1)]
    return _C16[0] * (s[0] + s[3]) + _C16[1] * (s[1] + s[2])


def _deriv_face(buf: Tensor, case: OracleCase, axis: int) -> Tensor:
    # derivative_stencil_face (deriv_face_4.py:37-50, deriv_face_2.py:30-45)
    if case.diss_deriv_face == "CENTRAL2":
        s = [buf[_stencil_slice(case, axis, k)] for k in (-1, 0)]
        return (1.0 / case.cell_size(axis)) * (s[1] - s[0])
    s = [buf[_stencil_slice(case, axis, k)] for k in (-2, -1, 0, 1)]
    return 1.0 / case.cell_size(axis) * (_C24[0] * (s[0] - s[3]) + _C24[1] * (s[2] - s[1]))


def viscous_flux_xi(P: Tensor, case: OracleCase, axis: int) -> Tensor:
    """compute_viscous_flux_xi for a constant viscosity (source_term_solver.py:264-350).

    vel_grad[a][b] = d u_a / d x_b at the faces of ``axis``: the normal
    derivative by the face stencil, tangential ones as centre derivatives
    interpolated to the face (compute_xi_derivatives_at_xj :538-580);
    tau (compute_tau :504-536); energy flux sum_k tau_k u_k at the face.
    Returns [tau_x, tau_y, tau_z, sum tau_k u_k] at the faces.
    """
    vel = P[1:4]
    shape = _deriv_face(vel, case, axis).shape[1:]
    zeros = torch.zeros(shape, dtype=P.dtype)
    g = [[zeros] * 3 for _ in range(3)]
    for i in range(3):
        if i not in case.active:
            continue
        if i == axis:
            d = _deriv_face(vel, case, i)
        else:
            d = _recon4_from_ring(_deriv_center_ring(vel, case, i), case, axis)
        for a in range(3):
            g[a][i] = d[a]
    mu1 = case.mu
    mu2 = case.bulk_viscosity - 2.0 / 3.0 * case.mu
    tau = []
    for k in range(3):
        if axis in case.active and k in case.active:
            tau.append(mu1 * (g[axis][k] + g[k][axis]))
        else:
            tau.append(zeros)
    tr = sum([g[k][k] for k in case.active])
    tau[axis] = tau[axis] + mu2 * tr
    velf = _recon4(vel, case, axis)
    if case.viscous_heat_production:
        vt = 0.0
        for k in case.active:
            vt = vt + tau[k] * velf[k]
    else:
        vt = zeros
    return torch.stack(tau + [vt], 0)


def heat_flux_xi(P: Tensor, case: OracleCase, axis: int) -> Tensor:
    """compute_heat_flux_xi (source_term_solver.py:188-254): -kappa dT/dx at the faces.

    T = p / (rho R) (ideal_gas.py:81-83) on the halo buffer.
    """
    T = (P[4] / (P[0] * case.R)).unsqueeze(0)
    return -case.kappa() * _deriv_face(T, case, axis)[0]


# ---------------------------------------------------------------------------
# Right-hand side, halos, time integration, dt
# ---------------------------------------------------------------------------

def compute_rhs(U: Tensor, P: Tensor, case: OracleCase) -> Tensor:
    """SpaceSolver.compute_rhs for the single-phase convective (+viscous) path.

    space_solver.py:151-453 (axis loop :289-314), compute_rhs_xi :456-674:
    flux = 0 + F_conv (+ -F_visc), rhs_xi = 0 + (1/dx)(F[:-1] - F[1:]),
    rhs = ((0.0 + rhs_x) + rhs_y) + rhs_z.
    """
    rhs = None
    for axis in case.active:
        if case.convective:
            flux = convective_flux_xi(P, case, axis, U)
        else:
            # space_solver.py:510: flux_xi = zeros(flux_shapes[axis])
            flux = torch.zeros((5,) + _deriv_face(P[:1], case, axis).shape[1:], dtype=P.dtype)
        if case.viscous:
            # space_solver.py:565-573: flux.at[1:5].add(-visc)
            visc = viscous_flux_xi(P, case, axis)
            flux = torch.cat([flux[:1], flux[1:] + (-visc)], 0)
        if case.heat:
            # space_solver.py:577-585: flux.at[4].add(heat_flux)
            flux = torch.cat([flux[:4], (flux[4] + heat_flux_xi(P, case, axis)).unsqueeze(0)], 0)
        sl_lo = [slice(None)] * 4
        sl_hi = [slice(None)] * 4
        sl_lo[axis + 1] = slice(None, -1)
        sl_hi[axis + 1] = slice(1, None)
        rhs_xi = case.one_cell_size(axis) * (flux[tuple(sl_lo)] - flux[tuple(sl_hi)])
        rhs = rhs_xi if rhs is None else rhs + rhs_xi
    if case.gravity is not None:
        rhs = rhs + gravity_forces(U[case.interior()], case)
    return rhs


def gravity_forces(Ui: Tensor, case: OracleCase) -> Tensor:
    """compute_gravity_forces (source_term_solver.py:165-186) added to
    rhs[1:5] (space_solver.py:377-384): momentum g_i rho, energy g . (rho u)
    summed in axis order; zero for the density."""
    g = [float(x) for x in case.gravity]
    mom = [g[i] * Ui[0] for i in range(3)]
    energy = (g[0] * Ui[1] + g[1] * Ui[2]) + g[2] * Ui[3]
    return torch.stack([torch.zeros_like(Ui[0])] + mom + [energy], 0)


def _face_fill_slice(case: OracleCase, face: str) -> Tuple[slice, ...]:
    # halos/halo_slices.py:46-75 (east = +x end [-nh:], west = [:nh])
    axis = FACE_AXIS[face]
    nh = case.nh
    s = slice(-nh, None) if face in ("east", "north", "top") else slice(None, nh)
    return _axis_slice(case, axis, s)


def _face_retrieve_slice(case: OracleCase, face: str, btype: str) -> Tuple[slice, ...]:
    # halos/outer/boundary_condition.py:539-604
    axis = FACE_AXIS[face]
    nh = case.nh
    hi = face in ("east", "north", "top")
    if btype == "PERIODIC":
        s = slice(nh, 2 * nh) if hi else slice(-2 * nh, -nh)
    elif btype in ("ZEROGRADIENT", "NEUMANN"):
        s = slice(-nh - 1, -nh) if hi else slice(nh, nh + 1)
    elif btype in ("SYMMETRY", "WALL"):
        # reference: [-nh-1:-2nh-1:-1] (hi) and [2nh-1:nh-1:-1] (lo); torch has no
        # negative steps, so return the forward slice and let the caller flip it
        s = slice(-2 * nh, -nh) if hi else slice(nh, 2 * nh)
    else:
        raise NotImplementedError(btype)
    return _axis_slice(case, axis, s)


# UPWIND DIRECTION FOR NEUMANN DERIVATIVE STENCIL (outer/material.py:41-44)
NEUMANN_SIGN = {"east": -1, "west": 1, "north": -1, "south": 1, "top": -1, "bottom": 1}


def _face_value_tensor(case: OracleCase, face: str, vals, dtype) -> Tensor:
    """Boundary values as a tensor [k, 1 along the face's axis, tangential
    extents]: constants, or an array [k, boundary cells] of the callables'
    values at the boundary cells (the later tangential axis fastest)."""
    axis = FACE_AXIS[face]
    if isinstance(vals, (tuple, list)):
        return torch.tensor([float(x) for x in vals], dtype=dtype).reshape(len(vals), 1, 1, 1)
    arr = torch.as_tensor(vals, dtype=dtype)
    dims = [case.cells[i] if i != axis else 1 for i in range(3)]
    return arr.reshape([arr.shape[0]] + dims)


def _face_halo(P: Tensor, case: OracleCase, face: str, btype: str, vals=None) -> Tensor:
    """Halo primitives of one face (outer/material.py:140-210): miscellaneous
    (:868-894) for PERIODIC / SYMMETRY / ZEROGRADIENT, wall (:473-531),
    dirichlet (:732-798), neumann (:825-866); values constant or per
    boundary cell."""
    axis = FACE_AXIS[face]
    fill_shape = P[_face_fill_slice(case, face)].shape
    if vals is None:
        vals = case.bc_values.get(face)
    if btype == "DIRICHLET":
        return _face_value_tensor(case, face, vals, P.dtype).expand(fill_shape).clone()
    h = P[_face_retrieve_slice(case, face, btype)].clone()
    if btype in ("SYMMETRY", "WALL"):
        h = torch.flip(h, dims=(axis + 1,))
    if btype == "SYMMETRY":
        sign = torch.ones(5, dtype=P.dtype).reshape(5, 1, 1, 1)
        sign[axis + 1] = -1.0
        h = h * sign
    elif btype == "WALL":
        # u_halo = 2 u_wall - u_mirror for every velocity component (:511-513)
        uw = 2 * _face_value_tensor(case, face, vals, P.dtype)
        h = torch.cat([h[0:1], uw[0:1] - h[1:2], uw[1:2] - h[2:3], uw[2:3] - h[3:4], h[4:5]])
    elif btype == "NEUMANN":
        # neumann_value *= sign; neumann_value *= dx; halo = P + neumann_value (:860-862)
        off = _face_value_tensor(case, face, vals, P.dtype) * NEUMANN_SIGN[face]
        off = off * case.cell_size(axis)
        h = h + off
    if h.shape != fill_shape:  # one retrieved layer fills all nh layers
        h = h.expand(fill_shape).clone()
    return h


def halo_update(P: Tensor, U: Optional[Tensor], case: OracleCase,
                t: float = 0.0) -> Tuple[Tensor, Optional[Tensor]]:
    """HaloManager.perform_halo_update_material, face halos (outer/material.py:94-287).

    Halo primitives follow each face's boundary rule; halo conservatives are
    recomputed from the halo primitives (:248-250).  The reference writes
    them as ``x.at[fill].mul(0).add(h)``, i.e. a plain set.  Edge halos
    follow when viscous or heat fluxes are on (halo_manager.py:126-129).
    """
    P = P.clone()
    U = U.clone() if U is not None else None
    for face in FACES:
        axis = FACE_AXIS[face]
        if axis not in case.active:
            continue
        fill = _face_fill_slice(case, face)
        if isinstance(case.bc[face], (list, tuple)):
            # several types on the face: each type's halos written through its
            # bounding-domain mask, x.at[fill].mul(1 - mask).add(h * mask)
            # (material.py:252-276)
            for btype, vals, mask in case.bc[face]:
                h = _face_halo(P, case, face, btype, vals)
                m = torch.as_tensor(mask, dtype=P.dtype)
                m = m.reshape([1] + [case.cells[i] if i != axis else 1 for i in range(3)])
                P[fill] = P[fill] * (1 - m) + h * m
                if U is not None:
                    U[fill] = U[fill] * (1 - m) + cons_from_prims(h, case.gamma) * m
            continue
        # callables of time are evaluated at the halo update's time (material.py:740-798)
        vals = case.bc_time[face](t) if face in case.bc_time else None
        h = _face_halo(P, case, face, case.bc[face], vals)
        P[fill] = h
        if U is not None:
            U[fill] = cons_from_prims(h, case.gamma)
    if case.viscous or case.heat:
        P, U = edge_halo_update(P, U, case)
    return P, U


def _rows(case: OracleCase, axis: int, kind: str, hi: bool) -> slice:
    """Buffer rows along `axis` (halo_slices.py:77-149 edge slices, in
    logical terms): the halo layers of one side, their periodic images, the
    interior rows a symmetry mirrors them from (forward order; the caller
    flips), or the interior rows nh cells inward (the '_10' / '_01' slices)."""
    n, nh = case.cells[axis], case.nh
    if kind == "halo":
        return slice(n + nh, n + 2 * nh) if hi else slice(0, nh)
    if kind == "wrap":
        return slice(nh, 2 * nh) if hi else slice(n, n + nh)
    if kind in ("mirror", "shift"):
        return slice(n, n + nh) if hi else slice(nh, 2 * nh)
    raise ValueError(kind)


def edge_halo_update(P: Tensor, U: Optional[Tensor], case: OracleCase):
    """MaterialBoundaryCondition.edge_halo_update / compute_edge_halos
    (outer/material.py:289-379) with the type combinations of
    boundary_condition.py:128-177 and :606-660: along the edge's faces in
    axis order, the first PERIODIC or SYMMETRY face decides (its periodic
    image, or its mirror with that axis' velocity negated, of the other
    face's halo); otherwise (ANY_ANY) the mean of the two face halos nh
    cells inward.  Vertex halos are not filled (single phase,
    halo_manager.py:131-143); conservatives are recomputed for the edge
    cells only.
    """
    P = P.clone()
    U = U.clone() if U is not None else None
    act = case.active
    for ia in range(len(act)):
        for ib in range(ia + 1, len(act)):
            a, b = act[ia], act[ib]
            c = [i for i in range(3) if i not in (a, b)][0]
            for hia in (False, True):
                for hib in (False, True):
                    fa = AXIS_FACES[a][1 if hia else 0]
                    fb = AXIS_FACES[b][1 if hib else 0]
                    ta, tb = case.bc[fa], case.bc[fb]

                    def block(ra, rb):
                        sl = [slice(None)] * 4
                        sl[a + 1], sl[b + 1], sl[c + 1] = ra, rb, case.inner(c)
                        return tuple(sl)

                    target = block(_rows(case, a, "halo", hia), _rows(case, b, "halo", hib))
                    if ta in ("PERIODIC", "SYMMETRY"):
                        ax, t, hi_ = a, ta, hia
                        src_blk = block(_rows(case, a, "wrap" if ta == "PERIODIC" else "mirror", hia),
                                        _rows(case, b, "halo", hib))
                    elif tb in ("PERIODIC", "SYMMETRY"):
                        ax, t, hi_ = b, tb, hib
                        src_blk = block(_rows(case, a, "halo", hia),
                                        _rows(case, b, "wrap" if tb == "PERIODIC" else "mirror", hib))
                    else:
                        t = "ANY"
                    if t == "ANY":
                        A = P[block(_rows(case, a, "shift", hia), _rows(case, b, "halo", hib))]
                        B = P[block(_rows(case, a, "halo", hia), _rows(case, b, "shift", hib))]
                        h = 0.5 * (A + B)
                    else:
                        h = P[src_blk].clone()
                        if t == "SYMMETRY":
                            h = torch.flip(h, dims=(ax + 1,))
                            sign = torch.ones(5, dtype=P.dtype).reshape(5, 1, 1, 1)
                            sign[ax + 1] = -1.0
                            h = h * sign
                    P[target] = h
                    if U is not None:
                        U[target] = cons_from_prims(h, case.gamma)
    return P, U


RK3_DT_MULT = (1.0, 0.25, 2.0 / 3.0)                 # RK3.py:27
RK3_CONS_MULT = ((0.25, 0.75), (2.0 / 3.0, 1.0 / 3.0))  # RK3.py:29


def rk3_stage_update(U: Tensor, Un: Tensor, rhs: Tensor, dt, stage: int, case: OracleCase) -> Tensor:
    """TimeIntegrator.perform_stage_integration (time_integrator.py:108-226, RK3.py:31-62)."""
    if stage > 0:
        a, b = RK3_CONS_MULT[stage - 1]
        U = a * U + b * Un
    ts = dt * RK3_DT_MULT[stage]
    U = U.clone()
    inner = case.interior()
    U[inner] = U[inner] + ts * rhs
    return U


RK3_TIME_INCREMENT = (1.0, 0.5, 1.0)                 # RK3.py:28


def rk3_step(U: Tensor, P: Tensor, dt, case: OracleCase, t: float = 0.0) -> Tuple[Tensor, Tensor]:
    """One TVD-RK3 step (simulation_manager.py:670-1077); the halos after stage
    k are filled at t + dt * timestep_increment_factor[k] (:855-857)."""
    Un = U
    for stage in range(3):
        rhs = compute_rhs(U, P, case)
        U = rk3_stage_update(U, Un, rhs, dt, stage, case)
        P = prims_from_cons(U, case.gamma)          # simulation_manager.py:943-944
        P, U = halo_update(P, U, case, t + float(dt) * RK3_TIME_INCREMENT[stage])  # :961-970
    return U, P


def compute_dt(P: Tensor, case: OracleCase) -> Tensor:
    """compute_time_step_size (time_integration/time_step_size.py:15-157)."""
    if case.fixed_dt:
        return torch.tensor(case.fixed_dt, dtype=torch.float64)
    Pi = P[case.interior()]
    rho = Pi[0]
    c = speed_of_sound(Pi[4], rho, case.gamma)
    abs_vel = 0.0
    for i in case.active:
        abs_vel = abs_vel + (torch.abs(Pi[i + 1]) + c)
    dt = rdiv(case.min_cell_size, torch.max(abs_vel) + EPS)
    if case.viscous:
        nu = rdiv(case.mu, rho)
        dt_v = rdiv(3.0 / 14.0 * (case.min_cell_size * case.min_cell_size), torch.max(nu) + EPS)
        dt = torch.minimum(dt, dt_v)
    if case.heat:
        alpha = rdiv(case.kappa(), rho * case.cp())
        dt_h = rdiv(0.1 * (case.min_cell_size * case.min_cell_size), torch.max(alpha) + EPS)
        dt = torch.minimum(dt, dt_h)
    return dt * case.cfl


def initialize(prims_interior: Tensor, case: OracleCase, inactive_velocity_eps: bool = True) -> Tuple[Tensor, Tensor]:
    """MaterialFieldsInitializer.create_material_fields (material_fields_initializer.py:148-210).

    The buffer starts as eps everywhere (initialization/helper_functions.py:49-60);
    the interior is set from the initial primitives; inactive velocity
    components keep eps unless the caller passes all five components
    (``feed_forward.py`` sets all five).
    """
    shape = case.buffer_shape()
    P = torch.ones(shape, dtype=torch.float64) * EPS
    inner = case.interior()
    if prims_interior.shape[0] == 5:
        P[inner] = prims_interior
    else:
        ids = [0] + [1 + i for i in case.active] + [4]
        for k, idx in enumerate(ids):
            P[(idx,) + inner[1:]] = prims_interior[k]
    U = cons_from_prims(P, case.gamma)
    P, U = halo_update(P, U, case)
    return U, P


def buffers_from_interior_cons(Uint: Tensor, case: OracleCase) -> Tuple[Tensor, Tensor]:
    """Halo buffers (U, P) of an interior conservative state: primitives from
    the conservatives, halos filled (the state after a stage, simulation_manager.py:943-970)."""
    P = torch.ones(case.buffer_shape(), dtype=torch.float64) * EPS
    P = P.clone()
    P[case.interior()] = prims_from_cons(Uint, case.gamma)
    U = cons_from_prims(P, case.gamma)
    U = U.clone()
    U[case.interior()] = Uint
    return tuple(reversed(halo_update(P, U, case)))


def rhs_of_interior_cons(Uint: Tensor, case: OracleCase) -> Tensor:
    """compute_rhs as a function of the interior conservatives (for autograd)."""
    U, P = buffers_from_interior_cons(Uint, case)
    return compute_rhs(U, P, case)


def rk3_step_interior(Uint: Tensor, dt, case: OracleCase) -> Tensor:
    """One fixed-dt TVD-RK3 step as a function of the interior conservatives."""
    U, P = buffers_from_interior_cons(Uint, case)
    U, P = rk3_step(U, P, dt, case)
    return U[case.interior()]


def simulate(U: Tensor, P: Tensor, case: OracleCase, end_time: float = None, end_step: int = None,
             t0: float = 0.0, log=None):
    """SimulationManager.advance (simulation_manager.py:297-425) without output.

    ``while t < end_time and step < end_step``; dt is computed from the state at
    the start of each step and not clipped to end_time.
    """
    t = t0
    step = 0
    dt = compute_dt(P, case)
    if log is not None:
        log.append((t, float(dt), float(P[case.interior()][0].min())))
    end_time = math.inf if end_time is None else end_time
    end_step = 1 << 62 if end_step is None else end_step
    while t < end_time and step < end_step:
        U, P = rk3_step(U, P, dt, case)
        t = t + float(dt)
        step += 1
        dt = compute_dt(P, case)
        if log is not None:
            log.append((t, float(dt), float(P[case.interior()][0].min())))
    return U, P, t, step
