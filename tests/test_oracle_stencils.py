"""The oracle's dissipative stencils (CENTRAL4 and CENTRAL2 in every
combination of reconstruction, centre derivative and face derivative;
source_term_solver.py:57-118) against closed forms on polynomial fields: the
viscous and heat fluxes of linear fields are exact for every combination, and
a field quadratic along the face normal separates the two reconstructions."""
import itertools

import pytest
import torch

from oracle import jf_oracle as O
from tests.cases import both

STENCILS = list(itertools.product(("CENTRAL4", "CENTRAL2"), repeat=3))
MU, BULK = 0.03, 0.01


def _case(stencils, cells=(12, 10, 1)):
    recon, center, face = stencils
    nh = 4 if (recon, center) == ("CENTRAL4", "CENTRAL4") else 3
    oc, _ = both(cells, {f: "PERIODIC" for f in O.FACES}, nh=nh, viscous=True, heat=True, mu=MU,
                 bulk_viscosity=BULK, prandtl=0.71, diss_recon=recon, diss_deriv_center=center,
                 diss_deriv_face=face)
    return oc


def _coords(oc):
    """Cell-centre coordinates over the whole halo buffer, per axis."""
    xs = []
    for a in range(3):
        if oc.cells[a] > 1:
            n = oc.cells[a] + 2 * oc.nh
            xs.append((torch.arange(n, dtype=torch.float64) - oc.nh + 0.5) * oc.cell_size(a))
        else:
            xs.append(torch.zeros(1, dtype=torch.float64))
    return torch.meshgrid(*xs, indexing="ij")


def _face_coords(oc, axis):
    """Coordinates of the x-faces of the interior (axis 0), interior cells along y."""
    assert axis == 0
    n0, n1 = oc.cells[0], oc.cells[1]
    xf = torch.arange(n0 + 1, dtype=torch.float64) * oc.cell_size(0)
    yc = (torch.arange(n1, dtype=torch.float64) + 0.5) * oc.cell_size(1)
    return torch.meshgrid(xf, yc, indexing="ij")


def _prims(oc, u, v, T_slope=0.0):
    x, y, _ = _coords(oc)
    P = torch.zeros((5,) + tuple(x.shape), dtype=torch.float64)
    P[0] = 1.0
    P[1] = u(x, y)
    P[2] = v(x, y)
    P[4] = oc.R * (2.0 + T_slope * x)  # T = p / (rho R) linear in x
    return P


@pytest.mark.parametrize("stencils", STENCILS, ids=["-".join(s[-1] for s in st) for st in STENCILS])
def test_linear_fields_exact(stencils):
    oc = _case(stencils)
    a, b, c, d = 0.7, -0.4, 0.25, 1.3
    P = _prims(oc, lambda x, y: a * x + b * y, lambda x, y: c * x + d * y, T_slope=0.9)
    F = O.viscous_flux_xi(P, oc, 0)[..., 0]
    xf, yf = _face_coords(oc, 0)
    mu2 = BULK - 2.0 / 3.0 * MU
    tau_x = MU * (2 * a) + mu2 * (a + d)
    tau_y = MU * (b + c)
    uf, vf = a * xf + b * yf, c * xf + d * yf
    torch.testing.assert_close(F[0], torch.full_like(xf, tau_x), rtol=1e-12, atol=1e-12)
    torch.testing.assert_close(F[1], torch.full_like(xf, tau_y), rtol=1e-12, atol=1e-12)
    torch.testing.assert_close(F[3], tau_x * uf + tau_y * vf, rtol=1e-12, atol=1e-12)
    H = O.heat_flux_xi(P, oc, 0)[..., 0]
    torch.testing.assert_close(H, torch.full_like(xf, -oc.kappa() * 0.9), rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("recon", ["CENTRAL4", "CENTRAL2"])
def test_reconstruction_order_separates(recon):
    """u = x^2 y: d u / d y = x^2 at the cells; CENTRAL4 interpolates it to
    the face exactly, CENTRAL2 as the mean of the two neighbours, x_f^2 + dx^2/4."""
    oc = _case((recon, "CENTRAL2", "CENTRAL2"))
    P = _prims(oc, lambda x, y: x * x * y, lambda x, y: 0.0 * x)
    F = O.viscous_flux_xi(P, oc, 0)[..., 0]
    xf, yf = _face_coords(oc, 0)
    dx = oc.cell_size(0)
    g_xy = xf * xf + (dx * dx / 4.0 if recon == "CENTRAL2" else 0.0)
    # tau_y = mu (d u / d y + d v / d x), v = 0
    torch.testing.assert_close(F[1], MU * g_xy, rtol=1e-11, atol=1e-13)
