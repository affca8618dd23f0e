"""Properties the full-size GPU tests rely on, shown on the oracle at sizes it
finishes in seconds: RK3 steps of the Taylor-Green vortex commute with the
reflection x <-> y (cells (i, j, k) -> (j, i, k), u <-> v), and the periodic
finite-volume update conserves mass, momentum and energy to rounding.  The
reflected run is compared bitwise: the per-cell arithmetic is the same up to
the order of commutative additions."""
import math

import pytest
import torch

from oracle import jf_oracle as O
from tests.cases import assert_conserved, both, reflect_xy, tgv_prims

CASES = [
    ("weno5z-hllc", (12, 12, 10), 3, {}),
    ("char-roe-viscous-heat", (10, 10, 8), 2, dict(nh=4, recon_var="CHAR-PRIMITIVE", frozen_state="ROE",
                                                   viscous=True, heat=True, mu=1.0 / 1600, prandtl=0.71)),
]


@pytest.mark.parametrize("name,cells,steps,kw", CASES, ids=[c[0] for c in CASES])
def test_oracle_steps_commute_with_reflection_and_conserve(name, cells, steps, kw):
    oc, _ = both(cells, "PERIODIC", ranges=((0, 2 * math.pi),) * 3, **kw)
    prims = tgv_prims(max(cells))[:, :cells[0], :cells[1], :cells[2]].contiguous()
    runs = []
    for P0 in (prims, reflect_xy(prims)):
        U, P = O.initialize(P0, oc)
        U0 = U[oc.interior()].clone()
        t = 0.0
        for _ in range(steps):
            dt = O.compute_dt(P, oc)
            U, P = O.rk3_step(U, P, dt, oc)
            t += dt.item()
        runs.append((U0, U[oc.interior()], t))
    (U0, UK, t), (V0, VK, s) = runs
    assert t == s
    assert torch.equal(reflect_xy(UK), VK)
    assert_conserved(U0, UK)
    assert_conserved(V0, VK)
