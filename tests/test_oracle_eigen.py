"""The oracle's conservative eigendecomposition (eigendecomposition.py:576-662,
Fedkiw et al. 1999) is a left/right pair: L R = I at every face, for both
frozen states and every axis; CHAR-CONSERVATIVE and CONSERVATIVE agree to the
order of the scheme on smooth data."""
import math

import pytest
import torch

from oracle import jf_oracle as O
from tests.cases import both, generic_cons


@pytest.mark.parametrize("frozen", ["ARITHMETIC", "ROE"])
@pytest.mark.parametrize("axis", [0, 1, 2])
def test_left_right_eigenvectors_are_inverse(frozen, axis):
    cells = (8, 9, 10)
    oc, _ = both(cells, "PERIODIC", frozen_state=frozen)
    U, P = O.buffers_from_interior_cons(generic_cons(cells, seed=2), oc)
    Rm, Lm = O.eigvecs_conservatives(P, oc, axis)
    for i in range(5):
        for k in range(5):
            prod = sum(Lm[i][j] * Rm[j][k] for j in range(5))
            torch.testing.assert_close(prod, torch.full_like(prod, float(i == k)), rtol=0, atol=1e-12)


def _rhs(n, recon_var):
    x = (torch.arange(n, dtype=torch.float64) + 0.5) / n
    prims = torch.stack([1.0 + 0.2 * torch.sin(2 * math.pi * x), 0.5 + 0.1 * torch.cos(2 * math.pi * x),
                         1.0 + 0.1 * torch.sin(4 * math.pi * x)]).reshape(3, n, 1, 1)
    oc, _ = both((n, 1, 1), "PERIODIC", recon_var=recon_var, frozen_state="ROE")
    U, P = O.initialize(prims, oc)
    return O.compute_rhs(U, P, oc)


def test_char_conservative_converges_to_conservative_on_smooth_data():
    """Both reconstruct the same smooth field: their difference is a
    truncation error that falls at high order under refinement."""
    gaps = []
    for n in (32, 64):
        a, b = _rhs(n, "CHAR-CONSERVATIVE"), _rhs(n, "CONSERVATIVE")
        gaps.append(float((a - b).abs().max()) / float(b.abs().max()))
    assert gaps[1] < 1e-4
    assert gaps[0] / gaps[1] > 8.0  # at least third order
