"""The oracle's TENO5 (shock_capturing/teno/teno5.py) against closed forms:
on smooth data no stencil is cut and the face value is the linear d-weighted
combination; across a jump the stencils that contain it are cut and the
smooth stencil's polynomial remains."""
import torch

from oracle import jf_oracle as O


def _t(*v):
    return [torch.tensor([x], dtype=torch.float64) for x in v]


def test_smooth_data_keeps_every_stencil():
    u = _t(*[0.3 + 0.01 * k + 0.002 * k * k for k in range(5)])
    c = O._WENO_CR
    p = [c[0][0] * u[0] + c[0][1] * u[1] + c[0][2] * u[2],
         c[1][0] * u[1] + c[1][1] * u[2] + c[1][2] * u[3],
         c[2][0] * u[2] + c[2][1] * u[3] + c[2][2] * u[4]]
    lin = (0.05 * p[0] + 0.55 * p[1] + 0.40 * p[2]) / (1.0 + O.STENCIL_EPS)
    torch.testing.assert_close(O.teno5_stencil(*u), lin, rtol=1e-15, atol=0.0)


def test_jump_cuts_the_stencils_across_it():
    # left-biased value at the face after cell u2 = 0 with the jump between u2 and u3
    u = _t(0.0, 0.0, 0.0, 1.0, 1.0)
    assert float(O.teno5_stencil(*u)) == 0.0
    # the same jump one level up: only stencil 0 is kept, its polynomial
    # (1/3 - 7/6 + 11/6, rounded) with weight d0 / (d0 + eps) = 1
    u = _t(1.0, 1.0, 1.0, 0.0, 0.0)
    c = O._WENO_CR[0]
    assert float(O.teno5_stencil(*u)) == c[0] * 1.0 + c[1] * 1.0 + c[2] * 1.0
