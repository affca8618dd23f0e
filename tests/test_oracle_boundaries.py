"""The oracle's boundary restatements that have no fixture in the reference:
a face of several types (bounding_domain masks, halos/outer/material.py:252-276)
is the per-cell selection of the single-type halos, and boundary values given
per boundary cell reproduce the constant-value halos when they are constant."""
import numpy as np
import pytest
import torch

from oracle import jf_oracle as O
from tests.cases import both, quadrant_prims

CELLS = (20, 16, 1)
STATE = (1.3, 0.2, -0.1, 0.0, 0.9)


def _faces(south):
    return {"west": "ZEROGRADIENT", "east": "ZEROGRADIENT", "north": "ZEROGRADIENT", "south": south,
            "top": "PERIODIC", "bottom": "PERIODIC"}


def _halos(bc, vals, **kw):
    oc, _ = both(CELLS, bc, bc_values=vals, **kw)
    return O.initialize(quadrant_prims(*CELLS[:2], seed=7), oc)


@pytest.mark.parametrize("viscous", [False, True])
def test_face_of_several_types_selects_per_cell(viscous):
    kw = dict(nh=4, viscous=True, mu=0.01) if viscous else {}
    x = (np.arange(CELLS[0]) + 0.5) / CELLS[0]
    mask = x < 0.4
    U, P = _halos(_faces([("DIRICHLET", STATE, mask), ("SYMMETRY", None, ~mask)]), {}, **kw)
    Ud, Pd = _halos(_faces("DIRICHLET"), {"south": STATE}, **kw)
    Us, Ps = _halos(_faces("SYMMETRY"), {}, **kw)
    nh = 4 if viscous else 3
    sel = torch.as_tensor(mask).reshape(1, -1, 1, 1)
    # south face halo rows: y in [0, nh), x over the interior
    blk = (slice(None), slice(nh, -nh), slice(0, nh), slice(None))
    assert torch.equal(P[blk], torch.where(sel, Pd[blk], Ps[blk]))
    assert torch.equal(U[blk], torch.where(sel, Ud[blk], Us[blk]))


@pytest.mark.parametrize("btype,vals", [("DIRICHLET", STATE), ("WALL", (0.3, -0.2, 0.0)),
                                        ("NEUMANN", (0.1, -0.3, 0.2, 0.0, 0.5))])
def test_constant_fields_match_constants(btype, vals):
    nt = CELLS[0]
    field = np.repeat(np.asarray(vals, dtype=np.float64)[:, None], nt, axis=1)
    U, P = _halos(_faces(btype), {"south": field})
    Uc, Pc = _halos(_faces(btype), {"south": vals})
    assert torch.equal(P, Pc) and torch.equal(U, Uc)
