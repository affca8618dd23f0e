"""Two independent CPU restatements of the reference agree bitwise: the plain-C
right-hand side (oracle/jf_rhs.c: WENO5-Z on primitives, HLLC with Einfeldt
speeds) against the torch oracle, on periodic, zero-gradient and symmetry
halos in 1-D to 3-D.  Built here with the system C compiler, contraction off."""
import ctypes
import os

import numpy as np
import pytest
import torch

from oracle import jf_oracle as O
from tests.cases import both, quadrant_prims, sod_prims, tgv_prims

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def crhs():
    import __graft_entry__
    so = __graft_entry__.build_oracle_c()  # oracle/_build/jf_rhs.so, rebuilt when the source is newer
    if not so:
        pytest.skip("no C compiler")
    lib = ctypes.CDLL(so)
    f = lib.jf_rhs_weno5z_hllc
    f.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                  ctypes.c_double, ctypes.c_double, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


CASES = [
    ("sod-1d", (120, 1, 1), "ZEROGRADIENT", "sod"),
    ("quad-2d-sym", (36, 28, 1), {"east": "ZEROGRADIENT", "west": "ZEROGRADIENT", "north": "SYMMETRY",
                                  "south": "SYMMETRY", "top": "PERIODIC", "bottom": "PERIODIC"}, "quad"),
    ("tgv-3d", (16, 12, 14), "PERIODIC", "tgv"),
]


@pytest.mark.parametrize("name,cells,bc,kind", CASES, ids=[c[0] for c in CASES])
def test_c_restatement_matches_torch_oracle(crhs, name, cells, bc, kind):
    oc, _ = both(cells, bc)
    if kind == "sod":
        prims = sod_prims(cells[0])
    elif kind == "quad":
        prims = quadrant_prims(cells[0], cells[1], seed=4)
    else:
        prims = tgv_prims(max(cells))[:, :cells[0], :cells[1], :cells[2]].contiguous()
    U, P = O.initialize(prims, oc)
    ref = O.compute_rhs(U, P, oc)
    Pn = np.ascontiguousarray(P.numpy())
    out = np.empty(ref.shape, dtype=np.float64)
    n = (ctypes.c_int * 3)(*cells)
    odx = (ctypes.c_double * 3)(*[oc.one_cell_size(a) if cells[a] > 1 else 0.0 for a in range(3)])
    assert crhs(Pn.ctypes.data, n, oc.nh, odx, oc.gamma, O.STENCIL_EPS, out.ctypes.data) == 0
    assert torch.equal(torch.from_numpy(out), ref)
