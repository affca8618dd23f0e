"""Algorithmic FP64 operation count of one TVD-RK3 step, from the oracle.

TEST INFRASTRUCTURE ONLY (measurement bookkeeping): it executes the oracle,
which restates the reference's algorithm op for op, under a torch dispatch mode
that counts every float64 elementwise arithmetic operation by the number of
elements it produces:

* ``add`` (add/sub, incl. in-place and scalar forms), ``mul``, ``div``
  (including the oracle's single-rounding scalar division ``rdiv``), ``sqrt``
  (the oracle's correctly rounded square root, counted at its call), and
  integer powers (``x**2`` = one multiplication, TENO5's ``x**6`` = three);
* FLOP = add + mul + div + sqrt (one each, the usual convention);
* ``other``: comparisons, abs, sign, min/max, select (not FLOPs; reported).

The reference evaluates some operations on the whole halo buffer (the
primitives from the conservatives, the halo fill) and its face arrays are
N + 1 long, so the per-cell count of a finite grid carries a surface term.
``per_cell_update`` runs the TGV workload at several sizes and returns the
coefficient of n^3 of the exact cubic through the counts: the count per
interior cell-update of an unbounded grid.
"""
from __future__ import annotations

import math
from collections import Counter

import numpy as np
import torch
from torch.utils._python_dispatch import TorchDispatchMode

from oracle import jf_oracle as O

aten = torch.ops.aten

_ADD = {aten.add.Tensor, aten.add_.Tensor, aten.sub.Tensor, aten.sub_.Tensor, aten.rsub.Scalar,
        aten.add.Scalar, aten.sub.Scalar, aten.rsub.Tensor}
_MUL = {aten.mul.Tensor, aten.mul_.Tensor, aten.mul.Scalar}
_DIV = {aten.div.Tensor, aten.div_.Tensor, aten.div.Scalar, aten.reciprocal.default}
_OTHER = {aten.abs.default, aten.sign.default, aten.maximum.default, aten.minimum.default, aten.where.self,
          aten.gt.Tensor, aten.gt.Scalar, aten.lt.Tensor, aten.lt.Scalar, aten.ge.Tensor, aten.ge.Scalar,
          aten.le.Tensor, aten.le.Scalar, aten.eq.Tensor, aten.eq.Scalar, aten.neg.default, aten.clamp.default,
          aten.max.default, aten.min.default, aten.amax.default, aten.amin.default, aten.fmax.default,
          aten.fmin.default}


class _Count(TorchDispatchMode):
    def __init__(self):
        super().__init__()
        self.c = Counter()

    def __torch_dispatch__(self, func, types, args=(), kwargs=None):
        out = func(*args, **(kwargs or {}))
        if isinstance(out, torch.Tensor) and out.dtype == torch.float64:
            n = out.numel()
            base = func.overloadpacket
            if func in _ADD:
                self.c["add"] += n
            elif func in _MUL:
                self.c["mul"] += n
            elif func in _DIV:
                self.c["div"] += n
            elif base is aten.pow:
                e = args[1] if len(args) > 1 else None
                if isinstance(e, (int, float)) and float(e).is_integer() and e >= 1:
                    k = int(e)
                    self.c["mul"] += n * (k.bit_length() - 1 + bin(k).count("1") - 1)
                else:
                    self.c["pow"] += n
            elif func in _OTHER or base in (aten.abs, aten.where, aten.maximum, aten.minimum, aten.sign):
                self.c["other"] += n
        return out


def count_step(n: int, case_kw: dict, prims_fn) -> Counter:
    """Counts of one RK3 step plus the next time step on an n^3 case."""
    case = O.OracleCase(cells=(n, n, n), **case_kw)
    U, P = O.initialize(prims_fn(n), case)
    dt = O.compute_dt(P, case)
    counter = _Count()
    sqrt_calls = Counter()
    orig = O.sqrt

    def counting_sqrt(x):
        sqrt_calls["sqrt"] += x.numel()
        return orig(x)

    O.sqrt = counting_sqrt
    try:
        with counter:
            U, P = O.rk3_step(U, P, dt, case)
            O.compute_dt(P, case)
    finally:
        O.sqrt = orig
    c = counter.c
    c["sqrt"] += sqrt_calls["sqrt"]
    c["flop"] = c["add"] + c["mul"] + c["div"] + c["sqrt"]
    return c


def tgv_prims(n):
    x = (torch.arange(n, dtype=torch.float64) + 0.5) * (2 * math.pi / n)
    X, Y, Z = torch.meshgrid(x, x, x, indexing="ij")
    p = 1.0 / (1.4 * 0.01) + (torch.cos(2 * X) + torch.cos(2 * Y)) * (torch.cos(2 * Z) + 2.0) / 16.0
    return torch.stack([torch.ones_like(X), torch.sin(X) * torch.cos(Y) * torch.cos(Z),
                        -torch.cos(X) * torch.sin(Y) * torch.cos(Z), torch.zeros_like(X), p])


TGV = dict(ranges=((0.0, 2 * math.pi),) * 3, nh=3, bc={f: "PERIODIC" for f in O.FACES}, recon="WENO5-Z",
           riemann="HLLC", signal_speed="EINFELDT", cfl=0.5)
VISCOUS_TGV = dict(ranges=((0.0, 2 * math.pi),) * 3, nh=4, bc={f: "PERIODIC" for f in O.FACES},
                   recon="WENO5-Z", recon_var="CHAR-PRIMITIVE", frozen_state="ROE", riemann="HLLC",
                   signal_speed="EINFELDT", cfl=0.5, viscous=True, heat=True, mu=1.0 / 1600, prandtl=0.71)


def per_cell_update(case_kw: dict = TGV, sizes=(8, 10, 12, 14)) -> dict:
    """Counts per interior cell-update of an unbounded grid: the n^3
    coefficient of the cubic through the counts at four sizes."""
    keys = ("add", "mul", "div", "sqrt", "flop", "other")
    counts = [count_step(n, case_kw, tgv_prims) for n in sizes]
    A = np.array([[n ** 3, n ** 2, n, 1.0] for n in sizes])
    out = {}
    for k in keys:
        coef = np.linalg.solve(A, np.array([c[k] for c in counts], dtype=np.float64))
        out[k] = float(coef[0])
    return out


if __name__ == "__main__":
    torch.set_num_threads(1)
    for name, kw in (("TGV WENO5-Z + HLLC", TGV), ("viscous TGV CHAR-ROE + HLLC + CENTRAL4", VISCOUS_TGV)):
        r = per_cell_update(kw)
        print(name, {k: round(v, 1) for k, v in r.items()})
