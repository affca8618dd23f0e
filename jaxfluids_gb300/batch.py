"""Batched fused TVD-RK3 of many independent cases of uneven size.

JAX-Fluids batches equal-size cases with ``jax.vmap`` over
``SimulationManager._feed_forward`` (simulation_manager.py:1248-1294).
``BatchedRK3`` advances cases of different grid sizes that share one scheme,
each with its own CFL time step, through ``gbf_batch_advance``: every RK stage
is the single-case fused stage (a face-kernel launch per active axis, then the
cell epilogue) over a (case, tile) work list, so a batch of small grids fills
the GPU the way one large grid does.  ``capture`` records a run of steps in a
CUDA graph; ``autotune`` picks the tile shape, threads per CTA and persistent
grid size by timing candidates on the batch itself.
"""
from __future__ import annotations

import ctypes
import time
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np
import torch

from . import _lib
from .config import CaseConfig
from .solver import _ptr, _stream

# layout of gbf_batch_case (include/gbfluids.h)
BATCH_CASE_DTYPE = np.dtype([("n", "<i4", 3), ("tiles", "<i4", 3), ("offset", "<i8"), ("dx", "<f8", 3)],
                            align=True)
assert BATCH_CASE_DTYPE.itemsize == 56

_SCHEME_KEYS = ("nh", "gamma", "R", "recon", "recon_var", "frozen_state", "riemann", "signal_speed",
                "cfl", "fixed_dt", "viscous", "heat", "eps", "stencil_eps")


def default_tile(dim: int) -> Tuple[int, int, int]:
    return {1: (256, 1, 1), 2: (16, 16, 1), 3: (8, 8, 8)}[dim]


def build_worklist(cells: Sequence[Tuple[int, int, int]], tile: Tuple[int, int, int]):
    """Case table fields and the (case, tile) work list, largest cases first.

    Returns (n, tiles, offsets, worklist, total_doubles) as numpy arrays; the
    packed state of case c starts at offsets[c] and holds 5 * cells(c) doubles.
    """
    n = np.asarray(cells, dtype=np.int64).reshape(-1, 3)
    t = np.array([tile[a] if np.any(n[:, a] > 1) else 1 for a in range(3)], dtype=np.int64)
    tiles = (n + t - 1) // t
    sizes = 5 * n.prod(axis=1)
    offsets = np.concatenate([[0], np.cumsum(sizes)[:-1]])
    order = np.argsort(-n.prod(axis=1), kind="stable")
    items = [(c, k) for c in order for k in range(int(tiles[c].prod()))]
    worklist = np.asarray(items, dtype=np.int32).reshape(-1, 2)
    return n.astype(np.int32), tiles.astype(np.int32), offsets.astype(np.int64), worklist, int(sizes.sum())


class BatchedRK3:
    def __init__(self, configs: List[CaseConfig], device="cuda", tile: Optional[Tuple[int, int, int]] = None,
                 threads: int = 256, ctas: int = 0):
        if not configs:
            raise ValueError("empty batch")
        c0 = configs[0]
        for c in configs[1:]:
            for k in _SCHEME_KEYS:
                if getattr(c, k) != getattr(c0, k):
                    raise ValueError(f"all cases of a batch share the scheme; '{k}' differs")
            if c.active != c0.active or c.bc != c0.bc:
                raise ValueError("all cases of a batch share active axes and boundary types")
        if c0.viscous or c0.heat or not c0.convective:
            raise NotImplementedError("the batched path is built for inviscid cases")
        if c0.riemann == "LAX-FRIEDRICHS" or c0.recon_var in ("CONSERVATIVE", "CHAR-CONSERVATIVE"):
            raise NotImplementedError(f"the batched path does not build {c0.riemann} / {c0.recon_var}")
        if c0.interpolation_limiter or c0.gravity is not None or any(c.has_bc_fields for c in configs):
            raise NotImplementedError("the batched path has no limiter, gravity or boundary value fields")
        self.configs = configs
        self.lib = _lib.load()
        self.device = torch.device(device)
        self.threads = threads
        self.ctas = ctas
        self._layout(tile or default_tile(c0.dim))
        self.cons = torch.zeros(self.total, dtype=torch.float64, device=self.device)
        self.dt_states = torch.zeros(4 * len(configs), dtype=torch.float64, device=self.device)
        nb = int(self.lib.gbf_batch_workspace_bytes(self.total))
        self.workspace = torch.empty(nb // 8, dtype=torch.float64, device=self.device)

    # ---- layout -----------------------------------------------------------
    def _layout(self, tile):
        cfgs = self.configs
        n, tiles, offsets, worklist, total = build_worklist([c.cells for c in cfgs], tile)
        table = np.zeros(len(cfgs), dtype=BATCH_CASE_DTYPE)
        table["n"] = n
        table["tiles"] = tiles
        table["offset"] = offsets
        table["dx"] = np.array([[c.cell_size(a) if c.cells[a] > 1 else 1.0 for a in range(3)] for c in cfgs])
        self.tile = tuple(int(x) for x in tile)
        self.offsets = offsets
        self.total = total
        self.ntiles = int(worklist.shape[0])
        self.case_table = torch.from_numpy(table.view(np.uint8).copy()).to(self.device)
        self.worklist = torch.from_numpy(worklist.reshape(-1).copy()).to(self.device)
        scheme = cfgs[0].to_c()
        for a in range(3):
            scheme.n[a] = int(max(c.cells[a] for c in cfgs))
            scheme.dx[a] = 1.0
        self.scheme = scheme
        self.gtile = _lib.GbfTile()
        for a in range(3):
            self.gtile.t[a] = self.tile[a]
        self.gtile.threads = self.threads

    def retile(self, tile, threads=None, ctas=None):
        """Change the tile shape (rebuilds the work list; states are kept)."""
        if threads is not None:
            self.threads = threads
        if ctas is not None:
            self.ctas = ctas
        self._layout(tile)

    # ---- state ------------------------------------------------------------
    def case_view(self, i: int) -> torch.Tensor:
        c = self.configs[i]
        o = int(self.offsets[i])
        return self.cons[o:o + 5 * c.n_cells].view(c.interior_shape())

    def set_states(self, states: List[torch.Tensor], t0: float = 0.0) -> None:
        for i, s in enumerate(states):
            self.case_view(i).copy_(s.reshape(self.configs[i].interior_shape()))
        _lib.check(self.lib.gbf_batch_init(
            ctypes.byref(self.scheme), _ptr_u8(self.case_table), len(self.configs),
            ctypes.c_void_p(self.worklist.data_ptr()), self.ntiles, ctypes.byref(self.gtile),
            _ptr(self.cons), _ptr(self.dt_states), float(t0), _stream()), "batch init")

    def advance(self, steps: int) -> None:
        _lib.check(self.lib.gbf_batch_advance(
            ctypes.byref(self.scheme), _ptr_u8(self.case_table), len(self.configs),
            ctypes.c_void_p(self.worklist.data_ptr()), self.ntiles, ctypes.byref(self.gtile), int(self.ctas),
            _ptr(self.cons), _ptr(self.dt_states), _ptr(self.workspace), self.total, int(steps), _stream()),
            "batch advance")

    def capture(self, steps: int) -> torch.cuda.CUDAGraph:
        """Record `steps` batched steps in a CUDA graph (replay with .replay())."""
        self.advance(1)  # sets kernel attributes outside the capture
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream(self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                self.advance(steps)
        torch.cuda.current_stream(self.device).wait_stream(s)
        return g

    @property
    def dt(self) -> torch.Tensor:
        return self.dt_states.view(-1, 4)[:, 0]

    @property
    def t(self) -> torch.Tensor:
        return self.dt_states.view(-1, 4)[:, 1]


def _ptr_u8(t: torch.Tensor) -> ctypes.c_void_p:
    if not t.is_cuda or not t.is_contiguous():
        raise ValueError("device table must be a contiguous CUDA tensor")
    return ctypes.c_void_p(t.data_ptr())


def autotune(batch: BatchedRK3, candidates: Optional[List[Tuple[Tuple[int, int, int], int, int]]] = None,
             steps: int = 2) -> Dict:
    """Time each (tile, threads, ctas) candidate on the batch and keep the fastest.

    The batch state is saved before and restored after every trial, so tuning
    does not advance the simulation.  Returns {"best": (tile, threads, ctas),
    "results": [(candidate, ms_per_step), ...]}.
    """
    dim = batch.configs[0].dim
    if candidates is None:
        sms = torch.cuda.get_device_properties(batch.device).multi_processor_count
        if dim == 2:
            # cell tiles whose faces along either axis fill whole rounds of
            # 128 or 256 threads
            shapes = [(16, 16, 1), (16, 8, 1), (8, 16, 1), (32, 16, 1), (16, 32, 1), (32, 32, 1)]
        elif dim == 3:
            shapes = [(7, 8, 8), (8, 8, 8), (8, 8, 16), (4, 8, 16), (8, 16, 8)]
        else:
            shapes = [(256, 1, 1), (512, 1, 1), (128, 1, 1)]
        candidates = [(sh, thr, k * sms) for sh in shapes for thr in (256, 128) for k in (1, 2, 3)]
    saved_cons = batch.cons.clone()
    saved_dt = batch.dt_states.clone()
    results = []
    for tile, thr, ctas in candidates:
        ncell = tile[0] * tile[1] * tile[2]
        if ncell > 4 * thr:
            continue
        try:
            batch.retile(tile, thr, ctas)
            batch.advance(1)  # warm-up (kernel attributes)
        except _lib.GbfError:
            continue
        torch.cuda.synchronize(batch.device)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        batch.advance(steps)
        b.record()
        b.synchronize()
        results.append(((tile, thr, ctas), a.elapsed_time(b) / steps))
        batch.cons.copy_(saved_cons)
        batch.dt_states.copy_(saved_dt)
    if not results:
        raise RuntimeError("no launch candidate ran")
    best = min(results, key=lambda r: r[1])[0]
    batch.retile(*best)
    batch.cons.copy_(saved_cons)
    batch.dt_states.copy_(saved_dt)
    return {"best": best, "results": results}
