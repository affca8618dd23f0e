"""Reverse mode of the fused TVD-RK3 path with checkpointing.

The reference differentiates ``SimulationManager._feed_forward`` (fixed time
step, ``lax.scan`` over steps with ``jax.checkpoint`` every ``inner_steps``,
feed_forward/feed_forward.py:231-524) with ``jax.grad``.  Here the adjoint of
one step is the hand-written ``gbf_rk3_step_vjp`` kernel sequence, and the
trajectory is replayed from checkpoints kept in device memory:

* uniform: a checkpoint every ``every`` steps (the reference's
  ``FeedForwardSetup(outer_steps, inner_steps, is_checkpoint_inner_step=True)``);
  each segment is recomputed once and its states kept for the reverse sweep;
* stored: every state and both stage states of every step are kept (when
  they fit in device memory), so nothing is recomputed;
* binomial: at most ``slots`` stored states, split points chosen by dynamic
  programming to minimise recomputed steps (Griewank-style revolve), so long
  trajectories of large grids fit in memory.

``RK3Trajectory`` wraps both as a ``torch.autograd.Function``.
"""
from __future__ import annotations

import ctypes
import functools
from dataclasses import replace
from typing import Callable, Dict, List, Optional, Tuple

import torch

from . import _lib
from .config import CaseConfig
from .simulation import FusedRK3
from .solver import _ptr, _stream


class AdjointRK3:
    """Fixed-dt RK3 stepping of interior conservatives and its adjoint."""

    def __init__(self, config: CaseConfig, dt: float, device="cuda", tile: Optional[_lib.GbfTile] = None):
        self.config = replace(config, fixed_dt=float(dt))
        self.dt = float(dt)
        self.device = torch.device(device)
        self.lib = _lib.load()
        self.case = self.config.to_c()
        self.tile = tile
        self.fwd = FusedRK3(self.config, self.device, tile)
        nb = int(self.lib.gbf_vjp_workspace_bytes(ctypes.byref(self.case)))
        self.ws = torch.empty(nb // 8, dtype=torch.float64, device=self.device)
        self.dt_dev = torch.full((), self.dt, dtype=torch.float64, device=self.device)
        self.forward_steps = 0  # steps advanced, including recomputation

    # ---- primitives -------------------------------------------------------
    def advance(self, U: torch.Tensor, steps: int) -> torch.Tensor:
        """U after `steps` fixed-dt steps (U is not modified)."""
        self.fwd.cons.copy_(U)
        self.fwd.dt_state.zero_()
        self.fwd.dt_state[0] = self.dt
        if steps:
            self.fwd.advance(steps)
            self.forward_steps += steps
        return self.fwd.cons.clone()

    def step_vjp(self, U: torch.Tensor, lam: torch.Tensor) -> torch.Tensor:
        out = torch.empty_like(lam)
        tile = ctypes.byref(self.tile) if self.tile is not None else None
        _lib.check(self.lib.gbf_rk3_step_vjp(ctypes.byref(self.case), _ptr(U), _ptr(self.dt_dev), _ptr(lam),
                                             _ptr(out), _ptr(self.ws), tile, _stream()), "rk3 step vjp")
        return out

    def step_vjp_stages(self, U: torch.Tensor, U1: torch.Tensor, U2: torch.Tensor, lam: torch.Tensor) -> torch.Tensor:
        out = torch.empty_like(lam)
        tile = ctypes.byref(self.tile) if self.tile is not None else None
        _lib.check(self.lib.gbf_rk3_step_vjp_stages(ctypes.byref(self.case), _ptr(U), _ptr(U1), _ptr(U2),
                                                    _ptr(self.dt_dev), _ptr(lam), _ptr(out), _ptr(self.ws), tile,
                                                    _stream()), "rk3 step vjp")
        return out

    def forward_stored(self, U0: torch.Tensor, nsteps: int):
        """U_N and every step's (U^n, U1, U2), copied out of the fused stage buffers."""
        n = self.config.n_cells * 5
        self.fwd.cons.copy_(U0)
        self.fwd.dt_state.zero_()
        self.fwd.dt_state[0] = self.dt
        store = []
        for _ in range(nsteps):
            Un = self.fwd.cons.clone()
            self.fwd.advance(1)
            self.forward_steps += 1
            A = self.fwd.workspace[:n].view_as(Un).clone()
            B = self.fwd.workspace[n:2 * n].view_as(Un).clone()
            store.append((Un, A, B))
        return self.fwd.cons.clone(), store

    def backward_stored(self, store, lam: torch.Tensor) -> torch.Tensor:
        for Un, U1, U2 in reversed(store):
            lam = self.step_vjp_stages(Un, U1, U2, lam)
        return lam

    def rhs_vjp(self, U: torch.Tensor, w: torch.Tensor) -> torch.Tensor:
        out = torch.empty_like(w)
        tile = ctypes.byref(self.tile) if self.tile is not None else None
        _lib.check(self.lib.gbf_rhs_vjp(ctypes.byref(self.case), _ptr(U), _ptr(w), _ptr(out), _ptr(self.ws),
                                        tile, _stream()), "rhs vjp")
        return out

    # ---- uniform checkpoints ----------------------------------------------
    def forward_uniform(self, U0: torch.Tensor, nsteps: int, every: int) -> Tuple[torch.Tensor, Dict[int, torch.Tensor]]:
        ckpt = {0: U0.clone()}
        U = U0
        k = 0
        while k < nsteps:
            m = min(every, nsteps - k)
            U = self.advance(U, m)
            k += m
            if k < nsteps:
                ckpt[k] = U.clone()
        return U, ckpt

    def backward_uniform(self, ckpt: Dict[int, torch.Tensor], nsteps: int, every: int,
                         lam: torch.Tensor, keep_stages: bool = True) -> torch.Tensor:
        """Reverse sweep over the uniform checkpoints.  Each segment is replayed
        once from its checkpoint; with keep_stages the replay keeps both stage
        states of every step (3 states per step of the segment) so the step
        VJPs recompute nothing, otherwise it keeps one state per step and each
        step VJP recomputes its two stage states."""
        starts = sorted(s for s in ckpt if s < nsteps)
        for s in reversed(starts):
            m = min(every, nsteps - s)
            if keep_stages:
                _, store = self.forward_stored(ckpt[s], m)
                lam = self.backward_stored(store, lam)
                del store
                continue
            states = [ckpt[s]]
            for _ in range(m - 1):
                states.append(self.advance(states[-1], 1))
            for U in reversed(states):
                lam = self.step_vjp(U, lam)
        return lam

    # ---- binomial checkpoints ---------------------------------------------
    @staticmethod
    @functools.lru_cache(maxsize=None)
    def _plan(n: int, slots: int) -> Tuple[int, Tuple]:
        """(cost, split) minimising recomputed steps to reverse n steps from a
        stored start state with `slots` extra stored states."""
        if n <= 1:
            return 0, ()
        if slots == 0:
            return n * (n - 1) // 2, ()
        best = None
        for m in range(1, n):
            c = m + AdjointRK3._plan(n - m, slots - 1)[0] + AdjointRK3._plan(m, slots)[0]
            if best is None or c < best[0]:
                best = (c, (m,))
        return best

    def _reverse(self, U: torch.Tensor, n: int, slots: int, lam: torch.Tensor) -> torch.Tensor:
        if n == 1:
            return self.step_vjp(U, lam)
        if slots == 0:
            for j in range(n - 1, -1, -1):
                lam = self.step_vjp(self.advance(U, j), lam)
            return lam
        m = self._plan(n, slots)[1][0]
        Um = self.advance(U, m)
        lam = self._reverse(Um, n - m, slots - 1, lam)
        del Um
        return self._reverse(U, m, slots, lam)

    def backward_binomial(self, U0: torch.Tensor, nsteps: int, slots: int, lam: torch.Tensor) -> torch.Tensor:
        return self._reverse(U0, nsteps, slots, lam)

    # ---- gradient -----------------------------------------------------------
    def gradient(self, U0: torch.Tensor, nsteps: int, loss_grad: Callable[[torch.Tensor], torch.Tensor],
                 schedule: str = "uniform", every: int = 50, slots: int = 8, keep_stages: bool = True):
        """(U_N, dL/dU_0) for a loss whose gradient w.r.t. U_N is loss_grad(U_N)."""
        if schedule == "uniform":
            UN, ckpt = self.forward_uniform(U0, nsteps, every)
            lam = loss_grad(UN)
            return UN, self.backward_uniform(ckpt, nsteps, every, lam, keep_stages)
        if schedule == "binomial":
            UN = self.advance(U0, nsteps)
            lam = loss_grad(UN)
            return UN, self.backward_binomial(U0, nsteps, slots, lam)
        if schedule == "stored":
            UN, store = self.forward_stored(U0, nsteps)
            lam = loss_grad(UN)
            return UN, self.backward_stored(store, lam)
        raise ValueError(schedule)


class RK3Trajectory(torch.autograd.Function):
    """U_N = RK3^nsteps(U_0) with the hand-written adjoint as backward."""

    @staticmethod
    def forward(ctx, U0: torch.Tensor, adj: AdjointRK3, nsteps: int, schedule: str = "uniform",
                every: int = 50, slots: int = 8):
        ctx.adj, ctx.nsteps, ctx.schedule, ctx.every, ctx.slots = adj, nsteps, schedule, every, slots
        U0c = U0.detach().contiguous()
        if schedule == "uniform":
            UN, ckpt = adj.forward_uniform(U0c, nsteps, every)
            ctx.ckpt = ckpt
        else:
            UN = adj.advance(U0c, nsteps)
            ctx.U0 = U0c
        return UN

    @staticmethod
    def backward(ctx, g):
        adj = ctx.adj
        lam = g.contiguous()
        if ctx.schedule == "uniform":
            dU0 = adj.backward_uniform(ctx.ckpt, ctx.nsteps, ctx.every, lam)
        else:
            dU0 = adj.backward_binomial(ctx.U0, ctx.nsteps, ctx.slots, lam)
        return dU0, None, None, None, None, None
