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
  trajectories of large grids fit in memory; the forward run for the loss
  places the first checkpoints, and segments of up to ``leaf`` steps are
  replayed once keeping their stage states (3 states per step of leaf memory)
  instead of recomputing stages inside every step VJP.

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
        if nb == 0:
            raise NotImplementedError("no adjoint for this setup")
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
        """Reverse the stored steps, releasing each step's states once used
        (the list is emptied)."""
        while store:
            Un, U1, U2 = store.pop()
            lam = self.step_vjp_stages(Un, U1, U2, lam)
            del Un, U1, U2
        return lam

    def rhs_vjp(self, U: torch.Tensor, w: torch.Tensor) -> torch.Tensor:
        out = torch.empty_like(w)
        tile = ctypes.byref(self.tile) if self.tile is not None else None
        _lib.check(self.lib.gbf_rhs_vjp(ctypes.byref(self.case), _ptr(U), _ptr(w), _ptr(out), _ptr(self.ws),
                                        tile, _stream()), "rhs vjp")
        return out

    # ---- uniform checkpoints ----------------------------------------------
    def forward_uniform(self, U0: torch.Tensor, nsteps: int, every: int,
                        keep_last: bool = False) -> Tuple[torch.Tensor, "UniformCheckpoints"]:
        """U_N and the states at steps 0, every, 2 every, ...  With keep_last the
        last segment runs keeping its stage states (ckpt.last = (start, store)),
        which the reverse sweep then uses instead of replaying that segment."""
        ckpt = UniformCheckpoints({0: U0.clone()})
        U = U0
        k = 0
        while k < nsteps:
            m = min(every, nsteps - k)
            if keep_last and k + m >= nsteps:
                U, store = self.forward_stored(U, m)
                ckpt.last = (k, store)
            else:
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
        last = getattr(ckpt, "last", None)
        for s in reversed(starts):
            m = min(every, nsteps - s)
            if last is not None and last[0] == s:
                # the forward run kept this segment's stage states
                lam = self.backward_stored(last[1], lam)
                ckpt.last = last = None
                continue
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
    @functools.lru_cache(maxsize=8)
    def _leaf_plan(n: int, slots: int, leaf: int):
        """Revolve with stored-stage leaves.  Costs in thirds of a step.  To
        reverse k steps from a stored state: one step costs 2 (its two stage
        states are recomputed inside the step VJP), a segment of 2..leaf steps
        costs 3k (replayed once keeping every stage state, held in 3k states of
        leaf memory); longer ones split at m: advance m (3m), reverse the tail
        with one slot fewer, then the head.  Without slots the tail segment is
        reached by re-advancing from the start.  Returns (cost, choice) tables
        indexed [s][k]; choice = (kind, m)."""
        INF = float("inf")
        cost = [[INF] * (n + 1) for _ in range(slots + 1)]
        choice = [[None] * (n + 1) for _ in range(slots + 1)]

        def leaf_cost(k):
            return 2 if k == 1 else 3 * k

        for sl in range(slots + 1):
            cost[sl][0] = 0
            for k in range(1, n + 1):
                if k <= max(leaf, 1):
                    best, ch = leaf_cost(k), ("step" if k == 1 else "leaf", k)
                else:
                    best, ch = INF, None
                if sl == 0:
                    for t in range(1, min(k - 1, leaf) + 1):  # last segment of t steps
                        c = 3 * (k - t) + leaf_cost(t) + cost[0][k - t]
                        if c < best:
                            best, ch = c, ("tail", t)
                else:
                    for m in range(1, k):
                        c = 3 * m + cost[sl - 1][k - m] + cost[sl][m]
                        if c < best:
                            best, ch = c, ("split", m)
                cost[sl][k] = best
                choice[sl][k] = ch
        return cost, choice

    def _reverse(self, U: torch.Tensor, n: int, slots: int, lam: torch.Tensor, choice) -> torch.Tensor:
        kind, m = choice[slots][n]
        if kind == "step":
            return self.step_vjp(U, lam)
        if kind == "leaf":
            _, store = self.forward_stored(U, n)
            lam = self.backward_stored(store, lam)
            del store
            return lam
        if kind == "tail":
            Ut = self.advance(U, n - m)
            lam = self._reverse(Ut, m, 0, lam, choice)
            del Ut
            return self._reverse(U, n - m, 0, lam, choice)
        Um = self.advance(U, m)
        lam = self._reverse(Um, n - m, slots - 1, lam, choice)
        del Um
        return self._reverse(U, m, slots, lam, choice)

    def forward_binomial(self, U0: torch.Tensor, nsteps: int, slots: int, leaf: int = 1):
        """The forward run for the loss, placing the checkpoints the reverse
        sweep reaches first (the right spine of the plan) and keeping the stage
        states of the last segment.  Returns (U_N, last-segment store, spine),
        spine = [(start state, steps, slots)] still to be reversed."""
        choice = self._leaf_plan(nsteps, slots, leaf)[1]
        U, n, sl = U0, nsteps, slots
        spine = []
        while True:
            kind, m = choice[sl][n]
            if kind == "split":
                Um = self.advance(U, m)
                spine.append((U, m, sl))
                U, n, sl = Um, n - m, sl - 1
            elif kind == "tail":
                Ut = self.advance(U, n - m)
                spine.append((U, n - m, 0))
                U, n = Ut, m
            else:
                UN, store = self.forward_stored(U, n)
                return UN, store, (spine, choice)

    def backward_binomial(self, store, spine, lam: torch.Tensor) -> torch.Tensor:
        parts, choice = spine
        lam = self.backward_stored(store, lam)
        del store
        while parts:
            U, m, sl = parts.pop()
            lam = self._reverse(U, m, sl, lam, choice)
        return lam

    def binomial_cost(self, nsteps: int, slots: int, leaf: int = 1) -> float:
        """Forward-step equivalents of the binomial schedule beyond the loss's
        forward run (stage recomputation inside step VJPs included)."""
        cost, choice = self._leaf_plan(nsteps, slots, leaf)
        total, n, sl = 0, nsteps, slots
        while True:  # the spine's left parts; the spine itself is the loss forward
            kind, m = choice[sl][n]
            if kind == "split":
                total += cost[sl][m]
                n, sl = n - m, sl - 1
            elif kind == "tail":
                total += cost[0][n - m]
                n = m
            else:
                return total / 3.0

    # ---- gradient -----------------------------------------------------------
    def gradient(self, U0: torch.Tensor, nsteps: int, loss_grad: Callable[[torch.Tensor], torch.Tensor],
                 schedule: str = "uniform", every: int = 50, slots: int = 8, keep_stages: bool = True,
                 leaf: int = 1):
        """(U_N, dL/dU_0) for a loss whose gradient w.r.t. U_N is loss_grad(U_N).

        The forward run (checkpoints placed) and the reverse sweep (replays and
        step VJPs) are timed apart with CUDA events on the current stream:
        self.last_split = (forward seconds, reverse seconds) after the call."""
        if schedule not in ("uniform", "binomial", "stored"):
            raise ValueError(schedule)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)] if U0.is_cuda else None
        if ev:
            ev[0].record()
        if schedule == "uniform":
            UN, ckpt = self.forward_uniform(U0, nsteps, every, keep_last=True)
        elif schedule == "binomial":
            UN, store, spine = self.forward_binomial(U0, nsteps, slots, leaf)
        else:
            UN, store = self.forward_stored(U0, nsteps)
        if ev:
            ev[1].record()
        lam = loss_grad(UN)
        if schedule == "uniform":
            dU0 = self.backward_uniform(ckpt, nsteps, every, lam, keep_stages)
        elif schedule == "binomial":
            dU0 = self.backward_binomial(store, spine, lam)
        else:
            dU0 = self.backward_stored(store, lam)
        if ev:
            ev[2].record()
            ev[2].synchronize()
            self.last_split = (ev[0].elapsed_time(ev[1]) / 1e3, ev[1].elapsed_time(ev[2]) / 1e3)
        return UN, dU0


class UniformCheckpoints(dict):
    """Uniform checkpoints {step: state}; `last` optionally holds the last
    segment's (start step, stored stage states) from the forward run."""

    last = None


class RK3Trajectory(torch.autograd.Function):
    """U_N = RK3^nsteps(U_0) with the hand-written adjoint as backward."""

    @staticmethod
    def forward(ctx, U0: torch.Tensor, adj: AdjointRK3, nsteps: int, schedule: str = "uniform",
                every: int = 50, slots: int = 8, leaf: int = 1):
        ctx.adj, ctx.nsteps, ctx.schedule, ctx.every, ctx.slots, ctx.leaf = adj, nsteps, schedule, every, slots, leaf
        U0c = U0.detach().contiguous()
        if schedule == "uniform":
            UN, ckpt = adj.forward_uniform(U0c, nsteps, every, keep_last=True)
            ctx.ckpt = ckpt
        else:
            UN, ctx.store, ctx.spine = adj.forward_binomial(U0c, nsteps, slots, leaf)
        return UN

    @staticmethod
    def backward(ctx, g):
        adj = ctx.adj
        lam = g.contiguous()
        if ctx.schedule == "uniform":
            dU0 = adj.backward_uniform(ctx.ckpt, ctx.nsteps, ctx.every, lam)
        else:
            dU0 = adj.backward_binomial(ctx.store, ctx.spine, lam)
            ctx.store = ctx.spine = None
        return dU0, None, None, None, None, None, None
