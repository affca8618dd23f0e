"""Time stepping on the GB300 path.

``SimulationManager`` mirrors the reference's stage loop
(simulation_manager.py:670-1077) on halo buffers with the drop-in kernels:
compute_rhs -> stage integration -> primitives from conservatives -> halo
update, three times per TVD-RK3 step, and the CFL time step afterwards.

``FusedRK3`` is the hot path: it keeps only the interior conservatives
([5, Nx, Ny, Nz]) and advances them with one face-kernel launch and one cell
epilogue per RK stage (boundary conditions by index remapping, no halo
buffers) plus one tiny time-step kernel per step; dt and t stay on the device, so a run of steps
needs no host synchronisation and can be captured in a CUDA graph.
"""
from __future__ import annotations

import ctypes
import math
from typing import Optional, Tuple

import torch

from . import _lib
from .config import EPS, CaseConfig
from .solver import (EquationManager, HaloManager, SpaceSolver, TimeIntegrator, TimeStepSize,
                     _ptr, _stream)


class SimulationManager:
    def __init__(self, config: CaseConfig, tile: Optional[_lib.GbfTile] = None):
        self.config = config
        self.equation_manager = EquationManager(config)
        self.halo_manager = HaloManager(config)
        self.space_solver = SpaceSolver(config, tile)
        self.time_integrator = TimeIntegrator(config)
        self.time_step_size = TimeStepSize(config)

    def initialize(self, prims_interior: torch.Tensor) -> Tuple[torch.Tensor, torch.Tensor]:
        """MaterialFieldsInitializer.create_material_fields (material_fields_initializer.py:148-210).

        The buffer starts as eps (initialization/helper_functions.py:49-60), the
        interior takes the given primitives (5 components, or rho, the active
        velocities and p), conservatives are computed over the whole buffer and
        the halos are filled.
        """
        cfg = self.config
        dev = prims_interior.device
        P = torch.full(cfg.halo_shape(), EPS, dtype=torch.float64, device=dev)
        inner = cfg.interior_slices()
        if prims_interior.shape[0] == 5:
            P[inner] = prims_interior.reshape(cfg.interior_shape())
        else:
            ids = [0] + [1 + i for i in cfg.active] + [4]
            for k, idx in enumerate(ids):
                P[(idx,) + inner[1:]] = prims_interior[k].reshape(cfg.cells)
        U = self.equation_manager.get_conservatives_from_primitives(P)
        P, U = self.halo_manager.perform_halo_update_material(P, 0.0, False, False, U)
        return U, P

    def compute_time_step_size(self, primitives: torch.Tensor) -> torch.Tensor:
        return self.time_step_size(primitives)

    # RK3.timestep_increment_factor (RK3.py:28): the halos after stage k are
    # filled at t + dt * factor[k] (simulation_manager.py:855-857)
    STAGE_TIME_FACTORS = (1.0, 0.5, 1.0)

    def do_integration_step(self, conservatives: torch.Tensor, primitives: torch.Tensor,
                            dt: torch.Tensor, t: float = 0.0):
        """One TVD-RK3 step through the drop-in kernels (do_runge_kutta_stages)."""
        init = conservatives
        cons, prims = conservatives, primitives
        # host time of the stage halos: only boundary values varying in time read it
        dt_host = float(dt) if self.config.time_varying_faces else 0.0
        for stage in range(3):
            (rhs_buf, _, _) = self.space_solver.compute_rhs(cons, prims, None, t, dt)
            rhs = rhs_buf.euler_buffers.conservatives
            cons = self.time_integrator.perform_stage_integration(
                cons, rhs, init if stage > 0 else None, dt, stage)
            prims = self.equation_manager.get_primitives_from_conservatives(cons)
            t_stage = t + dt_host * self.STAGE_TIME_FACTORS[stage]
            prims, cons = self.halo_manager.perform_halo_update_material(prims, t_stage, False, False, cons)
        return cons, prims

    def simulate(self, conservatives, primitives, end_time: float = math.inf,
                 end_step: int = 1 << 62, t0: float = 0.0, log=None):
        """SimulationManager.advance without output: host loop, dt not clipped."""
        t, step = t0, 0
        dt = self.compute_time_step_size(primitives)
        if log is not None:
            log.append((t, float(dt), float(primitives[self.config.interior_slices()][0].min())))
        while t < end_time and step < end_step:
            conservatives, primitives = self.do_integration_step(conservatives, primitives, dt, t)
            t += float(dt)
            step += 1
            dt = self.compute_time_step_size(primitives)
            if log is not None:
                log.append((t, float(dt), float(primitives[self.config.interior_slices()][0].min())))
        return conservatives, primitives, t, step

    def write(self, path: str, primitives: torch.Tensor, t: float) -> str:
        """Output of the interior primitives of a halo buffer and the time in the
        reference's field layout (restart.py; hdf5_writer.py:79-265 writes the
        same datasets with h5py)."""
        from .restart import write_fields
        return write_fields(path, self.config, primitives[self.config.interior_slices()], t)

    def restart(self, path: str, device="cuda") -> Tuple[torch.Tensor, torch.Tensor, float]:
        """(conservatives, primitives, time) from a file of write(): the halo
        buffers rebuilt from the primitives, as the reference restarts
        (material_fields_initializer.py:212-340, create_material_fields)."""
        from .restart import read_fields
        P, t = read_fields(path, self.config)
        U, Pb = self.initialize(torch.from_numpy(P).to(device))
        return U, Pb, t


class FusedRK3:
    """Fused TVD-RK3 stepping of interior conservatives (gbf_rk3_advance)."""

    def __init__(self, config: CaseConfig, device="cuda", tile: Optional[_lib.GbfTile] = None):
        if config.time_varying_faces:
            raise NotImplementedError("boundary values varying in time need the host time of every stage: "
                                      "use SimulationManager (the fused path keeps time on the device)")
        self.config = config
        self.lib = _lib.load()
        self.case = config.to_c()
        st = self.lib.gbf_case_check(ctypes.byref(self.case))
        if st == -2:
            raise NotImplementedError("setup not supported by the fused CUDA path")
        _lib.check(st, "case check")
        self.tile = tile
        nbytes = int(self.lib.gbf_rk3_workspace_bytes(ctypes.byref(self.case)))
        self.device = torch.device(device)
        self.workspace = torch.empty(nbytes // 8, dtype=torch.float64, device=self.device)
        # {dt, t, reduction slot (max signal speed), reduction slot (min density)}
        self.dt_state = torch.zeros(4, dtype=torch.float64, device=self.device)
        self.cons = torch.empty(config.interior_shape(), dtype=torch.float64, device=self.device)
        # primitives of the state for the first stage of the next advance (None:
        # derived from the conservatives)
        self._prims0: Optional[torch.Tensor] = None

    def set_state(self, cons_interior: torch.Tensor, t0: float = 0.0,
                  prims: Optional[torch.Tensor] = None) -> None:
        """Set the interior conservatives; `prims`, the interior primitives the
        state was built from (all five components), feed the initial time step
        and the first stage, as in the reference, where the first stage reads
        the initial primitives rather than primitives recomputed from the
        conservatives."""
        self.cons.copy_(cons_interior.reshape(self.config.interior_shape()))
        self._prims0 = None
        if prims is not None:
            self._prims0 = torch.empty_like(self.cons)
            self._prims0.copy_(prims.reshape(self.config.interior_shape()))
        _lib.check(self.lib.gbf_rk3_init(ctypes.byref(self.case), _ptr(self.cons),
                                         _ptr(self._prims0) if self._prims0 is not None else None,
                                         _ptr(self.dt_state), float(t0), _stream()), "rk3 init")

    def advance(self, steps: int) -> None:
        tile = ctypes.byref(self.tile) if self.tile is not None else None
        prims = _ptr(self._prims0) if self._prims0 is not None else None
        _lib.check(self.lib.gbf_rk3_advance(ctypes.byref(self.case), _ptr(self.cons), prims, _ptr(self.dt_state),
                                            _ptr(self.workspace), int(steps), tile, _stream()), "rk3 advance")
        if steps > 0:
            self._prims0 = None  # the state has moved on

    def capture(self, steps: int) -> torch.cuda.CUDAGraph:
        """A CUDA graph of `steps` fused steps on this object's buffers: each
        replay() advances the state, time step and time by `steps` steps with
        one host call (the multi-step loop of SimulationManager.simulate,
        simulation_manager.py:296-401, without its per-step host work).  The
        state is left as it was; one warm-up step sets the kernel attributes
        outside the capture and is undone."""
        saved = (self.cons.clone(), self.dt_state.clone())
        self.advance(1)
        torch.cuda.synchronize(self.device)
        self.cons.copy_(saved[0])
        self.dt_state.copy_(saved[1])
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream(self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                self.advance(steps)
        torch.cuda.current_stream(self.device).wait_stream(s)
        return g

    def write(self, path: str) -> str:
        """Output of the current state (its primitives) and time in the
        reference's field layout (restart.py)."""
        from .restart import write_fields
        return write_fields(path, self.config, self.primitives(), float(self.t))

    @classmethod
    def from_restart(cls, config: CaseConfig, path: str, device="cuda",
                     tile: Optional[_lib.GbfTile] = None) -> "FusedRK3":
        """A FusedRK3 continuing from a file of write(): conservatives rebuilt
        from the primitives, which also feed the first stage, as a reference
        restart does (material_fields_initializer.py:212-340)."""
        from .restart import read_fields
        P, t = read_fields(path, config)
        f = cls(config, device, tile)
        Pd = torch.from_numpy(P).to(f.device)
        U = EquationManager(config).get_conservatives_from_primitives(Pd)
        f.set_state(U, t0=t, prims=Pd)
        return f

    @property
    def dt(self) -> torch.Tensor:
        return self.dt_state[0]

    @property
    def t(self) -> torch.Tensor:
        return self.dt_state[1]

    def state_health(self) -> dict:
        """Counts of cells with non-finite values, rho <= 0 and p <= 0 in the
        current state (synchronises the stream to read them)."""
        counts = torch.zeros(3, dtype=torch.int64, device=self.device)
        _lib.check(self.lib.gbf_state_check(ctypes.byref(self.case), _ptr(self.cons),
                                            ctypes.c_void_p(counts.data_ptr()), _stream()), "state check")
        nonfinite, rho, p = counts.tolist()
        return {"nonfinite": nonfinite, "rho_nonpositive": rho, "p_nonpositive": p}

    def primitives(self) -> torch.Tensor:
        out = torch.empty_like(self.cons)
        _lib.check(self.lib.gbf_prims_from_cons(ctypes.byref(self.case), _ptr(self.cons), _ptr(out),
                                                self.config.n_cells, _stream()), "prims")
        return out
