"""Host-side mirror of the JAX-Fluids interfaces on the GB300 path.

The classes keep the reference's method names, argument meaning and return
containers so that a maintainer can swap them in for the single-phase
right-hand side:

* ``SpaceSolver.compute_rhs``            <- solvers/space_solver.py:151-453
* ``HaloManager.perform_halo_update_material`` <- halos/halo_manager.py:146-234
* ``EquationManager.get_{primitives,conservatives}_from_*`` <- equation_manager.py:44-171
* ``TimeIntegrator.perform_stage_integration`` <- time_integration/time_integrator.py:108-226
* ``compute_time_step_size``             <- time_integration/time_step_size.py:15-157

Buffers are torch CUDA float64 tensors in the reference layout.  All
arithmetic runs in libgbfluids.so through its C ABI on the tensors' device
memory and the current torch stream; a missing library raises.
"""
from __future__ import annotations

import ctypes
from typing import NamedTuple, Optional

import torch

from . import _lib
from .config import CaseConfig


# --- containers of the reference (data_types/buffers.py:103-120, information.py:52) ---
class EulerIntegrationBuffers(NamedTuple):
    conservatives: torch.Tensor
    levelset: Optional[torch.Tensor] = None
    solid_velocity: Optional[torch.Tensor] = None
    solid_energy: Optional[torch.Tensor] = None


class IntegrationBuffers(NamedTuple):
    euler_buffers: EulerIntegrationBuffers


class PositivityCounter(NamedTuple):
    interpolation_limiter: Optional[int] = None
    thinc_limiter: Optional[int] = None
    flux_limiter: Optional[int] = None
    acdi_limiter: Optional[int] = None
    volume_fraction_limiter: Optional[int] = None


class DiscretizationCounter(NamedTuple):
    acdi: Optional[int] = None
    thinc: Optional[int] = None


def _stream() -> ctypes.c_void_p:
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t: torch.Tensor, shape=None, name="buffer") -> ctypes.c_void_p:
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError(f"{name} must be a CUDA tensor")
    if t.dtype != torch.float64:
        raise TypeError(f"{name} must be float64")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")
    if shape is not None and tuple(t.shape) != tuple(shape):
        raise ValueError(f"{name} has shape {tuple(t.shape)}, expected {tuple(shape)}")
    return ctypes.c_void_p(t.data_ptr())


class _Base:
    def __init__(self, config: CaseConfig):
        self.config = config
        self.lib = _lib.load()
        self.case = config.to_c()
        st = self.lib.gbf_case_check(ctypes.byref(self.case))
        if st == -2:
            raise NotImplementedError(f"setup not supported by the CUDA path: {_lib.STATUS[st]}")
        _lib.check(st, "case check")


class EquationManager(_Base):
    def get_primitives_from_conservatives(self, conservatives: torch.Tensor) -> torch.Tensor:
        out = torch.empty_like(conservatives)
        n = conservatives.numel() // 5
        _lib.check(self.lib.gbf_prims_from_cons(ctypes.byref(self.case), _ptr(conservatives), _ptr(out),
                                                n, _stream()), "prims_from_cons")
        return out

    def get_conservatives_from_primitives(self, primitives: torch.Tensor) -> torch.Tensor:
        out = torch.empty_like(primitives)
        n = primitives.numel() // 5
        _lib.check(self.lib.gbf_cons_from_prims(ctypes.byref(self.case), _ptr(primitives), _ptr(out),
                                                n, _stream()), "cons_from_prims")
        return out


class HaloManager(_Base):
    def perform_halo_update_material(self, primitives: torch.Tensor, physical_simulation_time: float = 0.0,
                                     fill_edge_halos: bool = False, fill_vertex_halos: bool = False,
                                     conservatives: Optional[torch.Tensor] = None, **kwargs):
        """Fills halos in place of copies of the inputs; returns (prims, cons) or prims.
        Boundary values that vary in time are taken at physical_simulation_time."""
        shape = self.config.halo_shape()
        if self.config.time_varying_faces:
            self.config.refresh_bc_fields(float(physical_simulation_time))
        prims = primitives.clone()
        cons = conservatives.clone() if conservatives is not None else None
        _lib.check(self.lib.gbf_halo_fill(ctypes.byref(self.case), _ptr(prims, shape, "primitives"),
                                          _ptr(cons, shape, "conservatives") if cons is not None else None,
                                          _stream()), "halo fill")
        return (prims, cons) if cons is not None else prims


class SpaceSolver(_Base):
    """Drop-in for jaxfluids.solvers.space_solver.SpaceSolver (single phase).

    Constructed either from a CaseConfig, or with the reference's own
    constructor arguments (solvers/space_solver.py:45-57: domain_information,
    material_manager, equation_manager, halo_manager, numerical_setup, gravity,
    geometric_source, handlers), from which the setup is read
    (jax_binding.case_config_from_reference)."""

    def __init__(self, config, material_manager=None, equation_manager=None, halo_manager=None,
                 numerical_setup=None, gravity=None, geometric_source=None, levelset_handler=None,
                 diffuse_interface_handler=None, positivity_handler=None, *, tile: Optional[_lib.GbfTile] = None):
        if not isinstance(config, CaseConfig):
            from .jax_binding import case_config_from_reference
            if material_manager is None or halo_manager is None or numerical_setup is None:
                raise TypeError("SpaceSolver takes a CaseConfig or the reference's constructor arguments")
            if levelset_handler is not None or diffuse_interface_handler is not None:
                raise NotImplementedError("two-phase handlers are not on the GB300 path")
            config = case_config_from_reference(config, material_manager, numerical_setup, halo_manager, gravity)
        elif isinstance(material_manager, _lib.GbfTile):  # SpaceSolver(config, tile)
            tile = material_manager
        super().__init__(config)
        self.tile = tile
        # bytes of Lax-Friedrichs' axis speeds (0 for the other schemes)
        self.rhs_ws_bytes = int(self.lib.gbf_rhs_workspace_bytes(ctypes.byref(self.case)))

    def compute_rhs(self, conservatives: torch.Tensor, primitives: torch.Tensor,
                    temperature: Optional[torch.Tensor], physical_simulation_time: float,
                    physical_timestep_size: float, levelset=None, volume_fraction=None, apertures=None,
                    interface_velocity=None, interface_pressure=None, solid_velocity=None,
                    solid_temperature=None, interface_cells=None, forcing_buffers=None, ml_setup=None,
                    is_feed_forward: bool = False):
        if any(x is not None for x in (levelset, volume_fraction, apertures, interface_velocity,
                                       interface_pressure, solid_velocity, solid_temperature,
                                       interface_cells, forcing_buffers)):
            raise NotImplementedError("two-phase, solid and forcing inputs are not on this path")
        shape = self.config.halo_shape()
        rhs = torch.empty(self.config.interior_shape(), dtype=torch.float64, device=primitives.device)
        tile = ctypes.byref(self.tile) if self.tile is not None else None
        # Lax-Friedrichs' axis speeds: a workspace per call from torch's
        # stream-ordered allocator, so calls on concurrent streams share none
        nws = self.rhs_ws_bytes
        ws = torch.empty(max(1, nws // 8), dtype=torch.float64, device=primitives.device) if nws else None
        _lib.check(self.lib.gbf_rhs_ws(ctypes.byref(self.case), _ptr(primitives, shape, "primitives"),
                                       _ptr(conservatives, shape, "conservatives") if conservatives is not None
                                       else None, _ptr(rhs), tile, _ptr(ws) if ws is not None else None, _stream()),
                   "compute_rhs")
        if self.config.gravity is not None:
            # volume forces from the conservatives (space_solver.py:377-384)
            _lib.check(self.lib.gbf_volume_force(ctypes.byref(self.case), _ptr(conservatives, shape, "conservatives"),
                                                 _ptr(rhs), _stream()), "volume forces")
        return (IntegrationBuffers(EulerIntegrationBuffers(rhs)), PositivityCounter(),
                DiscretizationCounter())


class TimeIntegrator(_Base):
    """RK3 stage integration on halo buffers (RK3.py, time_integrator.py)."""
    no_stages = 3
    timestep_increment_factor = (1.0, 0.5, 1.0)

    def perform_stage_integration(self, conservatives: torch.Tensor, rhs: torch.Tensor,
                                  initial_conservatives: Optional[torch.Tensor], dt: torch.Tensor,
                                  stage: int) -> torch.Tensor:
        out = conservatives.clone()
        _lib.check(self.lib.gbf_stage_integrate(
            ctypes.byref(self.case), _ptr(out, self.config.halo_shape()),
            _ptr(initial_conservatives) if initial_conservatives is not None else None,
            _ptr(rhs, self.config.interior_shape(), "rhs"), _ptr(dt), stage, _stream()), "stage")
        return out


class TimeStepSize(_Base):
    def __init__(self, config: CaseConfig):
        super().__init__(config)
        self._ws = None

    def __call__(self, primitives: torch.Tensor) -> torch.Tensor:
        """compute_time_step_size on a halo primitive buffer -> device scalar."""
        if self._ws is None or self._ws.device != primitives.device:
            self._ws = torch.empty(int(self.lib.gbf_dt_workspace_bytes()) // 8, dtype=torch.float64,
                                   device=primitives.device)
        dt = torch.empty((), dtype=torch.float64, device=primitives.device)
        _lib.check(self.lib.gbf_dt(ctypes.byref(self.case), _ptr(primitives, self.config.halo_shape()),
                                   _ptr(dt), _ptr(self._ws), _stream()), "dt")
        return dt
