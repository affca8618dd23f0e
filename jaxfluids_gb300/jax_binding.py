"""The JAX-Fluids side of the GB300 path: the drop-in a JAX-Fluids program
installs to run its single-phase right-hand side and RK3 steps on the GB300
kernels.

JAX-Fluids runs inside ``jax.jit`` / ``lax.scan`` (simulation_manager.py:1230,
feed_forward/feed_forward.py:291-312), so its FFI for this path is an XLA
custom call.  This module provides:

* ``case_config_from_reference(domain_information, material_manager,
  numerical_setup, halo_manager, gravity)``: the ``CaseConfig`` of a running
  reference setup, read from the objects the reference's ``SpaceSolver``
  constructor receives (solvers/space_solver.py:45-57), scheme names by
  inverting the reference's own registries;
* ``pack_case`` / ``unpack_case``: the case descriptor as the int64 attribute
  ``desc`` the FFI handlers unpack (``ffi/gbf_ffi_desc.h``);
* ``register_ffi_targets``: loads ``libgbfluids_ffi.so`` (``ffi/gbf_ffi.cc``,
  built against ``jax.ffi.include_dir()`` by ``build.build_ffi``) and
  registers its handlers for the CUDA platform;
* ``space_solver_class()``: ``GB300SpaceSolver``, a subclass of the
  reference's ``SpaceSolver`` with its constructor and ``compute_rhs``
  signature (solvers/space_solver.py:151-453), whose ``compute_rhs`` is one
  ``jax.ffi.ffi_call`` of ``gbf_rhs_ffi``; ``install_space_solver(sim_manager)``
  swaps it into a constructed ``SimulationManager`` (simulation_manager.py:128-138);
* ``rk3_step_fn(config, dt)``: a fixed-dt TVD-RK3 step on interior
  conservatives as a ``jax.custom_vjp`` pair (``gbf_rk3_advance_ffi`` /
  ``gbf_rk3_step_vjp_ffi``), the body of ``_feed_forward``'s scan;
* ``fused_step_fn(config)``: the same step with the first stage's
  primitives, the time step and the time as arguments
  (``step(cons, prims, dt, t)``);
* ``simulation_manager_class()``: ``GB300SimulationManager``, a subclass of
  the reference's ``SimulationManager`` (simulation_manager.py:49-138) whose
  ``do_runge_kutta_stages`` (:670-1077) is one fused step, so the
  reference's own ``simulate`` / ``advance`` loop (:186-426), its next-dt
  computation and output, and ``_feed_forward`` (:1296-1412, differentiable
  through the hand-written VJP) run on the GB300 kernels.

Importing this module needs neither jax nor jaxfluids; each function imports
what it uses.  Descriptors of setups with boundary values that vary along a
face carry device pointers to arrays the ``CaseConfig`` owns: keep the
solver object alive while XLA may run the call, one descriptor per device.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional

import numpy as np

from . import _lib
from .config import CaseConfig, SetupError

FACES = ("east", "west", "north", "south", "top", "bottom")
FFI_LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libgbfluids_ffi.so")
FFI_TARGETS = ("gbf_rhs", "gbf_rk3_init", "gbf_rk3_advance", "gbf_rhs_vjp", "gbf_rk3_step_vjp")


# ---------------------------------------------------------------- descriptor
def pack_case(c: _lib.GbfCase) -> np.ndarray:
    """The bytes of a gbf_case as int64 words (the FFI attribute ``desc``)."""
    raw = bytes(c)
    if len(raw) % 8:
        raise ValueError("sizeof(gbf_case) is not a multiple of 8")
    return np.frombuffer(raw, dtype=np.int64).copy()


def unpack_case(words) -> _lib.GbfCase:
    """Inverse of pack_case."""
    w = np.ascontiguousarray(np.asarray(words, dtype=np.int64))
    if w.nbytes != ctypes.sizeof(_lib.GbfCase):
        raise ValueError(f"descriptor of {w.nbytes} bytes, gbf_case has {ctypes.sizeof(_lib.GbfCase)}")
    return _lib.GbfCase.from_buffer_copy(w.tobytes())


# ---------------------------------------------------------------- setups from the reference's objects
def _registry_name(obj, registry: dict, what: str) -> str:
    for name, entry in registry.items():
        if entry is obj:
            return name
    raise NotImplementedError(f"{what} {getattr(obj, '__name__', obj)} is not on the GB300 path")


def _is_constant(fn, ncoords: int) -> Optional[float]:
    """The value of a boundary callable of the reference (a wrapper of the
    boundary coordinates and time, input/setup_reader.py:123-214) when it is
    the same at every probed point and time, else None."""
    rng = np.random.default_rng(0)
    vals = []
    for t in (0.0, 0.37, 1.0):
        coords = [rng.uniform(-1.0, 2.0, 4) for _ in range(ncoords)] if ncoords else [np.zeros(4)]
        vals.append(np.asarray(fn(*coords, t), dtype=np.float64).reshape(-1))
    v = np.concatenate(vals)
    return float(v[0]) if np.all(v == v[0]) else None


def _face_spec(face_bcs, ncoords: int):
    """(type, values, bounding_domain) entries of one face from the reference's
    BoundaryConditionsFace tuple (data_types/case_setup/boundary_conditions.py)."""
    out = []
    for bc in face_bcs:
        t = bc.boundary_type
        vals = None
        if t == "WALL":
            cb = bc.wall_velocity_callable
            vals = tuple(_is_constant(getattr(cb, k), ncoords) if cb is not None else 0.0 for k in ("u", "v", "w"))
            fns = tuple(getattr(cb, k) for k in ("u", "v", "w")) if cb is not None else None
        elif t in ("DIRICHLET", "NEUMANN"):
            cb = bc.primitives_callable
            vals = tuple(_is_constant(getattr(cb, k), ncoords) for k in ("rho", "u", "v", "w", "p"))
            fns = tuple(getattr(cb, k) for k in ("rho", "u", "v", "w", "p"))
        if vals is not None and any(v is None for v in vals):
            vals = tuple(f if v is None else v for v, f in zip(vals, fns))
        out.append((t, vals, bc.bounding_domain_callable))
    return out


def case_config_from_reference(domain_information, material_manager, numerical_setup, halo_manager,
                               gravity=None) -> CaseConfig:
    """The CaseConfig of the setup a reference SpaceSolver was constructed
    with (the arguments of solvers/space_solver.py:45-57)."""
    from jaxfluids.solvers.riemann_solvers import DICT_RIEMANN_SOLVER, DICT_SIGNAL_SPEEDS
    from jaxfluids.stencils import DICT_SPATIAL_RECONSTRUCTION
    from jaxfluids.stencils.derivative import DICT_DERIVATIVE_FACE, DICT_FIRST_DERIVATIVE_CENTER
    from jaxfluids.stencils.reconstruction import CENTRAL_RECONSTRUCTION_DICT
    from jaxfluids.config import precision

    di, ns = domain_information, numerical_setup
    if getattr(di, "is_parallel", False):
        raise NotImplementedError("domain decomposition is not on the GB300 path")
    if any(np.atleast_1d(getattr(di, "is_mesh_stretching", False))):
        raise NotImplementedError("stretched meshes are not on the GB300 path")
    if material_manager.equation_type != "SINGLE-PHASE":
        raise NotImplementedError(f"equation type {material_manager.equation_type}")
    cons = ns.conservatives
    conv = cons.convective_fluxes
    god = conv.godunov
    if god is None:
        raise NotImplementedError("only the GODUNOV convective solver is on the GB300 path")
    phys = ns.active_physics
    cells = tuple(int(n) for n in di.global_number_of_cells)
    ranges = tuple((float(np.asarray(r)[0]), float(np.asarray(r)[1])) for r in di.get_global_domain_size())
    # boundary conditions, per face (halos/outer/material.py reads the same tuples)
    bcs_field = halo_manager.boundary_condition_material.boundary_conditions
    bc, bc_values = {}, {}
    axis = {"east": 0, "west": 0, "north": 1, "south": 1, "top": 2, "bottom": 2}
    for f in FACES:
        face_bcs = getattr(bcs_field, f)
        if face_bcs is None or face_bcs[0].boundary_type == "INACTIVE":
            continue
        ncoords = sum(1 for a in range(3) if a != axis[f] and cells[a] > 1)
        spec = _face_spec(face_bcs, ncoords)
        if len(spec) == 1 and spec[0][2] is None:
            bc[f] = spec[0][0]
            if spec[0][1] is not None:
                bc_values[f] = spec[0][1]
        else:
            bc[f] = [(t, v, bd) for t, v, bd in spec]
    mat = material_manager.material
    if getattr(mat, "dynamic_viscosity_model", "CUSTOM") != "CUSTOM" and phys.is_viscous_flux:
        raise NotImplementedError(f"dynamic viscosity model {mat.dynamic_viscosity_model}")
    mu = float(np.asarray(mat.get_dynamic_viscosity(1.0))) if phys.is_viscous_flux else 0.0
    kappa = 0.0
    if phys.is_heat_flux:
        if mat.thermal_conductivity_model not in ("CUSTOM", "PRANDTL"):
            raise NotImplementedError(f"thermal conductivity model {mat.thermal_conductivity_model}")
        kappa = float(np.asarray(mat.get_thermal_conductivity(1.0)))
    diss = cons.dissipative_fluxes
    ti = cons.time_integration
    pos = cons.positivity
    if pos.flux_limiter not in (None, False):
        raise NotImplementedError("positivity.flux_limiter is not on the GB300 path")
    g = None
    if phys.is_volume_force:
        g = tuple(float(x) for x in np.asarray(gravity).reshape(-1))
    return CaseConfig(
        cells=cells, ranges=ranges, nh=int(cons.halo_cells), gamma=float(mat.gamma), R=float(mat.R),
        bc=bc, bc_values=bc_values,
        recon=_registry_name(god.reconstruction_stencil, DICT_SPATIAL_RECONSTRUCTION, "reconstruction stencil"),
        recon_var=god.reconstruction_variable, frozen_state=god.frozen_state,
        riemann=_registry_name(god.riemann_solver, DICT_RIEMANN_SOLVER, "Riemann solver"),
        signal_speed=_registry_name(god.signal_speed, DICT_SIGNAL_SPEEDS, "signal speed"),
        cfl=float(ti.CFL), fixed_dt=float(ti.fixed_timestep) if ti.fixed_timestep else None,
        viscous=bool(phys.is_viscous_flux), heat=bool(phys.is_heat_flux), mu=mu, kappa=kappa,
        bulk_viscosity=float(getattr(mat, "bulk_viscosity", 0.0) or 0.0),
        viscous_heat_production=bool(phys.is_viscous_heat_production),
        diss_recon=_registry_name(diss.reconstruction_stencil, CENTRAL_RECONSTRUCTION_DICT, "stencil"),
        diss_deriv_center=_registry_name(diss.derivative_stencil_center, DICT_FIRST_DERIVATIVE_CENTER, "stencil"),
        diss_deriv_face=_registry_name(diss.derivative_stencil_face, DICT_DERIVATIVE_FACE, "stencil"),
        convective=bool(phys.is_convective_flux), gravity=g,
        interpolation_limiter=bool(pos.is_interpolation_limiter), limit_velocity=bool(pos.limit_velocity),
        eps=float(precision.get_eps()), stencil_eps=float(precision.get_spatial_stencil_eps()),
    )


# ---------------------------------------------------------------- FFI registration
_registered = False


def load_ffi_library(path: str = FFI_LIB_PATH) -> ctypes.CDLL:
    if not os.path.exists(path):
        raise _lib.GbfError(f"{path} is missing: build it with jaxfluids_gb300.build.build_ffi() "
                            "on a machine with jaxlib")
    return ctypes.CDLL(path)


def register_ffi_targets() -> None:
    """Register the handlers of libgbfluids_ffi.so with XLA (CUDA platform), once."""
    global _registered
    if _registered:
        return
    import jax
    lib = load_ffi_library()
    for name in FFI_TARGETS:
        jax.ffi.register_ffi_target(name, jax.ffi.pycapsule(getattr(lib, name + "_ffi")), platform="CUDA")
    _registered = True


# ---------------------------------------------------------------- SpaceSolver drop-in
def space_solver_class():
    """GB300SpaceSolver: the reference's SpaceSolver with compute_rhs on the
    GB300 kernels (defined against the installed jaxfluids)."""
    from jaxfluids.data_types.buffers import EulerIntegrationBuffers, IntegrationBuffers
    from jaxfluids.data_types.information import DiscretizationCounter, PositivityCounter
    from jaxfluids.solvers.space_solver import SpaceSolver

    class GB300SpaceSolver(SpaceSolver):
        def __init__(self, domain_information, material_manager, equation_manager, halo_manager,
                     numerical_setup, gravity, geometric_source, levelset_handler=None,
                     diffuse_interface_handler=None, positivity_handler=None) -> None:
            super().__init__(domain_information, material_manager, equation_manager, halo_manager,
                             numerical_setup, gravity, geometric_source, levelset_handler,
                             diffuse_interface_handler, positivity_handler)
            if geometric_source is not None and numerical_setup.active_physics.is_geometric_source:
                raise NotImplementedError("geometric source terms are not on the GB300 path")
            self.gb300_config = case_config_from_reference(domain_information, material_manager,
                                                           numerical_setup, halo_manager, gravity)
            if self.gb300_config.time_varying_faces:
                raise NotImplementedError("boundary values varying in time are not on the FFI path")
            c = self.gb300_config.to_c()
            self.gb300_desc = pack_case(c)
            self.gb300_ws_bytes = max(1, int(_lib.load().gbf_rhs_workspace_bytes(ctypes.byref(c))))

        def compute_rhs(self, conservatives, primitives, temperature, physical_simulation_time,
                        physical_timestep_size, levelset=None, volume_fraction=None, apertures=None,
                        interface_velocity=None, interface_pressure=None, solid_velocity=None,
                        solid_temperature=None, interface_cells=None, forcing_buffers=None, ml_setup=None,
                        is_feed_forward=False):
            if any(x is not None for x in (levelset, volume_fraction, apertures, interface_velocity,
                                           interface_pressure, solid_velocity, solid_temperature,
                                           interface_cells, forcing_buffers)):
                raise NotImplementedError("two-phase, solid and forcing inputs are not on the GB300 path")
            import jax
            import jax.numpy as jnp
            register_ffi_targets()
            shape = (5,) + tuple(int(n) for n in self.domain_information.device_number_of_cells)
            rhs, _ = jax.ffi.ffi_call("gbf_rhs", (jax.ShapeDtypeStruct(shape, jnp.float64),
                                                  jax.ShapeDtypeStruct((self.gb300_ws_bytes,), jnp.uint8)))(
                primitives, conservatives, desc=self.gb300_desc)
            return (IntegrationBuffers(EulerIntegrationBuffers(rhs, None, None, None)),
                    PositivityCounter(None, None, None, None, None), DiscretizationCounter(None, None))

    return GB300SpaceSolver


def install_space_solver(sim_manager):
    """Replace a constructed SimulationManager's space solver by the GB300 one
    (same constructor arguments as simulation_manager.py:128-138)."""
    cls = space_solver_class()
    old = sim_manager.space_solver
    sim_manager.space_solver = cls(
        old.domain_information, old.material_manager, old.equation_manager, old.halo_manager,
        old.numerical_setup, old.gravity, sim_manager.case_setup.forcing_setup.geometric_source,
        old.levelset_handler, old.diffuse_interface_handler, old.positivity_handler)
    return sim_manager.space_solver


# ---------------------------------------------------------------- the fixed-dt step and its VJP
def rk3_step_fn(config: CaseConfig, dt: float):
    """One fixed-dt TVD-RK3 step of interior conservatives [5, Nx, Ny, Nz] as a
    jax.custom_vjp function: forward gbf_rk3_advance (steps = 1), reverse
    gbf_rk3_step_vjp.  jax.checkpoint over a lax.scan of it reproduces
    FeedForwardSetup's schedules (feed_forward/feed_forward.py:231-524)."""
    import dataclasses

    import jax
    import jax.numpy as jnp
    register_ffi_targets()
    cfg = dataclasses.replace(config, fixed_dt=float(dt))
    c = cfg.to_c()
    lib = _lib.load()
    desc = pack_case(c)
    shape = (5,) + tuple(cfg.cells)
    ws = int(lib.gbf_rk3_workspace_bytes(ctypes.byref(c)))
    vjp_ws = int(lib.gbf_vjp_workspace_bytes(ctypes.byref(c)))
    if vjp_ws == 0:
        raise NotImplementedError("no adjoint for this setup")
    cons_t = jax.ShapeDtypeStruct(shape, jnp.float64)
    dt_state = jnp.array([dt, 0.0, 0.0, 0.0], dtype=jnp.float64)
    dt_dev = jnp.array(dt, dtype=jnp.float64)

    @jax.custom_vjp
    def step(cons):
        out, _, _ = jax.ffi.ffi_call(
            "gbf_rk3_advance", (cons_t, jax.ShapeDtypeStruct((4,), jnp.float64),
                                jax.ShapeDtypeStruct((ws,), jnp.uint8)),
            input_output_aliases={0: 0, 2: 1})(cons, cons, dt_state, desc=desc, steps=np.int64(1),
                                               with_prims=np.int64(0))
        return out

    def fwd(cons):
        return step(cons), cons

    def bwd(cons, lam):
        dU, _ = jax.ffi.ffi_call("gbf_rk3_step_vjp", (cons_t, jax.ShapeDtypeStruct((vjp_ws,), jnp.uint8)))(
            cons, dt_dev, lam, desc=desc)
        return (dU,)

    step.defvjp(fwd, bwd)
    return step


def fused_step_fn(config: CaseConfig):
    """One TVD-RK3 step of interior conservatives [5, Nx, Ny, Nz],
    step(cons, prims, dt, t): prims are the interior primitives the first
    stage reads (the reference's first stage reads the primitive buffer, not
    primitives re-derived from the conservatives), dt the step and t the time.
    A jax.custom_vjp function: forward gbf_rk3_advance (steps = 1,
    dt_state = [dt, t, 0, 0], with_prims = 1), reverse gbf_rk3_step_vjp with the
    same dt.  The reverse treats the primitives as those of the conservatives
    (the cotangent reaches the conservatives; for prims = p(cons) and
    cons = c(prims0) that is the whole derivative, p' c' = 1); dt and t get none."""
    import jax
    import jax.numpy as jnp
    register_ffi_targets()
    c = config.to_c()
    lib = _lib.load()
    desc = pack_case(c)
    shape = (5,) + tuple(config.cells)
    ws = int(lib.gbf_rk3_workspace_bytes(ctypes.byref(c)))
    vjp_ws = int(lib.gbf_vjp_workspace_bytes(ctypes.byref(c)))
    cons_t = jax.ShapeDtypeStruct(shape, jnp.float64)

    @jax.custom_vjp
    def step(cons, prims, dt, t):
        zero = jnp.zeros((), jnp.float64)
        dt_state = jnp.stack([jnp.asarray(dt, jnp.float64), jnp.asarray(t, jnp.float64), zero, zero])
        out, _, _ = jax.ffi.ffi_call(
            "gbf_rk3_advance", (cons_t, jax.ShapeDtypeStruct((4,), jnp.float64),
                                jax.ShapeDtypeStruct((ws,), jnp.uint8)),
            input_output_aliases={0: 0, 2: 1})(cons, prims, dt_state, desc=desc, steps=np.int64(1),
                                               with_prims=np.int64(1))
        return out

    def fwd(cons, prims, dt, t):
        return step(cons, prims, dt, t), (cons, prims, dt, t)

    def bwd(res, lam):
        cons, prims, dt, t = res
        if vjp_ws == 0:
            raise NotImplementedError("no adjoint for this setup")
        dU, _ = jax.ffi.ffi_call("gbf_rk3_step_vjp", (cons_t, jax.ShapeDtypeStruct((vjp_ws,), jnp.uint8)))(
            cons, jnp.asarray(dt, jnp.float64), lam, desc=desc)
        return dU, jnp.zeros_like(prims), jnp.zeros_like(dt), jnp.zeros_like(t)

    step.defvjp(fwd, bwd)
    return step


# ---------------------------------------------------------------- SimulationManager drop-in
def simulation_manager_class():
    """GB300SimulationManager: the reference's SimulationManager with each
    TVD-RK3 step one fused GB300 call (defined against the installed
    jaxfluids)."""
    from jaxfluids.data_types.buffers import MaterialFieldBuffers
    from jaxfluids.data_types.information import StepInformation
    from jaxfluids.simulation_manager import SimulationManager

    class GB300SimulationManager(SimulationManager):
        """The reference's SimulationManager whose RK stages
        (do_runge_kutta_stages, simulation_manager.py:670-1077) are one fused
        step of the GB300 kernels on the interior conservatives; the
        primitives of the new state and the halos are then formed by the
        reference's own equation and halo managers, as its last stage forms
        them (:943-974), and time and step advance as at :1046-1047.  The
        reference's loop (advance, :297-426), next-dt computation
        (_do_integration_step, :611-628), output and feed-forward
        (_feed_forward, :1296-1412) run unchanged around it; the space solver
        is GB300SpaceSolver for the calls that still ask for a right-hand side.

        step: optional replacement of the fused step, step(cons, prims, dt, t)
        -> cons on interior conservatives and primitives (default
        fused_step_fn of the case)."""

        def __init__(self, input_manager, callbacks=None, step=None):
            super().__init__(input_manager, callbacks)
            install_space_solver(self)
            cfg = self.space_solver.gb300_config
            if self.equation_information.levelset_model or self.equation_information.diffuse_interface_model:
                raise NotImplementedError("two-phase flows are not on the GB300 path")
            self.gb300_step = step if step is not None else fused_step_fn(cfg)

        def do_runge_kutta_stages(self, material_fields, time_control_variables, levelset_fields=None,
                                  solid_fields=None, forcing_buffers=None, control_flow_params=None,
                                  ml_setup=None):
            if forcing_buffers is not None:
                raise NotImplementedError("forcings are not on the GB300 path")
            nhx, nhy, nhz = self.domain_information.domain_slices_conservatives
            dt = time_control_variables.physical_timestep_size
            t = time_control_variables.physical_simulation_time
            cons = self.gb300_step(material_fields.conservatives[..., nhx, nhy, nhz],
                                   material_fields.primitives[..., nhx, nhy, nhz], dt, t)
            conservatives = material_fields.conservatives.at[..., nhx, nhy, nhz].set(cons)
            primitives = self.equation_manager.get_primitives_from_conservatives(conservatives)
            t_new = t + dt
            primitives, conservatives = self.halo_manager.perform_halo_update_material(
                primitives, t_new, self.halo_manager.fill_edge_halos_material,
                self.halo_manager.fill_vertex_halos_material, conservatives, ml_setup=ml_setup)
            temperature = material_fields.temperature
            if self.equation_information.is_compute_temperature:
                temperature = self.material_manager.get_temperature(primitives)
                temperature = self.halo_manager.perform_outer_halo_update_temperature(temperature, t_new)
            time_control_variables = time_control_variables._replace(
                simulation_step=time_control_variables.simulation_step + 1, physical_simulation_time=t_new)
            return (MaterialFieldBuffers(conservatives, primitives, temperature), time_control_variables,
                    levelset_fields, solid_fields, StepInformation((), ()))

    return GB300SimulationManager

