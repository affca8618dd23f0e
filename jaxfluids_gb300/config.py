"""Case / numerical setup of the GB300 path, read from JAX-Fluids setup dicts.

``CaseConfig.from_setups(case_setup, numerical_setup)`` accepts the same JSON
dictionaries ``jaxfluids.InputManager`` reads (input/input_manager.py:32-43)
and keeps the keys the single-phase right-hand side uses:

* case_setup: ``domain.{x,y,z}.{cells,range}``, ``boundary_conditions.<face>.type``,
  ``material_properties.equation_of_state.{model,specific_heat_ratio,specific_gas_constant}``,
  ``material_properties.transport.dynamic_viscosity`` / ``thermal_conductivity``;
* numerical_setup: ``conservatives.halo_cells``,
  ``conservatives.time_integration.{integrator,CFL,fixed_timestep}``,
  ``conservatives.convective_fluxes.{convective_solver,godunov.{riemann_solver,
  signal_speed,reconstruction_stencil,reconstruction_variable,frozen_state}}``
  (input/numerical_setup/read_conservatives.py:55-203),
  ``conservatives.dissipative_fluxes.*`` (:374-445) and ``active_physics.*``
  (data_types/numerical_setup/active_physics.py:3-13).

Setups the CUDA path does not implement are rejected here, at construction,
the way the reference rejects invalid setups with assertions; nothing is
rejected at run time.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Dict, Optional, Tuple

from . import _lib

FACES = ("east", "west", "north", "south", "top", "bottom")
FACE_AXIS = {"east": 0, "west": 0, "north": 1, "south": 1, "top": 2, "bottom": 2}

# precision.py:50 and :53
EPS = 2.220446049250313e-16
STENCIL_EPS = 1e-30


class SetupError(AssertionError):
    """An invalid or unsupported setup (raised at construction)."""


def _get(d: dict, path: str, default=None):
    cur = d
    for k in path.split("."):
        if not isinstance(cur, dict) or k not in cur:
            return default
        cur = cur[k]
    return cur


def _constant_callables(spec: dict, names: Tuple[str, ...], face: str) -> Tuple[float, ...]:
    """Values of the reference's boundary callables (case_setup
    boundary_conditions.<face>.wall_velocity_callable / primitives_callable)
    when they are constants: numbers, or strings holding a number.  Functions
    of the boundary coordinates or time are rejected."""
    out = []
    for k in names:
        v = spec.get(k, 0.0) if k == "w" else spec.get(k)
        if v is None:
            raise SetupError(f"boundary at '{face}': '{k}' missing")
        try:
            out.append(float(v))
        except (TypeError, ValueError):
            raise NotImplementedError(f"boundary at '{face}': only constant '{k}' values are supported, got {v!r}")
    return tuple(out)


@dataclass
class CaseConfig:
    cells: Tuple[int, int, int]
    ranges: Tuple[Tuple[float, float], ...] = ((0.0, 1.0), (0.0, 1.0), (0.0, 1.0))
    nh: int = 3
    gamma: float = 1.4
    R: float = 1.0
    bc: Dict[str, str] = field(default_factory=dict)
    recon: str = "WENO5-Z"
    recon_var: str = "PRIMITIVE"
    frozen_state: str = "ARITHMETIC"
    riemann: str = "HLLC"
    signal_speed: str = "EINFELDT"
    cfl: float = 0.5
    fixed_dt: Optional[float] = None
    viscous: bool = False
    heat: bool = False
    mu: float = 0.0
    bulk_viscosity: float = 0.0
    kappa: float = 0.0
    prandtl: Optional[float] = None
    viscous_heat_production: bool = True
    eps: float = EPS
    stencil_eps: float = STENCIL_EPS
    # constant boundary values per face: WALL (u, v, w), DIRICHLET and
    # NEUMANN (rho, u, v, w, p) (wall_velocity_callable / primitives_callable)
    bc_values: Dict[str, Tuple[float, ...]] = field(default_factory=dict)
    # dissipative_fluxes.{reconstruction_stencil, derivative_stencil_center,
    # derivative_stencil_face}: CENTRAL4 or CENTRAL2
    diss_recon: str = "CENTRAL4"
    diss_deriv_center: str = "CENTRAL4"
    diss_deriv_face: str = "CENTRAL4"
    # active_physics.is_convective_flux: False leaves only the dissipative fluxes
    convective: bool = True

    def __post_init__(self):
        self.cells = tuple(int(n) for n in self.cells)
        self.ranges = tuple(tuple(float(v) for v in r) for r in self.ranges)
        if any(n < 1 for n in self.cells):
            raise SetupError("cells must be >= 1 on every axis")
        if not self.active:
            raise SetupError("at least one axis needs more than one cell")
        for f in FACES:
            if FACE_AXIS[f] in self.active:
                if f not in self.bc:
                    raise SetupError(f"boundary condition for face '{f}' missing")
                if self.bc[f] not in _lib.BC:
                    raise NotImplementedError(f"boundary type {self.bc[f]} at {f}")
        for f in FACES:
            if FACE_AXIS[f] not in self.active:
                continue
            need_values = {"WALL": 3, "DIRICHLET": 5, "NEUMANN": 5}.get(self.bc[f])
            if need_values is not None:
                vals = self.bc_values.get(f)
                if vals is None or len(vals) != need_values:
                    raise SetupError(f"{self.bc[f]} boundary at '{f}' needs {need_values} values")
                self.bc_values[f] = tuple(float(v) for v in vals)
        for ax, (lo, hi) in ((0, ("west", "east")), (1, ("south", "north")), (2, ("bottom", "top"))):
            if ax in self.active and (self.bc[lo] == "PERIODIC") != (self.bc[hi] == "PERIODIC"):
                raise SetupError(f"PERIODIC must be set on both faces of axis {ax}")
        for key, table in (("recon", _lib.RECON), ("recon_var", _lib.RECVAR),
                           ("frozen_state", _lib.FROZEN), ("riemann", _lib.RIEMANN),
                           ("signal_speed", _lib.SIGNAL)):
            if getattr(self, key) not in table:
                raise NotImplementedError(f"{key} = {getattr(self, key)}")
        need = 3 if self.recon in ("WENO5-Z", "WENO5-JS") else 2
        if self.nh < need:
            raise SetupError(f"halo_cells = {self.nh} < {need} required by {self.recon}")
        for i in self.active:
            if self.cells[i] < self.nh:
                raise SetupError("each active axis needs at least halo_cells cells")
        if self.fixed_dt is None and not self.cfl > 0:
            raise SetupError("CFL must be positive")
        if self.heat and self.prandtl is not None and not self.kappa:
            # PRANDTL model (materials/single_materials/material.py:115-116)
            self.kappa = self.gamma / (self.gamma - 1.0) * self.R * self.mu / self.prandtl
        if not self.convective and not (self.viscous or self.heat):
            raise SetupError("no convective, viscous or heat flux is active")
        if self.viscous or self.heat:
            for key in ("diss_recon", "diss_deriv_center", "diss_deriv_face"):
                if getattr(self, key) not in _lib.CENTRAL:
                    raise NotImplementedError(f"dissipative stencil {getattr(self, key)}")
            # centre derivatives on a ring of the reconstruction's halo width
            # (source_term_solver.py:63-71): nh >= both halo widths together
            halos = {"CENTRAL4": 2, "CENTRAL2": 1}
            need_d = halos[self.diss_recon] + halos[self.diss_deriv_center] if self.viscous else 2
            if self.nh < need_d:
                raise SetupError(f"the dissipative stencils need halo_cells >= {need_d}")

    # domain/domain_information.py:80-206 and mesh_creation/homogenous.py:13
    @property
    def active(self):
        return [i for i in range(3) if self.cells[i] > 1]

    @property
    def dim(self) -> int:
        return len(self.active)

    def cell_size(self, axis: int) -> float:
        lo, hi = self.ranges[axis]
        return (hi - lo) / self.cells[axis]

    @property
    def n_cells(self) -> int:
        return self.cells[0] * self.cells[1] * self.cells[2]

    def halo_shape(self):
        return (5,) + tuple(n + 2 * self.nh if n > 1 else 1 for n in self.cells)

    def interior_shape(self):
        return (5,) + tuple(self.cells)

    def interior_slices(self):
        return (slice(None),) + tuple(slice(self.nh, -self.nh) if n > 1 else slice(None)
                                      for n in self.cells)

    def to_c(self) -> _lib.GbfCase:
        c = _lib.GbfCase()
        for i in range(3):
            c.n[i] = self.cells[i]
            c.dx[i] = self.cell_size(i) if self.cells[i] > 1 else 1.0
        c.nh = self.nh
        c.recon = _lib.RECON[self.recon]
        c.recon_var = _lib.RECVAR[self.recon_var]
        c.frozen_state = _lib.FROZEN[self.frozen_state]
        c.riemann = _lib.RIEMANN[self.riemann]
        c.signal_speed = _lib.SIGNAL[self.signal_speed]
        for k, f in enumerate(_lib.FACE_ORDER):
            c.bc[k] = _lib.BC[self.bc.get(f, "PERIODIC")]
            vals = self.bc_values.get(f)
            if vals is not None:
                row = [0.0, *vals, 0.0] if len(vals) == 3 else list(vals)
                for v in range(5):
                    c.bc_value[k][v] = float(row[v])
        flags = 0
        if self.viscous:
            flags |= _lib.FLAG_VISCOUS
        if self.heat:
            flags |= _lib.FLAG_HEAT
        if self.viscous_heat_production:
            flags |= _lib.FLAG_VISCOUS_HEAT_PRODUCTION
        if not self.convective:
            flags |= _lib.FLAG_NO_CONVECTIVE
        c.flags = flags
        c.gamma = self.gamma
        c.R = self.R
        c.mu = self.mu
        c.bulk_mu = self.bulk_viscosity
        c.kappa = self.kappa
        c.cfl = self.cfl
        c.fixed_dt = float(self.fixed_dt) if self.fixed_dt else 0.0
        c.eps = self.eps
        c.stencil_eps = self.stencil_eps
        c.dissipative_stencil[0] = _lib.CENTRAL[self.diss_recon]
        c.dissipative_stencil[1] = _lib.CENTRAL[self.diss_deriv_center]
        c.dissipative_stencil[2] = _lib.CENTRAL[self.diss_deriv_face]
        return c

    @classmethod
    def from_setups(cls, case_setup: dict, numerical_setup: dict) -> "CaseConfig":
        """Build from the reference's case_setup / numerical_setup dictionaries."""
        cells = tuple(int(_get(case_setup, f"domain.{a}.cells", 1)) for a in "xyz")
        ranges = tuple(tuple(_get(case_setup, f"domain.{a}.range", [0.0, 1.0])) for a in "xyz")
        bc, bc_values = {}, {}
        for f in FACES:
            t = _get(case_setup, f"boundary_conditions.{f}")
            if isinstance(t, list):
                if len(t) != 1:
                    raise NotImplementedError("multiple boundary types on one face")
                t = t[0]
            spec = t if isinstance(t, dict) else {}
            if isinstance(t, dict):
                t = t.get("type")
            if t is not None and t != "INACTIVE":
                bc[f] = t
                if t == "WALL":
                    bc_values[f] = _constant_callables(spec.get("wall_velocity_callable", {}), ("u", "v", "w"), f)
                elif t in ("DIRICHLET", "NEUMANN"):
                    bc_values[f] = _constant_callables(spec.get("primitives_callable", {}),
                                                       ("rho", "u", "v", "w", "p"), f)
        eos = _get(case_setup, "material_properties.equation_of_state", {}) or {}
        if eos.get("model", "IdealGas") != "IdealGas":
            raise NotImplementedError(f"equation of state {eos.get('model')}")
        cons = _get(numerical_setup, "conservatives", {}) or {}
        ti = cons.get("time_integration", {})
        if ti.get("integrator", "RK3") != "RK3":
            raise NotImplementedError(f"time integrator {ti.get('integrator')}")
        conv = cons.get("convective_fluxes", {})
        if conv.get("convective_solver", "GODUNOV") != "GODUNOV":
            raise NotImplementedError(f"convective solver {conv.get('convective_solver')}")
        god = conv.get("godunov", {})
        phys = _get(numerical_setup, "active_physics", {}) or {}
        viscous = bool(phys.get("is_viscous_flux", False))
        heat = bool(phys.get("is_heat_flux", False))
        for key in ("is_volume_force", "is_geometric_source", "is_surface_tension"):
            if phys.get(key, False):
                raise NotImplementedError(key)
        transport = _get(case_setup, "material_properties.transport", {}) or {}
        mu = 0.0
        if viscous:
            dv = transport.get("dynamic_viscosity", {})
            if dv.get("model", "CUSTOM") != "CUSTOM" or callable(dv.get("value")) or isinstance(dv.get("value"), str):
                raise NotImplementedError("only a constant CUSTOM dynamic viscosity")
            mu = float(dv.get("value", 0.0))
        gamma = float(eos.get("specific_heat_ratio", 1.4))
        R = float(eos.get("specific_gas_constant", 1.0))
        kappa = 0.0
        if heat:
            tc = transport.get("thermal_conductivity", {})
            if tc.get("model") == "PRANDTL":
                # materials/single_materials/material.py:70-74, :115-116: kappa = cp mu / Pr
                cp = gamma / (gamma - 1.0) * R
                kappa = cp * mu / float(tc["prandtl_number"])
                if not viscous:
                    dv = transport.get("dynamic_viscosity", {})
                    kappa = cp * float(dv.get("value", 0.0)) / float(tc["prandtl_number"])
            elif tc.get("model", "CUSTOM") == "CUSTOM":
                kappa = float(tc.get("value", 0.0))
            else:
                raise NotImplementedError("thermal conductivity model")
        diss = cons.get("dissipative_fluxes", {}) or {}
        if diss.get("is_laplacian", False):
            raise NotImplementedError("dissipative_fluxes.is_laplacian")
        fixed = ti.get("fixed_timestep")
        prec = _get(numerical_setup, "precision", {}) or {}
        if prec.get("is_double_precision_compute", True) is False:
            raise NotImplementedError("single-precision compute")
        return cls(
            cells=cells, ranges=ranges, nh=int(cons.get("halo_cells", 3)), gamma=gamma, R=R, bc=bc,
            bc_values=bc_values,
            recon=god.get("reconstruction_stencil", "WENO5-Z"),
            recon_var=god.get("reconstruction_variable", "PRIMITIVE"),
            frozen_state=god.get("frozen_state", "ARITHMETIC"),
            riemann=god.get("riemann_solver", "HLLC"),
            signal_speed=god.get("signal_speed", "EINFELDT"),
            cfl=float(ti.get("CFL", 0.5)), fixed_dt=float(fixed) if fixed else None,
            viscous=viscous, heat=heat, mu=mu, kappa=kappa,
            bulk_viscosity=float(transport.get("bulk_viscosity", 0.0) or 0.0),
            viscous_heat_production=bool(phys.get("is_viscous_heat_production", True)),
            diss_recon=diss.get("reconstruction_stencil", "CENTRAL4"),
            diss_deriv_center=diss.get("derivative_stencil_center", "CENTRAL4"),
            diss_deriv_face=diss.get("derivative_stencil_face", "CENTRAL4"),
            convective=bool(phys.get("is_convective_flux", True)),
            eps=float(prec.get("epsilon", EPS)) if isinstance(prec.get("epsilon"), float) else EPS,
            stencil_eps=float(prec.get("spatial_stencil_epsilon", STENCIL_EPS))
            if isinstance(prec.get("spatial_stencil_epsilon"), float) else STENCIL_EPS,
        )
