"""Case / numerical setup of the GB300 path, read from JAX-Fluids setup dicts.

``CaseConfig.from_setups(case_setup, numerical_setup)`` accepts the same JSON
dictionaries ``jaxfluids.InputManager`` reads (input/input_manager.py:32-43)
and keeps the keys the single-phase right-hand side uses:

* case_setup: ``domain.{x,y,z}.{cells,range}``; ``boundary_conditions.<face>``
  as one type or a list of types with ``bounding_domain`` masks, with
  ``wall_velocity_callable`` / ``primitives_callable`` values (numbers, or
  functions or "lambda" strings of the boundary coordinates and time,
  input/case_setup/read_boundary_conditions.py:28-393);
  ``material_properties.equation_of_state.{model,specific_heat_ratio,specific_gas_constant}``,
  ``material_properties.transport.dynamic_viscosity`` / ``thermal_conductivity``;
  ``forcings.gravity``;
* numerical_setup: ``conservatives.halo_cells``,
  ``conservatives.time_integration.{integrator,CFL,fixed_timestep}``,
  ``conservatives.convective_fluxes.{convective_solver,godunov.{riemann_solver,
  signal_speed,reconstruction_stencil,reconstruction_variable,frozen_state}}``
  (input/numerical_setup/read_conservatives.py:55-203),
  ``conservatives.dissipative_fluxes.*`` (:374-445),
  ``conservatives.positivity.{is_interpolation_limiter,limit_velocity,flux_limiter}``
  (read_positivity.py), ``active_physics.*``
  (data_types/numerical_setup/active_physics.py:3-13), ``active_forcings.*``
  and ``precision.*``.

Setups the CUDA path does not implement are rejected here, at construction,
the way the reference rejects invalid setups with assertions; nothing is
rejected at run time.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Dict, Optional, Tuple

import numpy as np

from . import _lib

FACES = ("east", "west", "north", "south", "top", "bottom")
FACE_AXIS = {"east": 0, "west": 0, "north": 1, "south": 1, "top": 2, "bottom": 2}

# precision.py:50 and :53
EPS = 2.220446049250313e-16
STENCIL_EPS = 1e-30


# values per boundary type: WALL (u, v, w), DIRICHLET / NEUMANN (rho, u, v, w, p)
_VALUE_COUNT = {"WALL": 3, "DIRICHLET": 5, "NEUMANN": 5}


class SetupError(AssertionError):
    """An invalid or unsupported setup (raised at construction)."""


def _get(d: dict, path: str, default=None):
    cur = d
    for k in path.split("."):
        if not isinstance(cur, dict) or k not in cur:
            return default
        cur = cur[k]
    return cur


def _callable(v, what: str):
    """A number, or a function: a Python callable or a "lambda ..." string
    (the reference evaluates these with jax.numpy as ``jnp``,
    input/setup_reader.py:123-230; here numpy stands in)."""
    if callable(v):
        return v
    if isinstance(v, str):
        try:
            return float(v)
        except ValueError:
            pass
        if not v.strip().startswith("lambda"):
            raise SetupError(f"{what}: {v!r} is neither a number nor a lambda")
        return eval(v, {"jnp": np, "np": np, "numpy": np})  # noqa: S307 (setup files are trusted input)
    try:
        return float(v)
    except (TypeError, ValueError):
        raise SetupError(f"{what}: {v!r} is neither a number nor a function")


def _boundary_callables(spec: dict, names: Tuple[str, ...], face: str):
    """The reference's boundary callables (case_setup boundary_conditions.<face>.
    wall_velocity_callable / primitives_callable): numbers, or functions of
    the active tangential boundary coordinates and time."""
    out = []
    for k in names:
        v = spec.get(k, 0.0) if k == "w" else spec.get(k)
        if v is None:
            raise SetupError(f"boundary at '{face}': '{k}' missing")
        out.append(_callable(v, f"boundary at '{face}', '{k}'"))
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
    # boundary values per face: WALL (u, v, w), DIRICHLET and NEUMANN
    # (rho, u, v, w, p) (wall_velocity_callable / primitives_callable), each a
    # number or a function of the active tangential coordinates and time
    # (constant in time); normalised to a tuple of constants or an array
    # [k, boundary cells].  A face of several types has bc[face] =
    # [(type, values, bounding_domain), ...] (bounding_domain: function of
    # the coordinates, or a boolean per boundary cell).
    bc_values: Dict[str, Tuple[float, ...]] = field(default_factory=dict)
    # dissipative_fluxes.{reconstruction_stencil, derivative_stencil_center,
    # derivative_stencil_face}: CENTRAL4 or CENTRAL2
    diss_recon: str = "CENTRAL4"
    diss_deriv_center: str = "CENTRAL4"
    diss_deriv_face: str = "CENTRAL4"
    # active_physics.is_convective_flux: False leaves only the dissipative fluxes
    convective: bool = True
    # conservatives.positivity.{is_interpolation_limiter, limit_velocity}
    interpolation_limiter: bool = False
    limit_velocity: bool = False
    # active_physics.is_volume_force with forcings.gravity: the gravity vector
    gravity: Optional[Tuple[float, float, float]] = None
    # device copies of the boundary value fields, per device
    _fields: dict = field(default_factory=dict, init=False, repr=False, compare=False)
    # boundary callables that vary in time, per face
    _time_fns: dict = field(default_factory=dict, init=False, repr=False, compare=False)

    def __post_init__(self):
        self.cells = tuple(int(n) for n in self.cells)
        self.ranges = tuple(tuple(float(v) for v in r) for r in self.ranges)
        if any(n < 1 for n in self.cells):
            raise SetupError("cells must be >= 1 on every axis")
        if not self.active:
            raise SetupError("at least one axis needs more than one cell")
        for f in FACES:
            if FACE_AXIS[f] not in self.active:
                continue
            if f not in self.bc:
                raise SetupError(f"boundary condition for face '{f}' missing")
            spec = self.bc[f]
            if isinstance(spec, (list, tuple)):
                self.bc[f] = self._face_segments(f, spec)
                continue
            if spec not in _lib.BC:
                raise NotImplementedError(f"boundary type {spec} at {f}")
            if spec in _VALUE_COUNT:
                self.bc_values[f] = self._face_values(f, spec, self.bc_values.get(f))
        for ax, (lo, hi) in ((0, ("west", "east")), (1, ("south", "north")), (2, ("bottom", "top"))):
            if ax in self.active and (self.bc[lo] == "PERIODIC") != (self.bc[hi] == "PERIODIC"):
                raise SetupError(f"PERIODIC must be set on both faces of axis {ax}")
        for key, table in (("recon", _lib.RECON), ("recon_var", _lib.RECVAR),
                           ("frozen_state", _lib.FROZEN), ("riemann", _lib.RIEMANN),
                           ("signal_speed", _lib.SIGNAL)):
            if getattr(self, key) not in table:
                raise NotImplementedError(f"{key} = {getattr(self, key)}")
        if self.recon_var != "PRIMITIVE" and self.recon != "WENO5-Z":
            raise NotImplementedError(f"{self.recon_var} is built with WENO5-Z")
        need = 3 if self.recon in ("WENO5-Z", "WENO5-JS", "TENO5") else 2
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

    # ---- boundary values along a face --------------------------------------

    def face_axes(self, face: str) -> Tuple[int, int]:
        """The two other axes of a face, in axis order (boundary cells are
        numbered with the later one fastest)."""
        a = FACE_AXIS[face]
        return tuple(i for i in range(3) if i != a)

    def face_cells(self, face: str) -> int:
        b, c = self.face_axes(face)
        return self.cells[b] * self.cells[c]

    def cell_centers(self, axis: int) -> np.ndarray:
        # mesh_creation/homogenous.py:13-14
        lo, hi = self.ranges[axis]
        dx = (hi - lo) / self.cells[axis]
        return np.linspace(lo + dx / 2, hi - dx / 2, self.cells[axis])

    def boundary_coordinates(self, face: str):
        """Cell-centre coordinates of the boundary cells along the face's
        active axes, flattened in boundary-cell order
        (get_boundary_coordinates_at_location, boundary_condition.py:105-126)."""
        b, c = self.face_axes(face)
        xb, xc = np.meshgrid(self.cell_centers(b), self.cell_centers(c), indexing="ij")
        return [x.reshape(-1) for x, ax in ((xb, b), (xc, c)) if ax in self.active]

    def _eval_on_face(self, face: str, fn, with_time: bool, t: float = 0.0) -> np.ndarray:
        nt = self.face_cells(face)
        coords = self.boundary_coordinates(face)
        if not callable(fn):
            return np.full(nt, float(fn))
        r = fn(*coords, t) if with_time else fn(*coords)
        return np.broadcast_to(np.asarray(r, dtype=np.float64 if with_time else bool), (nt,)).copy()

    def _varies_in_time(self, face: str, fn) -> bool:
        if not callable(fn):
            return False
        v0 = self._eval_on_face(face, fn, True, 0.0)
        return any(not np.array_equal(v0, self._eval_on_face(face, fn, True, t)) for t in (0.37, 1.0))

    def _face_values(self, face: str, btype: str, vals):
        """Values of a face's type: a tuple of constants, or an array
        [k, boundary cells] where a value varies along the face (k = 3 wall
        velocities for WALL, 5 primitives or derivatives for DIRICHLET and
        NEUMANN)."""
        k = _VALUE_COUNT.get(btype)
        if k is None:
            return None
        if vals is None:
            raise SetupError(f"{btype} boundary at '{face}' needs {k} values")
        if isinstance(vals, np.ndarray) or hasattr(vals, "numpy"):
            arr = np.asarray(vals, dtype=np.float64)
            if arr.shape == (k,):
                return tuple(float(v) for v in arr)
            if arr.shape != (k, self.face_cells(face)):
                raise SetupError(f"{btype} boundary at '{face}': values of shape {arr.shape}, "
                                 f"expected ({k}, {self.face_cells(face)})")
            return arr.copy()
        vals = tuple(vals)
        if len(vals) != k:
            raise SetupError(f"{btype} boundary at '{face}' needs {k} values")
        fns = [_callable(v, f"boundary at '{face}'") for v in vals]
        if not any(callable(fn) for fn in fns):
            return tuple(float(fn) for fn in fns)
        if any(self._varies_in_time(face, fn) for fn in fns):
            # re-evaluated at every halo update's time (refresh_bc_fields)
            self._time_fns[face] = fns
        return np.stack([self._eval_on_face(face, fn, True) for fn in fns])

    def _face_segments(self, face: str, spec):
        """A face of several types (bounding_domain masks, material.py:252-266):
        [(type, values, mask)] with the mask a boolean per boundary cell."""
        segs = []
        for seg in spec:
            if isinstance(seg, dict):
                seg = (seg.get("type"), seg.get("values"), seg.get("bounding_domain"))
            btype, vals, mask = seg
            if btype not in _lib.BC or btype == "PERIODIC":
                raise NotImplementedError(f"boundary type {btype} on a face of several types at '{face}'")
            if isinstance(mask, np.ndarray) or hasattr(mask, "numpy"):
                m = np.asarray(mask).astype(bool).reshape(-1)
                if m.shape != (self.face_cells(face),):
                    raise SetupError(f"bounding domain at '{face}': {m.shape} cells")
            else:
                m = self._eval_on_face(face, _callable(mask, f"bounding domain at '{face}'"), False)
            segs.append((btype, self._face_values(face, btype, vals), m))
            if face in self._time_fns:
                raise NotImplementedError(f"boundary values varying in time on a face of several types ('{face}')")
        cover = np.zeros(self.face_cells(face), dtype=bool)
        for _, _, m in segs:
            cover |= m
        if not cover.all():
            raise SetupError(f"the bounding domains at '{face}' leave boundary cells uncovered")
        return segs

    def face_is_mixed(self, face: str) -> bool:
        return isinstance(self.bc.get(face), list)

    def face_fields(self, face: str, values=None):
        """(values [5, nt] float64 or None, types [nt] int8 or None) of a face
        for gbf_case.bc_field_values / bc_field_types: per boundary cell the
        raw values laid out like bc_value, and for a face of several types the
        type of the last segment covering the cell (the reference's masked
        writes in face order, material.py:268-276)."""
        nt = self.face_cells(face)

        def rows(btype, vals):
            out = np.zeros((5, nt))
            if vals is None:
                return out
            arr = np.broadcast_to(np.asarray(vals, dtype=np.float64).reshape(len(vals), -1), (len(vals), nt))
            if btype == "WALL":
                out[1:4] = arr
            else:
                out[:] = arr
            return out

        if self.face_is_mixed(face):
            types = np.zeros(nt, dtype=np.int8)
            values = np.zeros((5, nt))
            any_values = False
            for btype, vals, m in self.bc[face]:
                types[m] = _lib.BC[btype]
                values[:, m] = rows(btype, vals)[:, m]
                any_values |= vals is not None
            return (values if any_values else None), types
        vals = self.bc_values.get(face) if values is None else values
        if isinstance(vals, np.ndarray):
            return rows(self.bc[face], vals), None
        return None, None

    @property
    def time_varying_faces(self):
        """Faces whose boundary values are functions of time (the drop-in
        halo update re-evaluates them at its time; the fused path, which keeps
        time on the device, rejects them)."""
        return sorted(self._time_fns)

    def bc_values_at(self, face: str, t: float) -> np.ndarray:
        """The values [k, boundary cells] of a time-varying face at time t."""
        return np.stack([self._eval_on_face(face, fn, True, t) for fn in self._time_fns[face]])

    def refresh_bc_fields(self, t: float) -> None:
        """Boundary values at time t into the device fields (stream-ordered
        copies on the current stream), for every time-varying face."""
        import torch
        for d in self._fields.values():
            for face in self._time_fns:
                vals, _ = self.face_fields(face, self.bc_values_at(face, t))
                d[face][0].copy_(torch.from_numpy(vals))

    @property
    def has_bc_fields(self) -> bool:
        return any(FACE_AXIS[f] in self.active and (self.face_is_mixed(f) or
                                                    isinstance(self.bc_values.get(f), np.ndarray))
                   for f in FACES)

    def _device_fields(self, device):
        """The face fields as tensors on `device`, kept alive by this object."""
        import torch
        key = str(device)
        if key not in self._fields:
            d = {}
            for f in FACES:
                if FACE_AXIS[f] not in self.active:
                    continue
                vals, types = self.face_fields(f)
                d[f] = (None if vals is None else torch.from_numpy(np.ascontiguousarray(vals)).to(device),
                        None if types is None else torch.from_numpy(types).to(device))
            self._fields[key] = d
        return self._fields[key]

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

    def to_c(self, device=None) -> _lib.GbfCase:
        """The gbf_case of this setup.  Boundary value fields go to `device`
        (default: the current CUDA device, or host memory without one, which
        only the host-side checks read)."""
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
        fields = None
        if self.has_bc_fields:
            import torch
            if device is None:
                device = torch.device("cuda", torch.cuda.current_device()) if torch.cuda.is_available() else "cpu"
            fields = self._device_fields(device)
        for k, f in enumerate(_lib.FACE_ORDER):
            if self.face_is_mixed(f):
                c.bc[k] = _lib.BC_MIXED
            else:
                c.bc[k] = _lib.BC[self.bc.get(f, "PERIODIC")]
            vals = self.bc_values.get(f)
            if isinstance(vals, tuple) and not self.face_is_mixed(f):
                row = [0.0, *vals, 0.0] if len(vals) == 3 else list(vals)
                for v in range(5):
                    c.bc_value[k][v] = float(row[v])
            if fields is not None and f in fields:
                fv, ft = fields[f]
                c.bc_field_values[k] = fv.data_ptr() if fv is not None else None
                c.bc_field_types[k] = ft.data_ptr() if ft is not None else None
        flags = 0
        if self.viscous:
            flags |= _lib.FLAG_VISCOUS
        if self.heat:
            flags |= _lib.FLAG_HEAT
        if self.viscous_heat_production:
            flags |= _lib.FLAG_VISCOUS_HEAT_PRODUCTION
        if not self.convective:
            flags |= _lib.FLAG_NO_CONVECTIVE
        if self.gravity is not None:
            flags |= _lib.FLAG_GRAVITY
            for i in range(3):
                c.gravity[i] = float(self.gravity[i])
        if self.interpolation_limiter:
            flags |= _lib.FLAG_INTERPOLATION_LIMITER
            if self.limit_velocity:
                flags |= _lib.FLAG_LIMIT_VELOCITY
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

        def values_of(spec, t, f):
            if t == "WALL":
                return _boundary_callables(spec.get("wall_velocity_callable", {}), ("u", "v", "w"), f)
            if t in ("DIRICHLET", "NEUMANN"):
                if spec.get("primitives_callable") is None:
                    raise NotImplementedError(f"{t} boundary at '{f}' without primitives_callable")
                return _boundary_callables(spec["primitives_callable"], ("rho", "u", "v", "w", "p"), f)
            return None

        for f in FACES:
            t = _get(case_setup, f"boundary_conditions.{f}")
            if isinstance(t, list) and len(t) == 1 and "bounding_domain" not in t[0]:
                t = t[0]  # a one-type list reads as that type
            if isinstance(t, list):
                # several types on the face (read_boundary_conditions.py:66-96)
                segs = []
                for spec in t:
                    st = spec.get("type")
                    segs.append((st, values_of(spec, st, f), spec.get("bounding_domain")))
                bc[f] = segs
                continue
            spec = t if isinstance(t, dict) else {}
            if isinstance(t, dict):
                t = t.get("type")
            if t is not None and t != "INACTIVE":
                bc[f] = t
                vals = values_of(spec, t, f)
                if vals is not None:
                    bc_values[f] = vals
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
        for key in ("is_geometric_source", "is_surface_tension"):
            if phys.get(key, False):
                raise NotImplementedError(key)
        gravity = None
        if phys.get("is_volume_force", False):
            # forcings.gravity (read_forcings / source_term_solver.py:165-186)
            g = _get(case_setup, "forcings.gravity")
            if g is None or len(g) != 3:
                raise SetupError("is_volume_force needs forcings.gravity = [gx, gy, gz]")
            gravity = tuple(float(x) for x in g)
        forcings = _get(numerical_setup, "active_forcings", {}) or {}
        for key, on in forcings.items():
            if on:
                raise NotImplementedError(f"active_forcings.{key}")
        if (_get(numerical_setup, "precision", {}) or {}).get("is_consistent_summation", False):
            raise NotImplementedError("precision.is_consistent_summation")
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
        pos = cons.get("positivity", {}) or {}
        if pos.get("flux_limiter", False):
            raise NotImplementedError(f"positivity.flux_limiter = {pos['flux_limiter']}")
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
            gravity=gravity,
            interpolation_limiter=bool(pos.get("is_interpolation_limiter", False)),
            limit_velocity=bool(pos.get("limit_velocity", False)),
            eps=float(prec.get("epsilon", EPS)) if isinstance(prec.get("epsilon"), float) else EPS,
            stencil_eps=float(prec.get("spatial_stencil_epsilon", STENCIL_EPS))
            if isinstance(prec.get("spatial_stencil_epsilon"), float) else STENCIL_EPS,
        )
