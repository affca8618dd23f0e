"""Setups shaped like the reference's single-phase examples (written here, not
copied: the same keys and kinds of values) read by CaseConfig.from_setups and
accepted by the library's case check: lid-driven cavity, Couette flow, heat
conduction with a sine Dirichlet wall, double Mach reflection, Rayleigh-Taylor
with gravity, and a viscous Taylor-Green vortex."""
import numpy as np
import pytest

from jaxfluids_gb300 import _lib
from jaxfluids_gb300.config import CaseConfig

FACES = ("east", "west", "north", "south", "top", "bottom")


def _case(cells, ranges, bcs, transport=None, **extra):
    d = {"domain": {a: {"cells": n, "range": list(r)} for a, n, r in zip("xyz", cells, ranges)},
         "boundary_conditions": {f: bcs.get(f, {"type": "INACTIVE"}) for f in FACES},
         "material_properties": {"equation_of_state": {"model": "IdealGas", "specific_heat_ratio": 1.4,
                                                       "specific_gas_constant": 1.0},
                                 "transport": transport or {}}}
    d.update(extra)
    return d


def _num(halo=4, recon="WENO5-Z", var="PRIMITIVE", riemann="HLLC", physics=None, diss=None, positivity=None):
    n = {"conservatives": {"halo_cells": halo, "time_integration": {"integrator": "RK3", "CFL": 0.5},
                           "convective_fluxes": {"convective_solver": "GODUNOV",
                                                 "godunov": {"riemann_solver": riemann, "signal_speed": "EINFELDT",
                                                             "reconstruction_stencil": recon,
                                                             "reconstruction_variable": var}}},
         "active_physics": physics or {"is_convective_flux": True}}
    if diss:
        n["conservatives"]["dissipative_fluxes"] = diss
    if positivity:
        n["conservatives"]["positivity"] = positivity
    return n


def wall(u=0.0):
    return {"type": "WALL", "wall_velocity_callable": {"u": u, "v": 0.0, "w": 0.0}}


def dirichlet(rho, u, v, p):
    return {"type": "DIRICHLET", "primitives_callable": {"rho": rho, "u": u, "v": v, "w": 0.0, "p": p}}


POST = (8.0, 7.144709581221618, -4.125, 116.5)
VISC = {"dynamic_viscosity": {"model": "CUSTOM", "value": 1e-2}, "bulk_viscosity": 0.0,
        "thermal_conductivity": {"model": "PRANDTL", "prandtl_number": 0.72}}

SETUPS = {
    "lid-driven-cavity": (
        _case((64, 64, 1), ((0, 1), (0, 1), (0, 1)),
              {"east": wall(), "west": wall(), "south": wall(), "north": wall(0.5)}, VISC),
        _num(recon="WENO5-JS", physics={"is_convective_flux": True, "is_viscous_flux": True,
                                        "is_viscous_heat_production": False},
             diss={"reconstruction_stencil": "CENTRAL4", "derivative_stencil_center": "CENTRAL4",
                   "derivative_stencil_face": "CENTRAL4"})),
    "couette": (
        _case((8, 64, 1), ((0, 1), (0, 1), (0, 1)),
              {"east": {"type": "PERIODIC"}, "west": {"type": "PERIODIC"}, "south": wall(), "north": wall(0.1)},
              VISC),
        _num(recon="WENO5-JS", physics={"is_convective_flux": False, "is_viscous_flux": True})),
    "heat-equation-2d": (
        _case((64, 64, 1), ((0, 1), (0, 1), (0, 1)),
              {"east": dirichlet(1.0, 0.0, 0.0, 1.0), "west": dirichlet(1.0, 0.0, 0.0, 1.0),
               "south": dirichlet(1.0, 0.0, 0.0, 1.0),
               "north": dirichlet(1.0, 0.0, 0.0, "lambda x,t: 1.0 + jnp.sin(jnp.pi * x)")},
              {"dynamic_viscosity": {"model": "CUSTOM", "value": 0.1}, "bulk_viscosity": 0.0,
               "thermal_conductivity": {"model": "CUSTOM", "value": 0.1}}),
        _num(recon="WENO5-JS", physics={"is_convective_flux": False, "is_heat_flux": True},
             diss={"reconstruction_stencil": "CENTRAL2", "derivative_stencil_center": "CENTRAL2",
                   "derivative_stencil_face": "CENTRAL2"})),
    "double-mach-reflection": (
        _case((128, 32, 1), ((0, 4), (0, 1), (0, 1)),
              {"east": {"type": "ZEROGRADIENT"}, "west": dirichlet(*POST), "north": {"type": "ZEROGRADIENT"},
               "south": [dict(dirichlet(*POST), bounding_domain="lambda x: x < 1.0 / 6.0"),
                         {"type": "SYMMETRY", "bounding_domain": "lambda x: x >= 1.0 / 6.0"}]}),
        _num(halo=5, var="CHAR-PRIMITIVE", positivity={"is_interpolation_limiter": True})),
    "rayleigh-taylor": (
        _case((32, 128, 1), ((0, 0.25), (0, 1), (0, 1)),
              {"east": {"type": "SYMMETRY"}, "west": {"type": "SYMMETRY"},
               "south": dirichlet(2.0, 0.0, 0.0, 1.0), "north": dirichlet(1.0, 0.0, 0.0, 2.5)},
              forcings={"gravity": [0.0, 1.0, 0.0]}),
        _num(var="CHAR-PRIMITIVE", physics={"is_convective_flux": True, "is_volume_force": True})),
    "viscous-tgv": (
        _case((32, 32, 32), ((0, 2 * np.pi),) * 3, {f: {"type": "PERIODIC"} for f in FACES}, VISC),
        _num(var="CHAR-CONSERVATIVE", physics={"is_convective_flux": True, "is_viscous_flux": True,
                                               "is_heat_flux": True})),
}


@pytest.mark.parametrize("name", list(SETUPS))
def test_example_shaped_setup_is_accepted(name):
    case, num = SETUPS[name]
    cfg = CaseConfig.from_setups(case, num)
    c = cfg.to_c()
    assert _lib.load().gbf_case_check(c) == _lib.GBF_OK
    if name == "couette":
        assert c.flags & _lib.FLAG_NO_CONVECTIVE and c.flags & _lib.FLAG_VISCOUS
    if name == "double-mach-reflection":
        assert cfg.face_is_mixed("south") and c.flags & _lib.FLAG_INTERPOLATION_LIMITER
    if name == "rayleigh-taylor":
        assert c.flags & _lib.FLAG_GRAVITY and cfg.gravity == (0.0, 1.0, 0.0)
    if name == "heat-equation-2d":
        assert isinstance(cfg.bc_values["north"], np.ndarray) and not cfg.time_varying_faces
