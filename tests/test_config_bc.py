"""Boundary conditions read from the reference's case_setup dictionaries
(input/case_setup/read_boundary_conditions.py layout) into the C descriptor."""
import numpy as np
import pytest

from jaxfluids_gb300 import _lib
from jaxfluids_gb300.config import CaseConfig, SetupError


def _setup(bcs, cells=(32, 24, 1)):
    case = {
        "domain": {a: {"cells": n, "range": [0.0, 1.0]} for a, n in zip("xyz", cells)},
        "boundary_conditions": bcs,
        "material_properties": {"equation_of_state": {"model": "IdealGas", "specific_heat_ratio": 1.4,
                                                      "specific_gas_constant": 1.0}},
    }
    num = {"conservatives": {"halo_cells": 4, "time_integration": {"integrator": "RK3", "CFL": 0.5}}}
    return case, num


def test_cavity_walls_and_lid_velocity():
    wall = {"type": "WALL", "wall_velocity_callable": {"u": 0.0, "v": 0.0, "w": 0.0}}
    lid = {"type": "WALL", "wall_velocity_callable": {"u": 5e-1, "v": 0.0, "w": 0.0}}
    case, num = _setup({"east": wall, "west": wall, "north": lid, "south": wall,
                        "top": {"type": "INACTIVE"}, "bottom": {"type": "INACTIVE"}})
    cfg = CaseConfig.from_setups(case, num)
    assert cfg.bc["north"] == "WALL" and cfg.bc_values["north"] == (0.5, 0.0, 0.0)
    c = cfg.to_c()
    k = _lib.FACE_ORDER.index("north")
    assert c.bc[k] == _lib.BC["WALL"]
    assert list(c.bc_value[k]) == [0.0, 0.5, 0.0, 0.0, 0.0]


def test_dirichlet_inflow_and_neumann_outflow():
    inflow = {"type": "DIRICHLET", "primitives_callable": {"rho": 8.0, "u": 7.144709581221618, "v": -4.125,
                                                           "w": 0.0, "p": 116.5}}
    outflow = {"type": "NEUMANN", "primitives_callable": {"rho": 0.0, "u": "0.5", "v": 0.0, "w": 0.0, "p": 0.0}}
    case, num = _setup({"west": inflow, "east": outflow, "north": {"type": "ZEROGRADIENT"},
                        "south": [{"type": "SYMMETRY"}], "top": {"type": "INACTIVE"},
                        "bottom": {"type": "INACTIVE"}})
    cfg = CaseConfig.from_setups(case, num)
    c = cfg.to_c()
    w, e = _lib.FACE_ORDER.index("west"), _lib.FACE_ORDER.index("east")
    assert list(c.bc_value[w]) == [8.0, 7.144709581221618, -4.125, 0.0, 116.5]
    assert c.bc[e] == _lib.BC["NEUMANN"] and list(c.bc_value[e]) == [0.0, 0.5, 0.0, 0.0, 0.0]
    assert _lib.load().gbf_case_check(c) == _lib.GBF_OK


def test_callables_of_the_boundary_coordinates():
    """Lambda strings are evaluated at the boundary cells' centres
    (get_boundary_coordinates_at_location, boundary_condition.py:105-126;
    homogenous.py:13-14) with numpy in place of jax.numpy."""
    f = {"type": "DIRICHLET", "primitives_callable": {"rho": "lambda y, t: 1.0 + y", "u": 0.0, "v": 0.0,
                                                      "w": 0.0, "p": "lambda y,t: 1.0 + jnp.sin(jnp.pi * y)"}}
    case, num = _setup({"west": f, "east": {"type": "ZEROGRADIENT"}, "north": {"type": "ZEROGRADIENT"},
                        "south": {"type": "ZEROGRADIENT"}})
    cfg = CaseConfig.from_setups(case, num)
    ny = cfg.cells[1]
    lo, hi = cfg.ranges[1]
    dy = (hi - lo) / ny
    y = np.linspace(lo + dy / 2, hi - dy / 2, ny)
    vals = cfg.bc_values["west"]
    assert vals.shape == (5, ny)
    np.testing.assert_array_equal(vals[0], 1.0 + y)
    np.testing.assert_array_equal(vals[4], 1.0 + np.sin(np.pi * y))
    np.testing.assert_array_equal(vals[1:4], 0.0)
    fv, ft = cfg.face_fields("west")
    assert ft is None and fv.shape == (5, ny)
    c = cfg.to_c()
    w = _lib.FACE_ORDER.index("west")
    assert c.bc[w] == _lib.BC["DIRICHLET"] and c.bc_field_values[w] and not c.bc_field_types[w]
    assert _lib.load().gbf_case_check(c) == _lib.GBF_OK


def test_time_varying_callables():
    """Callables of time are detected, evaluated at the halo update's time,
    and rejected by the fused path (time lives on the device there)."""
    f = {"type": "DIRICHLET", "primitives_callable": {"rho": "lambda y, t: 1.0 + t * y", "u": 0.0, "v": 0.0,
                                                      "w": 0.0, "p": 1.0}}
    case, num = _setup({"west": f, "east": {"type": "ZEROGRADIENT"}, "north": {"type": "ZEROGRADIENT"},
                        "south": {"type": "ZEROGRADIENT"}})
    cfg = CaseConfig.from_setups(case, num)
    assert cfg.time_varying_faces == ["west"]
    ny = cfg.cells[1]
    y = (np.arange(ny) + 0.5) / ny
    np.testing.assert_array_equal(cfg.bc_values_at("west", 0.25)[0], 1.0 + 0.25 * y)
    np.testing.assert_array_equal(cfg.bc_values["west"][0], np.ones(ny))  # t = 0
    from jaxfluids_gb300 import FusedRK3
    with pytest.raises(NotImplementedError, match="time"):
        FusedRK3(cfg, device="cpu")
    mixed = [dict(f, bounding_domain="lambda y: y < 0.5"), {"type": "SYMMETRY", "bounding_domain": "lambda y: y >= 0.5"}]
    case, num = _setup({"west": mixed, "east": {"type": "ZEROGRADIENT"}, "north": {"type": "ZEROGRADIENT"},
                        "south": {"type": "ZEROGRADIENT"}})
    with pytest.raises(NotImplementedError, match="time"):
        CaseConfig.from_setups(case, num)


def test_face_of_several_types():
    """bounding_domain masks (material.py:252-276): per boundary cell the type
    of the last segment covering it, its values in the value field."""
    mixed = [{"type": "DIRICHLET", "primitives_callable": {"rho": 1.0, "u": 0.0, "v": 0.0, "w": 0.0, "p": 1.0},
              "bounding_domain": "lambda x: x < 0.5"}, {"type": "SYMMETRY", "bounding_domain": "lambda x: x >= 0.5"}]
    case, num = _setup({"west": {"type": "ZEROGRADIENT"}, "east": {"type": "ZEROGRADIENT"},
                        "north": {"type": "ZEROGRADIENT"}, "south": mixed})
    cfg = CaseConfig.from_setups(case, num)
    assert cfg.face_is_mixed("south")
    nx = cfg.cells[0]
    x = (np.arange(nx) + 0.5) / nx
    fv, ft = cfg.face_fields("south")
    np.testing.assert_array_equal(ft, np.where(x < 0.5, _lib.BC["DIRICHLET"], _lib.BC["SYMMETRY"]))
    np.testing.assert_array_equal(fv[0], np.where(x < 0.5, 1.0, 0.0))
    c = cfg.to_c()
    s = _lib.FACE_ORDER.index("south")
    assert c.bc[s] == _lib.BC_MIXED and c.bc_field_types[s] and c.bc_field_values[s]
    assert _lib.load().gbf_case_check(c) == _lib.GBF_OK
    # the library wants per-cell types exactly on MIXED faces
    c.bc_field_types[s] = None
    assert _lib.load().gbf_case_check(c) == _lib.GBF_ERR_INVALID_ARGUMENT
    # uncovered boundary cells and PERIODIC segments are rejected
    gap = [dict(mixed[0]), {"type": "SYMMETRY", "bounding_domain": "lambda x: x >= 0.75"}]
    case, num = _setup({"west": {"type": "ZEROGRADIENT"}, "east": {"type": "ZEROGRADIENT"},
                        "north": {"type": "ZEROGRADIENT"}, "south": gap})
    with pytest.raises(SetupError, match="uncovered"):
        CaseConfig.from_setups(case, num)
    per = [dict(mixed[0]), {"type": "PERIODIC", "bounding_domain": "lambda x: x >= 0.5"}]
    case, num = _setup({"west": {"type": "ZEROGRADIENT"}, "east": {"type": "ZEROGRADIENT"},
                        "north": {"type": "ZEROGRADIENT"}, "south": per})
    with pytest.raises(NotImplementedError):
        CaseConfig.from_setups(case, num)


def test_positivity_setup():
    case, num = _setup({"west": {"type": "ZEROGRADIENT"}, "east": {"type": "ZEROGRADIENT"},
                        "north": {"type": "ZEROGRADIENT"}, "south": {"type": "ZEROGRADIENT"}})
    num["conservatives"]["positivity"] = {"is_interpolation_limiter": True}
    cfg = CaseConfig.from_setups(case, num)
    assert cfg.interpolation_limiter and not cfg.limit_velocity
    assert cfg.to_c().flags & _lib.FLAG_INTERPOLATION_LIMITER
    num["conservatives"]["positivity"] = {"flux_limiter": "NASA"}
    with pytest.raises(NotImplementedError, match="flux_limiter"):
        CaseConfig.from_setups(case, num)


def test_wall_needs_its_velocity():
    with pytest.raises(SetupError):
        CaseConfig(cells=(16, 1, 1), bc={"west": "WALL", "east": "ZEROGRADIENT"})


def test_viscous_walls_accepted_by_the_library():
    cfg = CaseConfig(cells=(16, 16, 1), nh=4, viscous=True, heat=True, mu=0.01, prandtl=0.71,
                     bc={f: "WALL" for f in ("east", "west", "north", "south")},
                     bc_values={f: (0.0, 0.0, 0.0) for f in ("east", "west", "north", "south")})
    assert _lib.load().gbf_case_check(cfg.to_c()) == _lib.GBF_OK


@pytest.mark.parametrize("recon,center,nh,ok", [
    ("CENTRAL4", "CENTRAL4", 4, True), ("CENTRAL4", "CENTRAL4", 3, False),
    ("CENTRAL2", "CENTRAL4", 3, True), ("CENTRAL4", "CENTRAL2", 3, True), ("CENTRAL2", "CENTRAL2", 3, True)])
def test_dissipative_stencil_halos(recon, center, nh, ok):
    """Centre derivatives cover a ring as wide as the reconstruction's halos
    (source_term_solver.py:57-79): the case needs nh >= both halo widths."""
    kw = dict(cells=(16, 16, 1), bc={f: "PERIODIC" for f in ("east", "west", "north", "south", "top", "bottom")},
              viscous=True, mu=0.01, diss_recon=recon, diss_deriv_center=center,
              diss_deriv_face="CENTRAL2")
    if ok:
        cfg = CaseConfig(nh=nh, **kw)
        assert _lib.load().gbf_case_check(cfg.to_c()) == _lib.GBF_OK
        c = cfg.to_c()
        c.nh = nh - 1
        assert _lib.load().gbf_case_check(c) == _lib.GBF_ERR_INVALID_ARGUMENT
    else:
        with pytest.raises(SetupError):
            CaseConfig(nh=nh, **kw)
        c = CaseConfig(nh=4, **kw).to_c()
        c.nh = nh
        assert _lib.load().gbf_case_check(c) == _lib.GBF_ERR_INVALID_ARGUMENT


def test_dissipative_stencils_from_setup():
    case = {"domain": {"x": {"cells": 16, "range": [0, 1]}, "y": {"cells": 16, "range": [0, 1]},
                       "z": {"cells": 1, "range": [0, 1]}},
            "boundary_conditions": {f: {"type": "PERIODIC"} for f in ("east", "west", "north", "south",
                                                                      "top", "bottom")},
            "material_properties": {"equation_of_state": {"model": "IdealGas", "specific_heat_ratio": 1.4,
                                                          "specific_gas_constant": 1.0},
                                    "transport": {"dynamic_viscosity": {"model": "CUSTOM", "value": 0.01},
                                                  "bulk_viscosity": 0.0,
                                                  "thermal_conductivity": {"model": "PRANDTL", "prandtl_number": 0.72}}}}
    num = {"conservatives": {"halo_cells": 3,
                             "dissipative_fluxes": {"reconstruction_stencil": "CENTRAL2",
                                                    "derivative_stencil_center": "CENTRAL2",
                                                    "derivative_stencil_face": "CENTRAL2"}},
           "active_physics": {"is_convective_flux": True, "is_viscous_flux": True, "is_heat_flux": True}}
    cfg = CaseConfig.from_setups(case, num)
    assert (cfg.diss_recon, cfg.diss_deriv_center, cfg.diss_deriv_face) == ("CENTRAL2",) * 3
    c = cfg.to_c()
    assert list(c.dissipative_stencil) == [_lib.CENTRAL["CENTRAL2"]] * 3
    assert _lib.load().gbf_case_check(c) == _lib.GBF_OK


def test_gravity_from_setup():
    """active_physics.is_volume_force with forcings.gravity (the Rayleigh-Taylor
    example's keys); other forcings and consistent summation are rejected."""
    case, num = _setup({"west": {"type": "SYMMETRY"}, "east": {"type": "SYMMETRY"},
                        "north": {"type": "ZEROGRADIENT"}, "south": {"type": "ZEROGRADIENT"}})
    case["forcings"] = {"gravity": [0.0, 1.0, 0.0]}
    num["active_physics"] = {"is_convective_flux": True, "is_volume_force": True}
    cfg = CaseConfig.from_setups(case, num)
    assert cfg.gravity == (0.0, 1.0, 0.0)
    c = cfg.to_c()
    assert c.flags & _lib.FLAG_GRAVITY and list(c.gravity) == [0.0, 1.0, 0.0]
    assert _lib.load().gbf_case_check(c) == _lib.GBF_OK
    num["active_forcings"] = {"is_mass_flow_forcing": True}
    with pytest.raises(NotImplementedError, match="mass_flow"):
        CaseConfig.from_setups(case, num)
    del num["active_forcings"]
    num["precision"] = {"is_consistent_summation": True}
    with pytest.raises(NotImplementedError, match="consistent"):
        CaseConfig.from_setups(case, num)


def _zg_setup():
    return _setup({f: {"type": "ZEROGRADIENT"} for f in ("west", "east", "north", "south")})


def _set(d, path, value):
    keys = path.split(".")
    for k in keys[:-1]:
        d = d.setdefault(k, {})
    d[keys[-1]] = value


# (which dictionary, key path, value): settings of the reference's setups
# outside the single-phase path this package builds
NOT_BUILT = [
    ("case", "boundary_conditions.east", {"type": "ISOTHERMALWALL"}),
    ("case", "boundary_conditions.east", {"type": "LINEAREXTRAPOLATION"}),
    ("case", "boundary_conditions.west", {"type": "SIMPLE_INFLOW"}),
    ("case", "material_properties.equation_of_state", {"model": "StiffenedGas"}),
    ("num", "conservatives.convective_fluxes.godunov.reconstruction_stencil", "WENO7"),
    ("num", "conservatives.convective_fluxes.godunov.reconstruction_stencil", "ALDM"),
    ("num", "conservatives.convective_fluxes.godunov.riemann_solver", "HLLC-LM"),
    ("num", "conservatives.convective_fluxes.godunov.riemann_solver", "AUSMP"),
    ("num", "conservatives.convective_fluxes.convective_solver", "FLUX-SPLITTING"),
    ("num", "conservatives.time_integration.integrator", "RK2"),
    ("num", "active_physics.is_geometric_source", True),
    ("num", "active_physics.is_surface_tension", True),
    ("num", "conservatives.dissipative_fluxes.is_laplacian", True),
    ("num", "precision.is_double_precision_compute", False),
    ("num", "active_forcings.is_turb_hit_forcing", True),
]


@pytest.mark.parametrize("where,path,value", NOT_BUILT, ids=[f"{p}={v}" for _, p, v in NOT_BUILT])
def test_settings_outside_the_path_are_rejected(where, path, value):
    """Raised while reading the setups, before any device work."""
    case, num = _zg_setup()
    _set(case if where == "case" else num, path, value)
    with pytest.raises(NotImplementedError):
        CaseConfig.from_setups(case, num)


def test_viscosity_and_conductivity_models_outside_the_path_are_rejected():
    case, num = _zg_setup()
    num["active_physics"] = {"is_viscous_flux": True}
    case["material_properties"]["transport"] = {"dynamic_viscosity": {"model": "SUTHERLAND"}}
    with pytest.raises(NotImplementedError):
        CaseConfig.from_setups(case, num)
    num["active_physics"] = {"is_viscous_flux": True, "is_heat_flux": True}
    case["material_properties"]["transport"] = {"dynamic_viscosity": {"model": "CUSTOM", "value": 1e-3},
                                                "thermal_conductivity": {"model": "SUTHERLAND"}}
    with pytest.raises(NotImplementedError):
        CaseConfig.from_setups(case, num)
    case["material_properties"]["transport"]["thermal_conductivity"] = {"model": "PRANDTL", "prandtl_number": 0.72}
    cfg = CaseConfig.from_setups(case, num)
    assert cfg.viscous and cfg.heat and abs(cfg.kappa - 3.5 * 1e-3 / 0.72) <= 1e-18
