"""Golden vectors computed by the reference's own source code.

JAX-Fluids is pure Python on top of jax.numpy.  jax and jaxlib are installed
on neither machine, so this script runs the reference package unmodified,
from its checkout, under ``jaxshim`` (a numpy stand-in for the jax API it
calls; float64, one IEEE rounding per operation).  The whole single-phase path
executes as the reference wrote it: ``InputManager`` reads the setup
dictionaries, ``InitializationManager.initialization(user_prime_init=...)``
builds the buffers and fills the halos, ``SpaceSolver.compute_rhs`` gives the
right-hand side of the initial state, and ``SimulationManager._do_integration_step``
advances the TVD-RK3 steps with the CFL time step.

Cases (seeded synthetic inputs):

* ``sod``            - 1-D Sod, 200 cells, WENO5-Z + HLLC/Einfeldt, CFL 0.5, to t = 0.2
* ``tgv32``          - 3-D inviscid Taylor-Green vortex, 32^3 periodic (the 128^3
                       workload's initial condition on a coarser grid), 2 steps
* ``tgv24-visc-char-roe`` - viscous TGV, 24^3, Re 1600, Pr 0.71, WENO5-Z on
                       Roe-characteristic variables + HLLC + CENTRAL4 viscous and heat fluxes
* ``quad64``         - 2-D four-quadrant Riemann problem, 64^2, states from default_rng(1000)
* ``kh64``           - 2-D Kelvin-Helmholtz, 64^2 periodic, noise from default_rng(7)
* scheme variants on a perturbed 2-D quadrant problem (40 x 32): CHAR-PRIMITIVE
  with the ARITHMETIC frozen state, Rusanov, the HLLC signal speeds, WENO5-JS +
  HLL, TENO5, WENO3-JS, WENO3-Z, CONSERVATIVE, CHAR-CONSERVATIVE, Lax-Friedrichs
* boundary variants with viscous and heat fluxes: a lid-driven cavity (WALL),
  a channel with DIRICHLET / NEUMANN / SYMMETRY / WALL faces, and a 3-D box
  with ZEROGRADIENT / SYMMETRY / PERIODIC faces (edge halos)

Each ``ref/<case>.npz`` holds the two setup dictionaries (JSON), the initial
primitives passed as ``user_prime_init`` (``prims0``, rho, the active
velocities, p), the interior right-hand side of the initial state (``rhs0``),
the time steps used (``dts``; the last entry is the time step of the final
state), the final time and the interior conservatives (and, for the small
cases, primitives) after the steps.

Run from the repository root, with the reference checkout at REFERENCE
(default /root/reference):  python tests/golden/make_ref_fixtures.py [case ...]
Nothing is written into the reference tree (no bytecode).  The outputs are
committed; the tests never read the reference.
"""
import sys

sys.dont_write_bytecode = True  # noqa: E402 (before any import of the reference)

import json
import math
import os
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REFERENCE = os.environ.get("REFERENCE", "/root/reference")
OUT = os.path.join(HERE, "ref")
FACES = ("east", "west", "north", "south", "top", "bottom")


# ------------------------------------------------------------------ setups
def case_setup(cells, ranges, bcs, transport=None, gamma=1.4, end_time=1.0):
    d = {
        "general": {"case_name": "fixture", "save_path": "/tmp/jf_fixture_out", "end_time": end_time,
                    "save_dt": end_time},
        "domain": {a: {"cells": int(n), "range": [float(r[0]), float(r[1])]} for a, n, r in zip("xyz", cells, ranges)},
        "boundary_conditions": {f: bcs.get(f, {"type": "INACTIVE"}) for f in FACES},
        "initial_condition": {"rho": 1.0, "u": 0.0, "v": 0.0, "w": 0.0, "p": 1.0},
        "material_properties": {"equation_of_state": {"model": "IdealGas", "specific_heat_ratio": gamma,
                                                      "specific_gas_constant": 1.0}},
        "output": {"primitives": ["density", "velocity", "pressure"]},
    }
    if transport:
        d["material_properties"]["transport"] = transport
    return d


def numerical_setup(nh=3, recon="WENO5-Z", var="PRIMITIVE", frozen=None, riemann="HLLC", speed="EINFELDT",
                    cfl=0.5, viscous=False, heat=False, heat_production=True, diss=None):
    g = {"riemann_solver": riemann, "signal_speed": speed, "reconstruction_stencil": recon,
         "reconstruction_variable": var}
    if frozen:
        g["frozen_state"] = frozen
    n = {
        "conservatives": {
            "halo_cells": nh,
            "time_integration": {"integrator": "RK3", "CFL": cfl},
            "convective_fluxes": {"convective_solver": "GODUNOV", "godunov": g},
        },
        "active_physics": {"is_convective_flux": True, "is_viscous_flux": viscous, "is_heat_flux": heat,
                           "is_volume_force": False, "is_viscous_heat_production": heat_production},
        "precision": {"is_double_precision_compute": True, "is_double_precision_output": True},
        "output": {"is_active": False, "is_xdmf": False},
    }
    if viscous or heat:
        n["conservatives"]["dissipative_fluxes"] = diss or {
            "reconstruction_stencil": "CENTRAL4", "derivative_stencil_center": "CENTRAL4",
            "derivative_stencil_face": "CENTRAL4"}
    return n


def transport(mu, prandtl=None, kappa=None):
    t = {"dynamic_viscosity": {"model": "CUSTOM", "value": mu}, "bulk_viscosity": 0.0}
    if prandtl is not None:
        t["thermal_conductivity"] = {"model": "PRANDTL", "prandtl_number": prandtl}
    else:
        t["thermal_conductivity"] = {"model": "CUSTOM", "value": kappa or 0.0}
    return t


def periodic(faces=FACES):
    return {f: {"type": "PERIODIC"} for f in faces}


def zerogradient(faces=FACES):
    return {f: {"type": "ZEROGRADIENT"} for f in faces}


def wall(u=0.0, v=0.0):
    return {"type": "WALL", "wall_velocity_callable": {"u": u, "v": v, "w": 0.0}}


def dirichlet(rho, u, v, p):
    return {"type": "DIRICHLET", "primitives_callable": {"rho": rho, "u": u, "v": v, "w": 0.0, "p": p}}


def neumann(rho, u, v, p):
    return {"type": "NEUMANN", "primitives_callable": {"rho": rho, "u": u, "v": v, "w": 0.0, "p": p}}


# ------------------------------------------------------------------ initial primitives
def centers(n, lo, hi):
    return lo + (np.arange(n) + 0.5) * ((hi - lo) / n)


def sod_prims(n=200):
    x = centers(n, 0.0, 1.0)
    rho = np.where(x <= 0.5, 1.0, 0.125)
    p = np.where(x <= 0.5, 1.0, 0.1)
    return np.stack([rho, np.zeros(n), p]).reshape(3, n, 1, 1)


def tgv_prims(n, ma=0.1, gamma=1.4):
    """u = sin x cos y cos z, v = -cos x sin y cos z, w = 0, rho = 1,
    p = p0 + (cos 2x + cos 2y)(cos 2z + 2)/16, p0 = 1/(gamma Ma^2) on [0, 2 pi]^3."""
    p0 = 1.0 / (gamma * ma * ma)
    x = centers(n, 0.0, 2 * math.pi)
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    u = np.sin(X) * np.cos(Y) * np.cos(Z)
    v = -np.cos(X) * np.sin(Y) * np.cos(Z)
    p = p0 + (np.cos(2 * X) + np.cos(2 * Y)) * (np.cos(2 * Z) + 2.0) / 16.0
    return np.stack([np.ones_like(X), u, v, np.zeros_like(X), p])


def quadrant_prims(nx, ny, seed):
    """Four-quadrant Riemann problem on [0,1]^2 split at (0.5, 0.5): per quadrant
    rho ~ U[0.1, 2], u, v ~ U[-1, 1], p ~ U[0.1, 2] from default_rng(seed)."""
    rng = np.random.default_rng(seed)
    st = np.stack([rng.uniform(0.1, 2, 4), rng.uniform(-1, 1, 4), rng.uniform(-1, 1, 4), rng.uniform(0.1, 2, 4)])
    X, Y = np.meshgrid(centers(nx, 0, 1), centers(ny, 0, 1), indexing="ij")
    q = (X >= 0.5).astype(int) + 2 * (Y >= 0.5).astype(int)
    return st[:, q].reshape(4, nx, ny, 1)


def smooth(shape, seed, amp):
    """Seeded sum of three random-phase cosine modes varying along every axis of `shape`."""
    rng = np.random.default_rng(seed)
    axes = [(np.arange(n) + 0.5) / n for n in shape]
    X = np.meshgrid(*axes, indexing="ij")
    f = np.zeros(shape)
    for _ in range(3):
        k = rng.integers(1, 3, size=len(shape))
        ph = rng.uniform(0, 2 * np.pi, size=len(shape))
        term = np.ones(shape)
        for a in range(len(shape)):
            if shape[a] > 1:
                term = term * np.cos(2 * np.pi * k[a] * X[a] + ph[a])
        f = f + amp * rng.uniform(0.3, 1.0) * term
    return f


def perturbed_quadrant(nx, ny, seed):
    P = quadrant_prims(nx, ny, seed)
    for v in range(4):
        P[v] = P[v] + smooth((nx, ny, 1), seed + 10 + v, 0.05)
    return P


def kh_prims(n, seed):
    """rho = 2, u = 0.5 for |y - 0.5| < 0.25, else rho = 1, u = -0.5; p = 2.5;
    v = 0.01 sin(4 pi x) + N(0, 1e-3) noise from default_rng(seed)."""
    rng = np.random.default_rng(seed)
    X, Y = np.meshgrid(centers(n, 0, 1), centers(n, 0, 1), indexing="ij")
    inner = np.abs(Y - 0.5) < 0.25
    rho = np.where(inner, 2.0, 1.0)
    u = np.where(inner, 0.5, -0.5)
    v = 0.01 * np.sin(4 * np.pi * X) + rng.normal(0.0, 1e-3, X.shape)
    return np.stack([rho, u, v, np.full_like(X, 2.5)]).reshape(4, n, n, 1)


def smooth3d_prims(shape, seed):
    return np.stack([1.0 + smooth(shape, seed, 0.2), smooth(shape, seed + 1, 0.3), smooth(shape, seed + 2, 0.3),
                     smooth(shape, seed + 3, 0.3), 1.0 + smooth(shape, seed + 4, 0.2)])


def cavity_prims(n):
    X, Y = np.meshgrid(centers(n, 0, 1), centers(n, 0, 1), indexing="ij")
    sh = (n, n, 1)
    return np.stack([1.0 + smooth(sh, 41, 0.05), smooth(sh, 42, 0.1), smooth(sh, 43, 0.1),
                     1.0 + smooth(sh, 44, 0.05)]).reshape(4, n, n, 1)


UNIT = ((0.0, 1.0),) * 3
TWO_PI = ((0.0, 2 * math.pi),) * 3
Q2 = dict(cells=(40, 32, 1), ranges=UNIT)


def _quad_variant(num, seed=3, bcs=None):
    return dict(case=case_setup(Q2["cells"], Q2["ranges"], bcs or zerogradient(FACES[:4])), num=num,
                prims=lambda: perturbed_quadrant(40, 32, seed), steps=3, keep_prims=True)


CASES = {
    "sod": dict(case=case_setup((200, 1, 1), UNIT, zerogradient(FACES[:2]), end_time=0.2),
                num=numerical_setup(), prims=lambda: sod_prims(200), steps="end", keep_prims=True),
    "tgv32": dict(case=case_setup((32, 32, 32), TWO_PI, periodic()), num=numerical_setup(),
                  prims=lambda: tgv_prims(32), steps=2, keep_prims=False),
    "tgv24-visc-char-roe": dict(
        case=case_setup((24, 24, 24), TWO_PI, periodic(), transport(1.0 / 1600, prandtl=0.71)),
        num=numerical_setup(nh=4, var="CHAR-PRIMITIVE", frozen="ROE", viscous=True, heat=True),
        prims=lambda: tgv_prims(24), steps=2, keep_prims=False),
    "quad64": dict(case=case_setup((64, 64, 1), UNIT, zerogradient(FACES[:4])), num=numerical_setup(),
                   prims=lambda: quadrant_prims(64, 64, 1000), steps=5, keep_prims=True),
    "kh64": dict(case=case_setup((64, 64, 1), UNIT, periodic(FACES[:4])), num=numerical_setup(),
                 prims=lambda: kh_prims(64, 7), steps=5, keep_prims=True),
    "q2-char-arith": _quad_variant(numerical_setup(var="CHAR-PRIMITIVE", frozen="ARITHMETIC")),
    "q2-char-roe-rusanov": _quad_variant(numerical_setup(var="CHAR-PRIMITIVE", frozen="ROE", riemann="RUSANOV")),
    "q2-rusanov": _quad_variant(numerical_setup(riemann="RUSANOV")),
    "q2-speed-davis": _quad_variant(numerical_setup(speed="DAVIS")),
    "q2-speed-toro": _quad_variant(numerical_setup(speed="TORO")),
    "q2-speed-arithmetic": _quad_variant(numerical_setup(speed="ARITHMETIC")),
    "q2-speed-rusanov": _quad_variant(numerical_setup(speed="RUSANOV")),
    "q2-weno5js-hll": _quad_variant(numerical_setup(recon="WENO5-JS", riemann="HLL")),
    "q2-teno5": _quad_variant(numerical_setup(recon="TENO5")),
    "q2-weno3js": _quad_variant(numerical_setup(recon="WENO3-JS")),
    "q2-weno3z": _quad_variant(numerical_setup(recon="WENO3-Z")),
    "q2-conservative": _quad_variant(numerical_setup(var="CONSERVATIVE")),
    "q2-char-conservative": _quad_variant(numerical_setup(var="CHAR-CONSERVATIVE")),
    "q2-lax-friedrichs": _quad_variant(numerical_setup(riemann="LAX-FRIEDRICHS")),
    "q2-symmetry-periodic": _quad_variant(numerical_setup(), seed=5, bcs={
        "east": {"type": "PERIODIC"}, "west": {"type": "PERIODIC"},
        "north": {"type": "SYMMETRY"}, "south": {"type": "SYMMETRY"}}),
    "cavity32-visc-heat": dict(
        case=case_setup((32, 32, 1), UNIT, {"east": wall(), "west": wall(), "south": wall(), "north": wall(0.5)},
                        transport(1e-2, prandtl=0.72)),
        num=numerical_setup(nh=4, viscous=True, heat=True), prims=lambda: cavity_prims(32), steps=3,
        keep_prims=True),
    "channel-bc-visc-heat": dict(
        case=case_setup((24, 20, 1), UNIT, {"west": dirichlet(1.2, 0.3, 0.05, 1.1), "east": neumann(0.0, 0.1, 0.0, -0.2),
                                            "north": {"type": "SYMMETRY"}, "south": wall(0.2)},
                        transport(5e-3, kappa=4e-3)),
        num=numerical_setup(nh=4, viscous=True, heat=True), prims=lambda: perturbed_quadrant(24, 20, 9), steps=3,
        keep_prims=True),
    "box3d-mixed-char-roe-visc": dict(
        case=case_setup((16, 12, 10), TWO_PI, {"east": {"type": "ZEROGRADIENT"}, "west": {"type": "ZEROGRADIENT"},
                                               "north": {"type": "SYMMETRY"}, "south": {"type": "SYMMETRY"},
                                               "top": {"type": "PERIODIC"}, "bottom": {"type": "PERIODIC"}},
                        transport(2e-3, prandtl=0.71)),
        num=numerical_setup(nh=4, var="CHAR-PRIMITIVE", frozen="ROE", viscous=True, heat=True),
        prims=lambda: smooth3d_prims((16, 12, 10), 21), steps=2, keep_prims=True),
}


# ------------------------------------------------------------------ reference run
def load_reference():
    sys.path.insert(0, HERE)
    import jaxshim
    jaxshim.install()
    jaxshim.install_stubs()
    sys.path.insert(0, os.path.join(REFERENCE, "src"))
    import logging
    logging.disable(logging.CRITICAL)
    import jaxfluids
    from jaxfluids.data_types import ml_buffers
    return jaxfluids, ml_buffers


def run_case(name, spec, jf, ml):
    import io
    import contextlib
    with contextlib.redirect_stdout(io.StringIO()):
        im = jf.InputManager(spec["case"], spec["num"])
        init = jf.InitializationManager(im)
        sim = jf.SimulationManager(im)
        prims0 = np.ascontiguousarray(spec["prims"](), dtype=np.float64)
        buf = init.initialization(user_prime_init=prims0)
    dom = sim.domain_information
    nhx, nhy, nhz = dom.domain_slices_conservatives
    mf = buf.simulation_buffers.material_fields
    tcv = buf.time_control_variables
    rhs_buf, _, _ = sim.space_solver.compute_rhs(
        mf.conservatives, mf.primitives, mf.temperature, tcv.physical_simulation_time,
        tcv.physical_timestep_size,
        ml_setup=ml.combine_callables_and_params(ml.CallablesSetup(), ml.ParametersSetup()))
    rhs0 = np.asarray(rhs_buf.euler_buffers.conservatives)
    dts = [float(tcv.physical_timestep_size)]
    steps = spec["steps"]
    end_time = spec["case"]["general"]["end_time"]
    k = 0
    while (steps == "end" and float(tcv.physical_simulation_time) < end_time) or (steps != "end" and k < steps):
        cfp = sim.compute_control_flow_params(tcv, buf.step_information)
        buf, _ = sim._do_integration_step(buf, cfp, ml.ParametersSetup(), ml.CallablesSetup())
        tcv = buf.time_control_variables
        dts.append(float(tcv.physical_timestep_size))
        k += 1
    mf = buf.simulation_buffers.material_fields
    out = {
        "case_setup": np.array(json.dumps(spec["case"])),
        "numerical_setup": np.array(json.dumps(spec["num"])),
        "prims0": prims0,
        "rhs0": rhs0,
        "dts": np.array(dts),
        "t": np.array(float(tcv.physical_simulation_time)),
        "steps": np.array(k),
        "cons": np.ascontiguousarray(np.asarray(mf.conservatives)[..., nhx, nhy, nhz]),
    }
    if spec.get("keep_prims"):
        out["prims"] = np.ascontiguousarray(np.asarray(mf.primitives)[..., nhx, nhy, nhz])
    return out


def main(argv):
    names = argv or list(CASES)
    jf, ml = load_reference()
    os.makedirs(OUT, exist_ok=True)
    for name in names:
        t0 = time.time()
        out = run_case(name, CASES[name], jf, ml)
        np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **out)
        print(f"{name}: {int(out['steps'])} steps, t = {float(out['t']):.6g}, {time.time() - t0:.1f} s", flush=True)


if __name__ == "__main__":
    main(sys.argv[1:])
