"""The oracle against golden vectors computed by the reference's own source.

tests/golden/make_ref_fixtures.py ran JAX-Fluids' InputManager,
InitializationManager, SpaceSolver.compute_rhs and
SimulationManager._do_integration_step, unmodified, on seeded inputs (jax
replaced by a float64 numpy stand-in, one IEEE rounding per operation).  The
oracle must reproduce every fixture bitwise: the right-hand side of the
initial state, every CFL time step, and the state after the steps.
"""
import numpy as np
import pytest
import torch

from oracle import jf_oracle as O
from tests import refcases

NAMES = refcases.names()


def test_fixtures_present():
    for name in ("sod", "tgv32", "tgv24-visc-char-roe", "quad64", "kh64"):
        assert name in NAMES


@pytest.mark.parametrize("name", NAMES)
def test_oracle_matches_reference_source(name):
    fx = refcases.load(name)
    oc, _ = refcases.configs(fx)
    U, P = O.initialize(refcases.prims0(fx), oc)
    rhs = O.compute_rhs(U, P, oc)
    inner = oc.interior()
    dt = O.compute_dt(P, oc)
    dts = [float(dt)]
    t = 0.0
    for _ in range(fx["steps"]):
        U, P = O.rk3_step(U, P, dt, oc, t)
        t = t + float(dt)
        dt = O.compute_dt(P, oc)
        dts.append(float(dt))
    assert np.array_equal(rhs.numpy(), fx["rhs0"]), refcases.rel_diff(rhs.numpy(), fx["rhs0"])
    assert dts == list(fx["dts"]), (dts[:4], list(fx["dts"][:4]))
    assert t == fx["t"]
    assert np.array_equal(U[inner].numpy(), fx["cons"]), refcases.rel_diff(U[inner].numpy(), fx["cons"])
    if "prims" in fx:
        assert np.array_equal(P[inner].numpy(), fx["prims"])


def test_numpy_standin_semantics():
    """The stand-in's JAX semantics that the fixtures rely on: functional
    updates, in-place operators that rebind instead of writing through views,
    integer powers by repeated squaring, None comparisons by identity."""
    import os
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    import jaxshim
    jnp = jaxshim._make_jnp()
    a = jnp.arange(6.0)
    view = a[1:4]
    b = a.at[2].set(9.0)
    assert a[2] == 2.0 and b[2] == 9.0
    view += 1.0
    assert a[1] == 1.0 and view[0] == 2.0
    x = jnp.asarray([1.1, 0.7, 3.3])
    xx = x * x
    assert np.array_equal(jnp.power(x, 6), xx * (xx * xx))
    assert (a != None) is True and (a == None) is False  # noqa: E711
