"""The CUDA path against golden vectors computed by the reference's own source
(tests/golden/ref, made by tests/golden/make_ref_fixtures.py: JAX-Fluids run
unmodified with a float64 numpy stand-in for jax).

Bounds: <= 1e-12 relative per right-hand side and <= 1e-10 after the steps
(max over the five variables of ||gpu - ref||_inf / ||ref||_inf); the kernels
follow the reference's operation order, so the results are also asserted
bitwise equal.  Both paths run through the C ABI of libgbfluids.so: the
drop-in path on halo buffers (SimulationManager: compute_rhs, stage
integration, primitives, halo fill, CFL time step) and the fused path
(FusedRK3: one launch sequence per RK stage on interior buffers), which starts
from the initial primitives as the reference's first stage does.
"""
import numpy as np
import pytest
import torch

from tests import refcases

pytestmark = pytest.mark.gpu

RHS_TOL = 1e-12
STEP_TOL = 1e-10
NAMES = refcases.names()


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from jaxfluids_gb300 import build
    build.build()


def _interior_prims5(fx, cc):
    """The five-component interior primitives the reference initialises:
    inactive velocities hold the buffer's fill value eps."""
    from jaxfluids_gb300.config import EPS
    p0 = refcases.prims0(fx)
    P = torch.full((5,) + cc.cells, EPS, dtype=torch.float64)
    ids = [0] + [1 + i for i in cc.active] + [4]
    for k, idx in enumerate(ids):
        P[idx] = p0[k].reshape(cc.cells)
    return P


@pytest.mark.parametrize("name", NAMES)
def test_dropin_matches_reference_source(name):
    from jaxfluids_gb300 import SimulationManager
    fx = refcases.load(name)
    _, cc = refcases.configs(fx)
    sim = SimulationManager(cc)
    U, P = sim.initialize(refcases.prims0(fx).cuda())
    rhs_buf, _, _ = sim.space_solver.compute_rhs(U, P, None, 0.0, 0.0)
    rhs = rhs_buf.euler_buffers.conservatives.cpu().numpy()
    assert refcases.rel_diff(rhs, fx["rhs0"]) <= RHS_TOL
    assert np.array_equal(rhs, fx["rhs0"])
    log = []
    U, P, t, steps = sim.simulate(U, P, end_step=fx["steps"], log=log)
    inner = cc.interior_slices()
    cons = U[inner].cpu().numpy()
    assert steps == fx["steps"]
    assert [row[1] for row in log] == list(fx["dts"])
    assert t == fx["t"]
    assert refcases.rel_diff(cons, fx["cons"]) <= STEP_TOL
    assert np.array_equal(cons, fx["cons"])
    if "prims" in fx:
        assert np.array_equal(P[inner].cpu().numpy(), fx["prims"])


@pytest.mark.parametrize("name", NAMES)
def test_fused_matches_reference_source(name):
    from jaxfluids_gb300 import FusedRK3
    from jaxfluids_gb300.solver import EquationManager
    fx = refcases.load(name)
    _, cc = refcases.configs(fx)
    f = FusedRK3(cc)
    P0 = _interior_prims5(fx, cc).cuda()
    U0 = EquationManager(cc).get_conservatives_from_primitives(P0)
    f.set_state(U0, prims=P0)
    dts = [float(f.dt)]
    for _ in range(fx["steps"]):
        f.advance(1)
        dts.append(float(f.dt))
    cons = f.cons.cpu().numpy()
    assert dts == list(fx["dts"])
    assert float(f.t) == fx["t"]
    assert refcases.rel_diff(cons, fx["cons"]) <= STEP_TOL
    assert np.array_equal(cons, fx["cons"])
