"""Run by tests/test_jax_binding.py in a subprocess (it installs a numpy
stand-in for jax into sys.modules, which must not leak into the test process):
drive GB300SimulationManager, the reference's SimulationManager with each RK3
step one fused call, through the reference's own integration-step loop and
feed-forward, with the oracle's step on interior conservatives standing in for
the fused GPU step (this checks the subclass's plumbing: buffer slices, halos,
primitives, time and step bookkeeping; the kernels are checked against the
oracle elsewhere).  Compares with the reference's own results (the golden
fixtures, and its stock feed-forward run).  Prints one JSON object."""
import sys

sys.dont_write_bytecode = True  # noqa: E402

import contextlib
import io
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_ref_fixtures  # noqa: E402

from tests import refcases  # noqa: E402

CASES = ("sod", "tgv24-visc-char-roe", "quad64", "cavity32-visc-heat", "channel-bc-visc-heat",
         "box3d-mixed-char-roe-visc", "q2-lax-friedrichs", "q2-char-conservative", "q2-conservative",
         "q2-symmetry-periodic", "q2-teno5")


def oracle_step(fx):
    """step(cons, prims, dt, t) of the oracle on interior conservatives and
    the first stage's interior primitives (halos by the boundary rules at t)."""
    import torch
    from oracle import jf_oracle as O
    oc, _ = refcases.configs(fx)

    def step(cons, prims, dt, t):
        Ui = torch.from_numpy(np.array(cons, dtype=np.float64))
        U, P = O.buffers_from_interior_cons(Ui, oc)
        P = P.clone()
        P[oc.interior()] = torch.from_numpy(np.array(prims, dtype=np.float64))
        P, U = O.halo_update(P, U, oc, float(t))
        U, P = O.rk3_step(U, P, torch.tensor(float(dt), dtype=torch.float64), oc, float(t))
        return np.asarray(U[oc.interior()].numpy())
    return step


def main():
    jf, ml = make_ref_fixtures.load_reference()
    from jaxfluids_gb300 import jax_binding
    cls = jax_binding.simulation_manager_class()
    out = {}
    names = [n for n in CASES if n in refcases.names()]
    for name in names:
        fx = refcases.load(name)
        with contextlib.redirect_stdout(io.StringIO()):
            im = jf.InputManager(fx["case_setup"], fx["numerical_setup"])
            init = jf.InitializationManager(im)
            sim = cls(im, step=oracle_step(fx))
            buf = init.initialization(user_prime_init=np.ascontiguousarray(fx["prims0"]))
        tcv = buf.time_control_variables
        dts = [float(tcv.physical_timestep_size)]
        for _ in range(int(fx["steps"])):
            cfp = sim.compute_control_flow_params(tcv, buf.step_information)
            buf, _ = sim.do_integration_step(buf, cfp, ml.ParametersSetup(), ml.CallablesSetup())
            tcv = buf.time_control_variables
            dts.append(float(tcv.physical_timestep_size))
        nhx, nhy, nhz = sim.domain_information.domain_slices_conservatives
        cons = np.asarray(buf.simulation_buffers.material_fields.conservatives)[..., nhx, nhy, nhz]
        out[name] = {
            "subclass": isinstance(sim, jf.SimulationManager) and type(sim).__name__ == "GB300SimulationManager",
            "space_solver": type(sim.space_solver).__name__,
            "cons_equal": bool(np.array_equal(cons, fx["cons"])),
            "dts_equal": bool(np.array_equal(np.array(dts), fx["dts"])),
            "t_equal": float(tcv.physical_simulation_time) == float(fx["t"]),
            "steps": int(tcv.simulation_step), "steps_ref": int(fx["steps"]),
        }
    # feed-forward: the reference's _feed_forward (lax.scan + jax.checkpoint of
    # its _do_integration_step) on the subclass against the stock manager
    from jaxfluids.feed_forward.data_types import FeedForwardSetup
    fx = refcases.load("tgv24-visc-char-roe")
    setup = FeedForwardSetup(outer_steps=3, inner_steps=2, is_checkpoint_inner_step=True)
    res = {}
    for kind in ("stock", "gb300"):
        with contextlib.redirect_stdout(io.StringIO()):
            im = jf.InputManager(fx["case_setup"], fx["numerical_setup"])
            sim = jf.SimulationManager(im) if kind == "stock" else cls(im, step=oracle_step(fx))
            sol, times = sim._feed_forward(np.ascontiguousarray(fx["prims0"]), float(fx["dts"][0]), 0.0, setup)
        res[kind] = (np.asarray(sol["primitives"]), np.asarray(times))
    out["feed_forward"] = {
        "prims_equal": bool(np.array_equal(res["stock"][0], res["gb300"][0])),
        "times_equal": bool(np.array_equal(res["stock"][1], res["gb300"][1])),
        "shape": list(res["gb300"][0].shape),
    }
    print(json.dumps(out))


if __name__ == "__main__":
    main()
