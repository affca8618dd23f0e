"""Run by tests/test_jax_binding.py in a subprocess (it installs a numpy
stand-in for jax into sys.modules, which must not leak into the test process):
for every golden setup, build the reference's own SimulationManager from the
setup dictionaries and compare the GB300 case descriptor read from the objects
the reference's SpaceSolver was constructed with against the one read from the
dictionaries; also construct GB300SpaceSolver with the reference's
constructor arguments.  Prints one JSON object."""
import sys

sys.dont_write_bytecode = True  # noqa: E402

import contextlib
import io
import json
import os

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_ref_fixtures  # noqa: E402

from tests import refcases  # noqa: E402


def main():
    jf, ml = make_ref_fixtures.load_reference()
    from jaxfluids_gb300 import jax_binding
    from jaxfluids_gb300.config import CaseConfig
    from jaxfluids_gb300.solver import SpaceSolver as HostSpaceSolver
    out = {}
    cls = jax_binding.space_solver_class()
    for name in refcases.names():
        fx = refcases.load(name)
        with contextlib.redirect_stdout(io.StringIO()):
            im = jf.InputManager(fx["case_setup"], fx["numerical_setup"])
            sim = jf.SimulationManager(im)
        ss = sim.space_solver
        ref = jax_binding.case_config_from_reference(ss.domain_information, ss.material_manager,
                                                     ss.numerical_setup, ss.halo_manager, ss.gravity)
        mine = CaseConfig.from_setups(fx["case_setup"], fx["numerical_setup"])
        # the host-side SpaceSolver with the reference's constructor arguments
        host = HostSpaceSolver(ss.domain_information, ss.material_manager, ss.equation_manager, ss.halo_manager,
                               ss.numerical_setup, ss.gravity, None)
        with contextlib.redirect_stdout(io.StringIO()):
            gb = jax_binding.install_space_solver(sim)
        out[name] = {
            "desc_equal": bytes(ref.to_c()) == bytes(mine.to_c()),
            "solver_desc_equal": bytes(gb.gb300_desc.tobytes()) == bytes(mine.to_c()),
            "is_subclass": isinstance(gb, type(ss)) and type(gb).__name__ == "GB300SpaceSolver",
            "host_desc_equal": bytes(host.case) == bytes(mine.to_c()),
            "recon": ref.recon, "riemann": ref.riemann, "bc": {f: str(v) for f, v in ref.bc.items()},
        }
    print(json.dumps(out))


if __name__ == "__main__":
    main()
