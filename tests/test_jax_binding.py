"""The JAX-Fluids binding without jax and without a GPU.

* The case descriptor round-trips through its int64 packing (the XLA FFI
  attribute ``desc``) in Python, and through ``gbf_ffi_desc.h`` in C into the
  library's own case check (a small C program built here with the same unpack
  helper the FFI handlers use).
* ``case_config_from_reference`` reads, from the objects the reference's
  ``SpaceSolver`` constructor receives, the same descriptor that
  ``CaseConfig.from_setups`` reads from the setup dictionaries, for every golden
  setup; ``GB300SpaceSolver`` and the host-side ``SpaceSolver`` are constructed
  with the reference's constructor arguments (the reference runs under its
  numpy stand-in, in a subprocess).
* ``GB300SimulationManager`` reproduces the reference's own runs through the
  reference's loop and feed-forward (the oracle's step standing in for the
  fused GPU step).
* Every FFI target the Python side registers has a handler in ``gbf_ffi.cc``.
"""
import ctypes
import json
import os
import shutil
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FACES = ("east", "west", "north", "south", "top", "bottom")


def _cases():
    from jaxfluids_gb300.config import CaseConfig
    return [
        CaseConfig(cells=(200, 1, 1), bc={"east": "ZEROGRADIENT", "west": "ZEROGRADIENT"}),
        CaseConfig(cells=(24, 20, 1), nh=4, bc={"east": "NEUMANN", "west": "DIRICHLET", "north": "SYMMETRY",
                                                "south": "WALL"},
                   bc_values={"east": (0.0, 0.1, 0.0, 0.0, -0.2), "west": (1.2, 0.3, 0.05, 0.0, 1.1),
                              "south": (0.2, 0.0, 0.0)}, viscous=True, heat=True, mu=5e-3, kappa=4e-3),
        CaseConfig(cells=(16, 12, 10), nh=4, bc={f: "PERIODIC" for f in FACES}, recon_var="CHAR-PRIMITIVE",
                   frozen_state="ROE", riemann="RUSANOV", cfl=0.4, gravity=(0.0, -1.0, 0.0)),
    ]


def test_descriptor_round_trips_in_python():
    from jaxfluids_gb300 import jax_binding
    for cfg in _cases():
        c = cfg.to_c()
        words = jax_binding.pack_case(c)
        assert words.dtype == np.int64 and words.nbytes == ctypes.sizeof(c)
        assert bytes(jax_binding.unpack_case(words)) == bytes(c)
    with pytest.raises(ValueError):
        jax_binding.unpack_case(words[:-1])


HARNESS = r"""
#include <dlfcn.h>
#include <stdio.h>
#include "gbf_ffi_desc.h"
int main(int argc, char** argv) {
  int64_t words[GBF_DESC_WORDS + 1];
  size_t n = 0;
  long long w;
  while (n < GBF_DESC_WORDS + 1 && scanf("%lld", &w) == 1) words[n++] = (int64_t)w;
  gbf_case c;
  int st = gbf_case_from_words(words, n, &c);
  if (st != GBF_OK) { printf("unpack %d\n", st); return 0; }
  void* h = dlopen(argv[1], RTLD_NOW);
  if (!h) { printf("dlopen failed\n"); return 1; }
  int (*check)(const gbf_case*) = (int (*)(const gbf_case*))dlsym(h, "gbf_case_check");
  printf("check %d n %d %d %d nh %d recon %d riemann %d flags %u dx0 %.17g gamma %.17g cfl %.17g\n", check(&c),
         c.n[0], c.n[1], c.n[2], c.nh, c.recon, c.riemann, c.flags, c.dx[0], c.gamma, c.cfl);
  return 0;
}
"""


def test_descriptor_unpacks_in_c_into_the_library(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    from jaxfluids_gb300 import _lib, build, jax_binding
    build.build()
    src = tmp_path / "unpack.c"
    src.write_text(HARNESS)
    exe = tmp_path / "unpack"
    subprocess.run([cc, "-std=c99", "-I", os.path.join(ROOT, "include"), "-I",
                    os.path.join(ROOT, "jaxfluids_gb300", "ffi"), str(src), "-o", str(exe), "-ldl"], check=True)
    lib = _lib.load()
    for cfg in _cases():
        c = cfg.to_c()
        words = jax_binding.pack_case(c)
        out = subprocess.run([str(exe), _lib.LIB_PATH], input=" ".join(str(int(x)) for x in words),
                             capture_output=True, text=True, check=True).stdout.split()
        assert out[0] == "check" and int(out[1]) == lib.gbf_case_check(ctypes.byref(c))
        vals = dict(zip(out[2::2], out[3::2]))
        assert int(out[3]) == c.n[0] and int(vals["nh"]) == c.nh and int(vals["recon"]) == c.recon
        assert int(vals["riemann"]) == c.riemann and int(vals["flags"]) == c.flags
        assert float(vals["dx0"]) == c.dx[0] and float(vals["gamma"]) == c.gamma and float(vals["cfl"]) == c.cfl
    # a descriptor one word short is refused
    short = " ".join(str(int(x)) for x in jax_binding.pack_case(_cases()[0].to_c())[:-1])
    out = subprocess.run([str(exe), _lib.LIB_PATH], input=short, capture_output=True, text=True,
                         check=True).stdout.split()
    assert out == ["unpack", str(_lib.GBF_ERR_INVALID_ARGUMENT)]


def test_descriptor_from_the_reference_objects_equals_the_one_from_the_setups():
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import make_ref_fixtures
    if not os.path.isdir(os.path.join(make_ref_fixtures.REFERENCE, "src", "jaxfluids")):
        pytest.skip("the reference checkout is not available on this machine")
    r = subprocess.run([sys.executable, "-B", os.path.join(ROOT, "tests", "reference_binding_check.py")],
                       capture_output=True, text=True, timeout=900, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    from tests import refcases
    assert sorted(res) == refcases.names()
    for name, v in res.items():
        assert v["desc_equal"] and v["solver_desc_equal"] and v["is_subclass"], (name, v)
        assert v["host_desc_equal"], (name, v)


def test_simulation_manager_subclass_reproduces_the_references_own_runs():
    """GB300SimulationManager (the reference's SimulationManager with each RK3
    step one fused call) driven through the reference's integration-step loop
    and _feed_forward, the oracle's step standing in for the GPU's: bitwise the
    reference's own conservatives, time steps and times (golden fixtures), and
    its stock feed-forward trajectory."""
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import make_ref_fixtures
    if not os.path.isdir(os.path.join(make_ref_fixtures.REFERENCE, "src", "jaxfluids")):
        pytest.skip("the reference checkout is not available on this machine")
    r = subprocess.run([sys.executable, "-B", os.path.join(ROOT, "tests", "reference_simulation_check.py")],
                       capture_output=True, text=True, timeout=1800, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    ff = res.pop("feed_forward")
    assert ff["prims_equal"] and ff["times_equal"], ff
    assert len(res) >= 10
    for name, v in res.items():
        assert v["subclass"] and v["space_solver"] == "GB300SpaceSolver", (name, v)
        assert v["cons_equal"] and v["dts_equal"] and v["t_equal"] and v["steps"] == v["steps_ref"], (name, v)


def test_every_registered_target_has_a_handler():
    from jaxfluids_gb300 import jax_binding
    src = open(os.path.join(ROOT, "jaxfluids_gb300", "ffi", "gbf_ffi.cc")).read()
    for name in jax_binding.FFI_TARGETS:
        assert f"XLA_FFI_DEFINE_HANDLER_SYMBOL({name}_ffi," in src, name
