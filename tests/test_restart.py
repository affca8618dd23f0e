"""Output and restart in the reference's field layout (restart.py).

CPU: the archive holds the reference's dataset names and orientations
(``buffer.T``), round-trips, and is read back by the reference's own restart
loader (``initialization/helper_functions.py`` ``load_buffer``, run under the
numpy stand-in in a subprocess).  GPU: a fused run written, restarted and
continued equals the oracle restarted from the same primitives, bitwise."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _cfg():
    from jaxfluids_gb300.config import CaseConfig
    return CaseConfig(cells=(12, 10, 8), ranges=((0.0, 1.0), (0.0, 2.0), (-1.0, 1.0)), nh=3,
                      bc={f: "PERIODIC" for f in ("east", "west", "north", "south", "top", "bottom")})


def test_fields_round_trip_in_the_reference_layout(tmp_path):
    from jaxfluids_gb300.restart import read_fields, write_fields
    cfg = _cfg()
    P = np.random.default_rng(3).uniform(0.5, 2.0, (5,) + cfg.cells)
    path = write_fields(str(tmp_path / "out"), cfg, P, 0.125)
    with np.load(path) as z:
        assert z["primitives/density"].shape == (8, 10, 12)
        assert z["primitives/velocity"].shape == (8, 10, 12, 3)
        assert np.array_equal(z["primitives/velocity"][2, 3, 4], P[1:4, 4, 3, 2])
        assert np.array_equal(z["domain/gridY"], cfg.cell_centers(1)) and float(z["time"]) == 0.125
    Q, t = read_fields(path, cfg)
    assert np.array_equal(Q, P) and t == 0.125


def test_the_reference_loader_reads_the_fields(tmp_path):
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import make_ref_fixtures
    if not os.path.isdir(os.path.join(make_ref_fixtures.REFERENCE, "src", "jaxfluids")):
        pytest.skip("the reference checkout is not available on this machine")
    from jaxfluids_gb300.restart import write_fields
    cfg = _cfg()
    P = np.random.default_rng(4).uniform(0.5, 2.0, (5,) + cfg.cells)
    path = write_fields(str(tmp_path / "out"), cfg, P, 0.25)
    code = (
        "import sys; sys.dont_write_bytecode = True; sys.path.insert(0, %r);"
        "import make_ref_fixtures, json, numpy as np; make_ref_fixtures.load_reference();"
        "from jaxfluids.initialization.helper_functions import load_buffer;"
        "z = dict(np.load(%r));"
        "rho = load_buffer('primitives/density', (z,)); vel = load_buffer('primitives/velocity', (z,), True);"
        "p = load_buffer('primitives/pressure', (z,));"
        "np.save(%r, np.concatenate([rho[None], vel, p[None]]))"
    ) % (os.path.join(ROOT, "tests", "golden"), path, str(tmp_path / "loaded.npy"))
    r = subprocess.run([sys.executable, "-B", "-c", code], capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    assert np.array_equal(np.load(tmp_path / "loaded.npy"), P)


@pytest.mark.gpu
def test_restarted_fused_run_continues_like_the_oracle(tmp_path):
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    import math
    from jaxfluids_gb300 import FusedRK3, build
    from oracle import jf_oracle as O
    from tests.cases import both, rel_err, tgv_prims
    build.build()
    oc, cc = both((24, 20, 16), "PERIODIC", ranges=((0, 2 * math.pi),) * 3)
    U, P = O.initialize(tgv_prims(24)[:, :24, :20, :16].contiguous(), oc)
    inner = oc.interior()
    f = FusedRK3(cc)
    f.set_state(U[inner].contiguous().cuda(), prims=P[inner].contiguous().cuda())
    f.advance(3)
    path = f.write(str(tmp_path / "state"))
    g = FusedRK3.from_restart(cc, path)
    assert float(g.t) == float(f.t)
    g.advance(2)
    # the oracle restarted from the written primitives (create_material_fields)
    from jaxfluids_gb300.restart import read_fields
    Pr, t = read_fields(path, cc)
    Ur, Pb = O.initialize(torch.from_numpy(Pr), oc)
    dt = O.compute_dt(Pb, oc)
    for _ in range(2):
        Ur, Pb = O.rk3_step(Ur, Pb, dt, oc)
        dt = O.compute_dt(Pb, oc)
    got = g.cons.cpu()
    assert rel_err(got, Ur[inner]) <= 1e-10
    assert torch.equal(got, Ur[inner])
    assert float(g.dt) == float(dt)
