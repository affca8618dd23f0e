"""gbf_rk3_advance_noalloc: the RK3 entry point for callers that cannot allocate.

An XLA custom call, host code with a fixed device-memory budget, or a loop
that must not stall on cudaFree cannot give the library a workspace or let it
call cudaMalloc; this entry point keeps its workspace in a fixed array inside
the library instead.  The test drives it through the C ABI and checks that two
calls in a row give the same state and time step as the allocating entry point
(gbf_rk3_advance): within the parity tolerance of the other tests and, since
both run the same kernels on the same inputs, bitwise.  Cases: inviscid TGV,
Lax-Friedrichs, viscous CHAR-ROE, and a smaller grid after a larger one, so
that whatever an earlier call left in the shared array is shown not to be read.
It builds everything it needs itself, so it runs alone in a fresh process as
well as after the rest of the suite (this file is collected last).
"""
import ctypes
import math
import os
import re

import pytest
import torch

TOL = 1e-12  # relative, per variable: the right-hand-side parity tolerance
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FACES = ("east", "west", "north", "south", "top", "bottom")


def _rel(a, b):
    a = a.reshape(a.shape[0], -1)
    b = b.reshape(b.shape[0], -1)
    return max(((a[v] - b[v]).abs().max() / b[v].abs().max()).item() for v in range(a.shape[0]))


def _tgv_cons(n, device):
    gamma, ma = 1.4, 0.1
    x = (torch.arange(n, dtype=torch.float64, device=device) + 0.5) * (2 * math.pi / n)
    X, Y, Z = torch.meshgrid(x, x, x, indexing="ij")
    u = torch.sin(X) * torch.cos(Y) * torch.cos(Z)
    v = -torch.cos(X) * torch.sin(Y) * torch.cos(Z)
    p = 1.0 / (gamma * ma * ma) + (torch.cos(2 * X) + torch.cos(2 * Y)) * (torch.cos(2 * Z) + 2.0) / 16.0
    E = p / (gamma - 1.0) + 0.5 * (u * u + v * v)
    return torch.stack([torch.ones_like(X), u, v, torch.zeros_like(X), E]).contiguous()


def _cases():
    from jaxfluids_gb300.config import CaseConfig
    per = {f: "PERIODIC" for f in FACES}
    two_pi = ((0.0, 2 * math.pi),) * 3
    return [
        ("tgv-32", CaseConfig(cells=(32, 32, 32), ranges=two_pi, nh=3, bc=per)),
        ("tgv-24-lax-friedrichs", CaseConfig(cells=(24, 24, 24), ranges=two_pi, nh=3, bc=per,
                                             riemann="LAX-FRIEDRICHS")),
        ("tgv-20-char-roe-viscous", CaseConfig(cells=(20, 20, 20), ranges=two_pi, nh=4, bc=per,
                                               recon_var="CHAR-PRIMITIVE", frozen_state="ROE", viscous=True,
                                               heat=True, mu=1.0 / 1600, prandtl=0.71)),
        ("tgv-16", CaseConfig(cells=(16, 16, 16), ranges=two_pi, nh=3, bc=per)),  # smaller, after larger ones
    ]


@pytest.mark.gpu
def test_noalloc_matches_allocating_entry_point_on_two_calls():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from jaxfluids_gb300 import _lib, build
    build.build()
    lib = _lib.load()
    dev = torch.device("cuda", 0)
    P = ctypes.c_void_p
    s = P(torch.cuda.current_stream(dev).cuda_stream)
    for name, cfg in _cases():
        case = cfg.to_c()
        assert lib.gbf_rk3_workspace_bytes(ctypes.byref(case)) <= _lib.NOALLOC_SCRATCH_BYTES, name
        U0 = _tgv_cons(cfg.cells[0], dev)
        # allocating entry point, caller-owned workspace
        ua = U0.clone()
        da = torch.zeros(4, dtype=torch.float64, device=dev)
        ws = torch.empty(int(lib.gbf_rk3_workspace_bytes(ctypes.byref(case))) // 8, dtype=torch.float64,
                         device=dev)
        assert lib.gbf_rk3_init(ctypes.byref(case), P(ua.data_ptr()), None, P(da.data_ptr()), 0.0, s) == 0
        # allocation-free entry point
        ub = U0.clone()
        db = torch.zeros(4, dtype=torch.float64, device=dev)
        assert lib.gbf_rk3_init(ctypes.byref(case), P(ub.data_ptr()), None, P(db.data_ptr()), 0.0, s) == 0
        for steps in (3, 2):  # two calls in a row
            assert lib.gbf_rk3_advance(ctypes.byref(case), P(ua.data_ptr()), None, P(da.data_ptr()),
                                       P(ws.data_ptr()), steps, None, s) == 0
            assert lib.gbf_rk3_advance_noalloc(ctypes.byref(case), P(ub.data_ptr()), P(db.data_ptr()),
                                               steps, None, s) == 0
            torch.cuda.synchronize(dev)
            assert _rel(ub.cpu(), ua.cpu()) <= TOL, name
            assert abs(db[0].item() - da[0].item()) <= TOL * da[0].item(), name   # next dt
            assert abs(db[1].item() - da[1].item()) <= TOL * da[1].item(), name   # simulated time
            assert torch.equal(ub, ua), name
            assert torch.equal(db[:2], da[:2]), name
        assert not torch.equal(ua, U0), name  # the state did advance


def test_noalloc_rejects_cases_beyond_its_scratch():
    from jaxfluids_gb300 import _lib, build
    from jaxfluids_gb300.config import CaseConfig
    build.build()
    lib = _lib.load()
    n = 50  # 3-D periodic: 280 B per cell of workspace, 50^3 cells need 35 MB > 32 MiB
    cfg = CaseConfig(cells=(n, n, n), nh=3, bc={f: "PERIODIC" for f in FACES})
    case = cfg.to_c()
    assert lib.gbf_rk3_workspace_bytes(ctypes.byref(case)) > _lib.NOALLOC_SCRATCH_BYTES
    dummy = ctypes.c_void_p(256)  # never dereferenced: the size check comes first
    assert lib.gbf_rk3_advance_noalloc(ctypes.byref(case), dummy, dummy, 1, None, None) == _lib.GBF_ERR_SIZE
    small = CaseConfig(cells=(48, 48, 48), nh=3, bc={f: "PERIODIC" for f in FACES}).to_c()
    assert lib.gbf_rk3_workspace_bytes(ctypes.byref(small)) <= _lib.NOALLOC_SCRATCH_BYTES


def test_scratch_size_constant_matches_the_header():
    from jaxfluids_gb300 import _lib
    txt = open(os.path.join(ROOT, "include", "gbfluids.h")).read()
    m = re.search(r"#define GBF_NOALLOC_SCRATCH_BYTES (\d+)", txt)
    assert m and int(m.group(1)) == _lib.NOALLOC_SCRATCH_BYTES == 32 * 1024 * 1024
