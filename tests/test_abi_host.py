"""Host-side entry points of the C ABI that need no GPU: the per-thread last
status, the batch work-list builder (against the Python builder), and
argument validation of the stage entry points (which returns before any
CUDA call)."""
import ctypes

import numpy as np
import pytest

from jaxfluids_gb300 import _lib
from jaxfluids_gb300.batch import BATCH_CASE_DTYPE, build_worklist
from jaxfluids_gb300.config import CaseConfig


@pytest.fixture(scope="module")
def lib():
    from jaxfluids_gb300 import build
    build.build()
    return _lib.load()


def _case(**kw):
    base = dict(cells=(32, 24, 1), bc={f: "ZEROGRADIENT" for f in ("east", "west", "north", "south")})
    base.update(kw)
    return CaseConfig(**base).to_c()


def test_last_status_follows_the_latest_call(lib):
    bad = _case()
    bad.nh = 1
    assert lib.gbf_case_check(ctypes.byref(bad)) == _lib.GBF_ERR_INVALID_ARGUMENT
    assert lib.gbf_last_status() == _lib.GBF_ERR_INVALID_ARGUMENT
    good = _case()
    assert lib.gbf_case_check(ctypes.byref(good)) == _lib.GBF_OK
    assert lib.gbf_last_status() == _lib.GBF_OK


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_batch_worklist_matches_python_builder(lib, seed):
    rng = np.random.default_rng(seed)
    ncases = int(rng.integers(1, 40))
    cells = np.stack([rng.choice([64, 96, 128, 192, 256], size=ncases), rng.choice([32, 64, 160], size=ncases),
                      np.ones(ncases, dtype=np.int64)], axis=1).astype(np.int32)
    dx = rng.uniform(0.001, 0.1, size=(ncases, 3))
    tile = (15, 32, 1)
    n, tiles, offsets, worklist, total = build_worklist([tuple(c) for c in cells], tile)
    gt = _lib.GbfTile()
    gt.t[0], gt.t[1], gt.t[2] = tile
    table = np.zeros(ncases, dtype=BATCH_CASE_DTYPE)
    nitems, tot = ctypes.c_int64(), ctypes.c_int64()
    cells_c = np.ascontiguousarray(cells)
    dx_c = np.ascontiguousarray(dx)
    # size query first
    st = lib.gbf_batch_worklist(cells_c.ctypes.data, dx_c.ctypes.data, ncases, ctypes.byref(gt),
                                table.ctypes.data, None, 0, ctypes.byref(nitems), ctypes.byref(tot))
    assert st == _lib.GBF_ERR_SIZE and nitems.value == worklist.shape[0] and tot.value == total
    wl = np.zeros((nitems.value, 2), dtype=np.int32)
    st = lib.gbf_batch_worklist(cells_c.ctypes.data, dx_c.ctypes.data, ncases, ctypes.byref(gt),
                                table.ctypes.data, wl.ctypes.data, nitems.value, ctypes.byref(nitems),
                                ctypes.byref(tot))
    assert st == _lib.GBF_OK
    assert np.array_equal(wl, worklist)
    assert np.array_equal(table["n"], n) and np.array_equal(table["tiles"], tiles)
    assert np.array_equal(table["offset"], offsets) and np.array_equal(table["dx"], dx)


def test_stage_entry_points_validate_before_any_device_call(lib):
    c = _case()
    buf = ctypes.c_void_p(8)  # never dereferenced: validation fails first
    # stage out of range, aliasing output, stage 0 with distinct states
    assert lib.gbf_rk3_stage(ctypes.byref(c), 3, buf, buf, ctypes.c_void_p(16), buf, None, None, None) \
        == _lib.GBF_ERR_INVALID_ARGUMENT
    assert lib.gbf_rk3_stage(ctypes.byref(c), 1, buf, buf, buf, buf, None, None, None) \
        == _lib.GBF_ERR_INVALID_ARGUMENT
    assert lib.gbf_rk3_stage(ctypes.byref(c), 0, buf, ctypes.c_void_p(24), ctypes.c_void_p(16), buf, None, None,
                             None) == _lib.GBF_ERR_INVALID_ARGUMENT
    assert lib.gbf_last_status() == _lib.GBF_ERR_INVALID_ARGUMENT
    # the stage VJP validates its stage index before any device call
    hll = _case(riemann="HLL", signal_speed="DAVIS")
    assert lib.gbf_rk3_stage_vjp(ctypes.byref(hll), 3, buf, buf, buf, ctypes.c_void_p(16), ctypes.c_void_p(24),
                                 buf, None, None) == _lib.GBF_ERR_INVALID_ARGUMENT
    # a solver handle needs a valid case
    bad = _case()
    bad.nh = 1
    out = ctypes.c_void_p()
    assert lib.gbf_create(ctypes.byref(bad), None, ctypes.byref(out)) == _lib.GBF_ERR_INVALID_ARGUMENT
    assert out.value is None
    assert lib.gbf_destroy(None) == _lib.GBF_OK


@pytest.mark.parametrize("kw,has_adjoint", [
    (dict(), True),
    (dict(recon="TENO5"), True),
    (dict(riemann="LAX-FRIEDRICHS"), True),
    (dict(riemann="LAX-FRIEDRICHS", recon="MINMOD-AD", nh=4), True),
    (dict(recon="MINMOD", nh=4), True),
    (dict(riemann="LAX-FRIEDRICHS", recon="MINMOD", nh=4), True),
    (dict(signal_speed="DAVIS"), True),
    (dict(signal_speed="ARITHMETIC"), True),
    (dict(signal_speed="RUSANOV"), True),
    (dict(signal_speed="TORO"), True),
    (dict(riemann="HLL", signal_speed="TORO"), True),
    (dict(riemann="LAX-FRIEDRICHS", recon_var="CHAR-PRIMITIVE"), True),
    (dict(riemann="LAX-FRIEDRICHS", recon_var="CONSERVATIVE"), True),
    (dict(riemann="LAX-FRIEDRICHS", recon_var="CHAR-CONSERVATIVE"), True),
    (dict(recon_var="CONSERVATIVE"), True),
    (dict(recon_var="CONSERVATIVE", interpolation_limiter=True), True),
    (dict(recon_var="CHAR-CONSERVATIVE", frozen_state="ROE"), True),
    (dict(recon_var="CHAR-CONSERVATIVE", interpolation_limiter=True), True),
    (dict(recon_var="CHAR-PRIMITIVE", interpolation_limiter=True), True),
    (dict(interpolation_limiter=True), True),
    (dict(nh=4, viscous=True, mu=0.01, convective=False), True),
])
def test_adjoint_coverage_is_reported_without_a_device(lib, kw, has_adjoint):
    """Every valid setup has an adjoint: gbf_vjp_workspace_bytes is non-zero
    for each (and 0 only for an invalid case)."""
    c = _case(**kw)
    assert lib.gbf_case_check(ctypes.byref(c)) == _lib.GBF_OK
    assert (lib.gbf_vjp_workspace_bytes(ctypes.byref(c)) > 0) == has_adjoint


def test_conservative_reconstructions_need_the_conservatives(lib):
    c = _case(recon_var="CONSERVATIVE")
    buf = ctypes.c_void_p(8)
    assert lib.gbf_rhs_cons(ctypes.byref(c), buf, None, buf, None, None) == _lib.GBF_ERR_INVALID_ARGUMENT
    assert lib.gbf_rhs_cons(ctypes.byref(c), buf, ctypes.c_void_p(12), buf, None, None) == _lib.GBF_ERR_ALIGNMENT
    # the characteristic and conservative variables are built with WENO5-Z only
    bad = _case(recon_var="CONSERVATIVE")
    bad.recon = _lib.RECON["WENO5-JS"]
    assert lib.gbf_case_check(ctypes.byref(bad)) == _lib.GBF_ERR_UNSUPPORTED
    # gravity: the drop-in volume force validates before any device call
    g = _case(gravity=(0.0, -1.0, 0.0))
    assert lib.gbf_volume_force(ctypes.byref(g), None, buf, None) == _lib.GBF_ERR_INVALID_ARGUMENT


def test_rhs_workspace_holds_the_face_buffers(lib):
    """gbf_rhs_ws: the workspace holds the face buffers of the reference's face
    arrays (N + 1 faces per line on every active axis, periodic ones too) and
    the Lax-Friedrichs speed slots; 0 bytes for an invalid case; a missing or
    misaligned workspace is refused before any device call."""
    for kw in ({}, {"riemann": "LAX-FRIEDRICHS"}, {"bc": {f: "PERIODIC" for f in ("east", "west", "north", "south")}}):
        c = _case(**kw)
        assert lib.gbf_rhs_workspace_bytes(ctypes.byref(c)) == (5 * (33 * 24 + 32 * 25) + 4) * 8
    bad = _case(riemann="LAX-FRIEDRICHS")
    bad.nh = 1
    assert lib.gbf_rhs_workspace_bytes(ctypes.byref(bad)) == 0
    lf = _case(riemann="LAX-FRIEDRICHS")
    buf = ctypes.c_void_p(8)
    assert lib.gbf_rhs_ws(ctypes.byref(lf), buf, None, buf, None, None, None) == _lib.GBF_ERR_INVALID_ARGUMENT
    assert lib.gbf_rhs_ws(ctypes.byref(lf), buf, None, buf, None, ctypes.c_void_p(12), None) == \
        _lib.GBF_ERR_ALIGNMENT
    # the conservative reconstructions still need the conservatives
    cv = _case(recon_var="CONSERVATIVE")
    assert lib.gbf_rhs_ws(ctypes.byref(cv), buf, None, buf, None, buf, None) == _lib.GBF_ERR_INVALID_ARGUMENT
