"""The C-ABI library builds, loads and exports every declared symbol (no GPU needed)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from jaxfluids_gb300 import _lib, build
    build.build()
    return _lib.load()


def _declared():
    txt = open(os.path.join(ROOT, "include", "gbfluids.h")).read()
    return sorted(set(re.findall(r"^\s*(?:[A-Za-z_][\w\s\*]*?)\b(gbf_\w+)\s*\(", txt, re.M)))


def test_every_declared_symbol_is_exported(lib):
    from jaxfluids_gb300 import _lib
    declared = _declared()
    assert declared, "no declarations parsed"
    assert sorted(_lib.EXPORTS) == declared
    for name in declared:
        assert hasattr(lib, name), name


def test_version_and_status_strings(lib):
    from jaxfluids_gb300 import _lib
    assert lib.gbf_abi_version() == _lib.ABI_VERSION == 6
    assert lib.gbf_status_string(0) == b"ok"
    assert lib.gbf_status_string(-2) == b"unsupported setup"


def _cfg(**kw):
    from jaxfluids_gb300.config import CaseConfig
    base = dict(cells=(64, 1, 1), bc={f: "ZEROGRADIENT" for f in ("east", "west")})
    base.update(kw)
    return CaseConfig(**base)


def test_case_check_accepts_and_rejects(lib):
    c = _cfg().to_c()
    assert lib.gbf_case_check(ctypes.byref(c)) == 0
    c.recon_var = 1  # CHAR-PRIMITIVE is handled by a different kernel family
    assert lib.gbf_case_check(ctypes.byref(c)) in (0, -2)
    c = _cfg().to_c()
    c.nh = 2  # WENO5-Z needs three halo cells
    assert lib.gbf_case_check(ctypes.byref(c)) == -1
    c = _cfg().to_c()
    c.n[0] = 0
    assert lib.gbf_case_check(ctypes.byref(c)) == -4
    c = _cfg().to_c()
    c.riemann = 7
    assert lib.gbf_case_check(ctypes.byref(c)) == -2


def test_null_pointers_are_rejected_without_a_gpu(lib):
    c = _cfg().to_c()
    assert lib.gbf_rhs(ctypes.byref(c), None, None, None, None) == -1
    assert lib.gbf_halo_fill(ctypes.byref(c), None, None, None) == -1
    assert lib.gbf_rk3_advance(ctypes.byref(c), None, None, None, None, 1, None, None) == -1
    # U1, U2, two primitive buffers, the x faces (65 on a zero-gradient axis)
    # and the Lax-Friedrichs speed slots (4 doubles)
    assert lib.gbf_rk3_workspace_bytes(ctypes.byref(c)) == (4 * 5 * 64 + 5 * 65 + 4) * 8
    p = _cfg(bc={f: "PERIODIC" for f in ("east", "west")}).to_c()
    assert lib.gbf_rk3_workspace_bytes(ctypes.byref(p)) == (4 * 5 * 64 + 5 * 64 + 4) * 8


def test_config_from_reference_setup_dicts():
    from jaxfluids_gb300.config import CaseConfig, SetupError
    case = {
        "domain": {"x": {"cells": 100, "range": [0.0, 1.0]}, "y": {"cells": 1, "range": [0.0, 1.0]},
                   "z": {"cells": 1, "range": [0.0, 1.0]}},
        "boundary_conditions": {"east": {"type": "ZEROGRADIENT"}, "west": {"type": "ZEROGRADIENT"},
                                "north": {"type": "INACTIVE"}, "south": {"type": "INACTIVE"},
                                "top": {"type": "INACTIVE"}, "bottom": {"type": "INACTIVE"}},
        "material_properties": {"equation_of_state": {"model": "IdealGas", "specific_heat_ratio": 1.4,
                                                      "specific_gas_constant": 1.0}},
    }
    num = {"conservatives": {"halo_cells": 4, "time_integration": {"integrator": "RK3", "fixed_timestep": 1e-3},
                             "convective_fluxes": {"convective_solver": "GODUNOV", "godunov": {
                                 "riemann_solver": "RUSANOV", "signal_speed": "EINFELDT",
                                 "reconstruction_stencil": "MINMOD-AD", "reconstruction_variable": "PRIMITIVE"}}},
           "active_physics": {"is_convective_flux": True, "is_viscous_flux": False}}
    cfg = CaseConfig.from_setups(case, num)
    assert cfg.cells == (100, 1, 1) and cfg.nh == 4 and cfg.recon == "MINMOD-AD"
    assert cfg.riemann == "RUSANOV" and cfg.fixed_dt == 1e-3 and cfg.active == [0]
    bad = dict(num)
    bad["conservatives"] = dict(num["conservatives"], halo_cells=2)
    bad["conservatives"]["convective_fluxes"] = {"godunov": {"reconstruction_stencil": "WENO5-Z"}}
    with pytest.raises(SetupError):
        CaseConfig.from_setups(case, bad)
    with pytest.raises(NotImplementedError):
        CaseConfig.from_setups(case, {"conservatives": {"convective_fluxes": {"convective_solver": "FLUX-SPLITTING"}}})


def test_ctypes_mirror_matches_the_c_layout(tmp_path):
    """Every field of gbf_case / gbf_tile / gbf_batch_case sits at the offset
    the C compiler gives it (the ctypes mirror in _lib.py is hand-written)."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    from jaxfluids_gb300 import _lib
    from jaxfluids_gb300.batch import BATCH_CASE_DTYPE

    def ctypes_layout(ct):
        return ctypes.sizeof(ct), {f: getattr(ct, f).offset for f, _ in ct._fields_}
    layouts = {"gbf_case": ctypes_layout(_lib.GbfCase), "gbf_tile": ctypes_layout(_lib.GbfTile),
               "gbf_batch_case": (BATCH_CASE_DTYPE.itemsize,
                                  {f: BATCH_CASE_DTYPE.fields[f][1] for f in BATCH_CASE_DTYPE.names})}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "gbfluids.h"', "int main(void) {"]
    for cname, (_, offsets) in layouts.items():
        lines.append(f'  printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for fname in offsets:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    subprocess.run([cc, "-std=c99", "-I", inc, str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    for line in filter(None, out):
        cname, field, value = line.split()
        size, offsets = layouts[cname]
        assert int(value) == (size if field == "sizeof" else offsets[field]), (cname, field)
