"""ctypes binding of libgbfluids.so (declarations in include/gbfluids.h).

The library is the only compute path: if it is missing or cannot be loaded
every call raises; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libgbfluids.so")

GBF_OK = 0
GBF_ERR_INVALID_ARGUMENT = -1
GBF_ERR_UNSUPPORTED = -2
GBF_ERR_CUDA = -3
GBF_ERR_SIZE = -4
GBF_ERR_ALIGNMENT = -5
STATUS = {0: "ok", -1: "invalid argument", -2: "unsupported setup", -3: "CUDA launch error",
          -4: "invalid or unsupported size", -5: "misaligned pointer"}

RECON = {"WENO5-Z": 0, "MINMOD": 1, "MINMOD-AD": 2, "WENO5-JS": 3, "WENO3-JS": 4, "WENO3-Z": 5, "TENO5": 6}
RECVAR = {"PRIMITIVE": 0, "CHAR-PRIMITIVE": 1, "CONSERVATIVE": 2, "CHAR-CONSERVATIVE": 3}
FROZEN = {"ARITHMETIC": 0, "ROE": 1}
RIEMANN = {"LAX-FRIEDRICHS": 3, "HLLC": 0, "RUSANOV": 1, "HLL": 2}
SIGNAL = {"EINFELDT": 0, "DAVIS": 1, "ARITHMETIC": 2, "RUSANOV": 3, "TORO": 4}
ABI_VERSION = 6  # GBF_ABI_VERSION of include/gbfluids.h (gbf_case layout)
CENTRAL = {"CENTRAL4": 0, "CENTRAL2": 1}
BC = {"PERIODIC": 0, "ZEROGRADIENT": 1, "SYMMETRY": 2, "WALL": 3, "DIRICHLET": 4, "NEUMANN": 5}
BC_MIXED = 6  # a face of several types, per-cell types in bc_field_types
FACE_ORDER = ("west", "east", "south", "north", "bottom", "top")
FLAG_VISCOUS, FLAG_HEAT, FLAG_VISCOUS_HEAT_PRODUCTION, FLAG_NO_CONVECTIVE = 1, 2, 4, 8
FLAG_INTERPOLATION_LIMITER, FLAG_LIMIT_VELOCITY, FLAG_GRAVITY = 16, 32, 64

# every symbol include/gbfluids.h declares
EXPORTS = (
    "gbf_abi_version", "gbf_last_status", "gbf_status_string", "gbf_case_check", "gbf_rhs", "gbf_rhs_cons",
    "gbf_rhs_workspace_bytes", "gbf_rhs_ws", "gbf_halo_fill", "gbf_volume_force",
    "gbf_prims_from_cons", "gbf_cons_from_prims", "gbf_stage_integrate",
    "gbf_dt_workspace_bytes", "gbf_dt", "gbf_rk3_workspace_bytes", "gbf_rk3_init",
    "gbf_rk3_advance", "gbf_rk3_advance_noalloc",
    "gbf_batch_workspace_bytes", "gbf_batch_init", "gbf_batch_advance",
    "gbf_vjp_workspace_bytes", "gbf_rhs_vjp", "gbf_rk3_step_vjp", "gbf_rk3_step_vjp_stages",
    "gbf_rk3_stage", "gbf_rk3_stage_vjp", "gbf_batch_worklist", "gbf_state_check",
    "gbf_create", "gbf_destroy", "gbf_solver_init", "gbf_solver_advance", "gbf_solver_time",
)

# bytes of the allocation-free entry point's built-in scratch
# (GBF_NOALLOC_SCRATCH_BYTES): cases whose gbf_rk3_workspace_bytes fit run there
NOALLOC_SCRATCH_BYTES = 33554432


class GbfCase(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_int32 * 3),
        ("nh", ctypes.c_int32),
        ("recon", ctypes.c_int32),
        ("recon_var", ctypes.c_int32),
        ("frozen_state", ctypes.c_int32),
        ("riemann", ctypes.c_int32),
        ("signal_speed", ctypes.c_int32),
        ("bc", ctypes.c_int32 * 6),
        ("flags", ctypes.c_uint32),
        ("dx", ctypes.c_double * 3),
        ("gamma", ctypes.c_double),
        ("R", ctypes.c_double),
        ("mu", ctypes.c_double),
        ("bulk_mu", ctypes.c_double),
        ("kappa", ctypes.c_double),
        ("cfl", ctypes.c_double),
        ("fixed_dt", ctypes.c_double),
        ("eps", ctypes.c_double),
        ("stencil_eps", ctypes.c_double),
        ("bc_value", (ctypes.c_double * 5) * 6),
        ("dissipative_stencil", ctypes.c_int32 * 3),
        ("reserved", ctypes.c_int32),
        ("bc_field_values", ctypes.c_void_p * 6),
        ("bc_field_types", ctypes.c_void_p * 6),
        ("gravity", ctypes.c_double * 3),
    ]


class GbfTile(ctypes.Structure):
    _fields_ = [("t", ctypes.c_int32 * 3), ("threads", ctypes.c_int32)]


class GbfError(RuntimeError):
    pass


_lib: Optional[ctypes.CDLL] = None


def load() -> ctypes.CDLL:
    """Load the library once; raise if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise GbfError(f"{LIB_PATH} is missing: build it with jaxfluids_gb300.build.build()")
    lib = ctypes.CDLL(LIB_PATH)
    P = ctypes.c_void_p
    I = ctypes.c_int
    C = ctypes.POINTER(GbfCase)
    T = ctypes.POINTER(GbfTile)
    sig = {
        "gbf_abi_version": (I, []),
        "gbf_last_status": (I, []),
        "gbf_status_string": (ctypes.c_char_p, [I]),
        "gbf_case_check": (I, [C]),
        "gbf_rhs": (I, [C, P, P, T, P]),
        "gbf_rhs_cons": (I, [C, P, P, P, T, P]),
        "gbf_rhs_workspace_bytes": (ctypes.c_size_t, [C]),
        "gbf_rhs_ws": (I, [C, P, P, P, T, P, P]),
        "gbf_halo_fill": (I, [C, P, P, P]),
        "gbf_volume_force": (I, [C, P, P, P]),
        "gbf_prims_from_cons": (I, [C, P, P, ctypes.c_int64, P]),
        "gbf_cons_from_prims": (I, [C, P, P, ctypes.c_int64, P]),
        "gbf_stage_integrate": (I, [C, P, P, P, P, I, P]),
        "gbf_dt_workspace_bytes": (ctypes.c_size_t, []),
        "gbf_dt": (I, [C, P, P, P, P]),
        "gbf_rk3_workspace_bytes": (ctypes.c_size_t, [C]),
        "gbf_rk3_init": (I, [C, P, P, P, ctypes.c_double, P]),
        "gbf_rk3_advance": (I, [C, P, P, P, P, I, T, P]),
        "gbf_rk3_advance_noalloc": (I, [C, P, P, I, T, P]),
        "gbf_batch_workspace_bytes": (ctypes.c_size_t, [ctypes.c_int64]),
        "gbf_vjp_workspace_bytes": (ctypes.c_size_t, [C]),
        "gbf_rhs_vjp": (I, [C, P, P, P, P, T, P]),
        "gbf_rk3_step_vjp": (I, [C, P, P, P, P, P, T, P]),
        "gbf_rk3_step_vjp_stages": (I, [C, P, P, P, P, P, P, P, T, P]),
        "gbf_batch_init": (I, [C, P, I, P, I, T, P, P, ctypes.c_double, P]),
        "gbf_batch_advance": (I, [C, P, I, P, I, T, I, P, P, P, ctypes.c_int64, I, P]),
        "gbf_rk3_stage": (I, [C, I, P, P, P, P, P, T, P]),
        "gbf_state_check": (I, [C, P, P, P]),
        "gbf_rk3_stage_vjp": (I, [C, I, P, P, P, P, P, P, T, P]),
        "gbf_batch_worklist": (I, [P, P, I, T, P, P, ctypes.c_int64, P, P]),
        "gbf_create": (I, [C, T, ctypes.POINTER(ctypes.c_void_p)]),
        "gbf_destroy": (I, [P]),
        "gbf_solver_init": (I, [P, P, ctypes.c_double, P]),
        "gbf_solver_advance": (I, [P, P, I, P]),
        "gbf_solver_time": (I, [P, P, P]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.gbf_abi_version() != ABI_VERSION:
        raise GbfError(f"{LIB_PATH} has ABI version {lib.gbf_abi_version()}, this package needs {ABI_VERSION}: "
                       "rebuild it with jaxfluids_gb300.build.build()")
    _lib = lib
    return lib


def check(status: int, what: str) -> None:
    if status != GBF_OK:
        raise GbfError(f"{what}: {STATUS.get(status, status)} ({status})")
