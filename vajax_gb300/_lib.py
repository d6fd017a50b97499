"""ctypes binding of ``libvajax_gb300.so`` (the C ABI in ``include/vajax_gb300.h``).

The library is the only compute path: if it is missing or cannot be loaded
the import fails loudly instead of falling back to anything else.
"""

from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libvajax_gb300.so"

_lib = None

i32p = C.POINTER(C.c_int)
f64p = C.POINTER(C.c_double)
i64p = C.POINTER(C.c_int64)
vp = C.c_void_p

# name -> (restype, argtypes)
SIGNATURES = {
    "vgb_version": (C.c_int, []),
    "vgb_math_eval": (C.c_int, [C.c_int, C.c_int, vp, vp, vp, vp]),
    "vgb_fp64_rate": (C.c_int, [C.c_int, f64p]),
    "vgb_batch_create": (C.c_int, [vp, C.c_int, C.POINTER(vp)]),
    "vgb_batch_set_group": (C.c_int, [vp, C.c_int, C.c_int, vp, vp, vp]),
    "vgb_batch_set_sources": (C.c_int, [vp, C.c_int, vp]),
    "vgb_batch_transient": (C.c_int, [vp, vp, vp, vp, vp, vp, vp, vp, vp, vp]),
    "vgb_batch_info": (C.c_int, [vp, vp]),
    "vgb_batch_set_coop": (C.c_int, [vp, C.c_int]),
    "vgb_batch_last_error": (C.c_char_p, [vp]),
    "vgb_batch_destroy": (C.c_int, [vp]),
    "vgb_num_models": (C.c_int, []),
    "vgb_model_info": (C.c_int, [C.c_int, C.c_char_p, C.c_int, i32p, i32p, i32p, i32p, i32p]),
    "vgb_circuit_create": (C.c_int, [C.c_int, C.c_int, i32p, i32p, C.c_int, i32p, i32p, C.POINTER(vp)]),
    "vgb_circuit_destroy": (C.c_int, [vp]),
    "vgb_last_error": (C.c_char_p, [vp]),
    "vgb_circuit_add_group": (C.c_int, [vp, C.c_int, C.c_int, i32p, f64p, C.c_int, i32p, f64p, f64p, C.c_double]),
    "vgb_circuit_set_sources": (C.c_int, [vp, C.c_int, C.c_int, i32p, i32p, i32p, f64p]),
    "vgb_circuit_set_internal_nodes": (C.c_int, [vp, C.c_int, i32p]),
    "vgb_circuit_set_noi_nodes": (C.c_int, [vp, C.c_int, i32p]),
    "vgb_set_tuning": (C.c_int, [vp, C.c_int, C.c_int]),
    "vgb_get_tuning": (C.c_int, [vp, C.c_int, i32p]),
    "vgb_circuit_analyze": (C.c_int, [vp]),
    "vgb_profile": (C.c_int, [vp, C.c_int, f64p]),
    "vgb_solver_order": (C.c_int, [vp, i32p, i32p]),
    "vgb_solver_match": (C.c_int, [vp, f64p]),
    "vgb_weighted_matching": (C.c_int, [C.c_int, i32p, i32p, f64p, i32p, f64p, f64p]),
    "vgb_solver_info": (C.c_int, [vp, i64p]),
    "vgb_circuit_finalize": (C.c_int, [vp, C.c_double, C.c_int, C.c_int]),
    "vgb_set_precision": (C.c_int, [vp, C.c_int, C.c_int]),
    "vgb_set_shunt_ref": (C.c_int, [vp, vp]),
    "vgb_pattern_info": (C.c_int, [vp, i32p, i32p, i64p, i64p]),
    "vgb_pattern_csr": (C.c_int, [vp, i32p, i32p]),
    "vgb_stamp_positions": (C.c_int, [vp, C.c_int, i32p]),
    "vgb_special_positions": (C.c_int, [vp, i32p, i32p]),
    "vgb_build_system": (C.c_int, [vp, vp, vp, vp, vp, vp, vp, f64p, vp, vp, vp, vp, vp, vp]),
    "vgb_eval_group": (C.c_int, [vp, C.c_int, vp, vp, vp]),
    "vgb_linear_solve": (C.c_int, [vp, vp, vp, vp, vp]),
    "vgb_nr_solve": (C.c_int, [vp, vp, vp, vp, vp, vp, vp, vp, f64p, C.c_int, i32p, i32p, f64p,
                               vp, vp, vp, vp, vp]),
    "vgb_transient": (C.c_int, [vp, f64p, f64p, f64p, f64p, f64p, f64p, f64p, f64p, f64p]),
    "vgb_tran_create": (C.c_int, [vp, f64p, f64p, f64p, f64p, f64p, C.POINTER(vp)]),
    "vgb_tran_advance": (C.c_int, [vp, C.c_int, i32p, i32p]),
    "vgb_tran_read": (C.c_int, [vp, f64p, f64p, f64p, f64p]),
    "vgb_tran_state": (C.c_int, [vp, f64p, f64p]),
    "vgb_tran_destroy": (C.c_int, [vp]),
    "vgb_linear_solve_dense_static": (C.c_int, [vp, vp, vp, vp, vp, vp]),
}


class VGBError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"vajax_gb300 error {code}: {msg}")
        self.code = code


def load():
    """Load the shared library (building it first if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        from vajax_gb300.build import build
        build()
    lib = C.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(code: int, handle=None):
    if code != 0:
        lib = load()
        msg = lib.vgb_last_error(handle)
        raise VGBError(code, msg.decode() if msg else "unknown error")


def exported_symbols():
    return list(SIGNATURES)
