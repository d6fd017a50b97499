"""The C-ABI library builds, loads and exports every declared symbol (CPU only)."""

import ctypes
import re
from pathlib import Path

from vajax_gb300 import _lib

HEADER = Path(__file__).resolve().parents[1] / "include" / "vajax_gb300.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(vgb_\w+)\s*\(", text)))


def test_header_matches_binding_table():
    assert declared_functions() == sorted(_lib.exported_symbols())


def test_library_exports_all_symbols():
    lib = _lib.load()
    for name in declared_functions():
        assert hasattr(lib, name), name
    assert lib.vgb_version() >= 100


def test_model_registry_matches_fixtures():
    from vajax_gb300.devices import model_info, model_keys
    lib = _lib.load()
    assert lib.vgb_num_models() == len(model_keys())
    for key in model_keys():
        info = model_info(key)
        name = ctypes.create_string_buffer(64)
        nn, nj, np_ = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        jrow = (ctypes.c_int * 64)()
        jcol = (ctypes.c_int * 64)()
        assert lib.vgb_model_info(info.model_id, name, 64, ctypes.byref(nn), ctypes.byref(nj), ctypes.byref(np_),
                                  jrow, jcol) == 0
        assert name.value.decode() == key
        assert (nn.value, nj.value, np_.value) == (len(info.nodes), len(info.jac), len(info.user_params))
        assert [(jrow[k], jcol[k]) for k in range(nj.value)] == list(info.jac)


def test_invalid_arguments_return_status():
    lib = _lib.load()
    h = ctypes.c_void_p()
    assert lib.vgb_circuit_create(0, 0, None, None, 0, None, None, ctypes.byref(h)) == 1
    assert lib.vgb_model_info(9999, None, 0, None, None, None, None, None) == 1
    assert b"model id" in lib.vgb_last_error(None)
