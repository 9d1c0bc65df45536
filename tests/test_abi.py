"""The C-ABI library loads and exports every symbol include/trixi_gb300.h declares
(no compute calls: CPU only)."""
import ctypes
import os
import re

import pytest

from trixi_gb300 import _lib

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                      "trixi_gb300.h")


def declared_symbols():
    src = open(HEADER, encoding="utf-8").read()
    return sorted(set(re.findall(r"^int\s+(tg_\w+)\s*\(", src, flags=re.M)))


def test_header_lists_match_binding():
    assert declared_symbols() == sorted(_lib.EXPORTS)


def test_library_exports_every_declared_symbol():
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("libtrixi_gb300.so not built")
    lib = ctypes.CDLL(_lib.LIB_PATH)
    for name in declared_symbols():
        assert hasattr(lib, name), name
    assert _lib.load().tg_api_version() == 3


def test_invalid_config_is_rejected_without_gpu():
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("libtrixi_gb300.so not built")
    lib = _lib.load()
    cfg = _lib.tg_config()
    cfg.ndims = 4
    h = ctypes.c_void_p()
    rc = lib.tg_ctx_create(ctypes.byref(cfg), ctypes.byref(h))
    assert rc == -2 and not h.value
    assert "ndims" in _lib.last_error()
    cfg.ndims, cfg.polydeg, cfg.nelements, cfg.ninterfaces = 2, 3, 4, 9
    assert lib.tg_ctx_create(ctypes.byref(cfg), ctypes.byref(h)) == _lib.TG_ERR_INVALID_ARGUMENT
    assert "interfaces" in _lib.last_error()
    cfg.ninterfaces, cfg.nmortars = 8, -1
    assert lib.tg_ctx_create(ctypes.byref(cfg), ctypes.byref(h)) == _lib.TG_ERR_INVALID_ARGUMENT
