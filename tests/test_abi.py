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


def test_config_struct_layout_matches_header(tmp_path):
    # the ctypes mirror of tg_config (trixi_gb300/_lib.py) against the C header,
    # field by field: offsetof from a C program compiled against include/
    import shutil
    import subprocess
    gcc = shutil.which("gcc") or shutil.which("cc")
    if gcc is None:
        pytest.skip("no C compiler")
    fields = [f[0] for f in _lib.tg_config._fields_]
    src = tmp_path / "layout.c"
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "trixi_gb300.h"',
             'int main(void) {', '  printf("size %zu\\n", sizeof(tg_config));']
    lines += [f'  printf("{f} %zu\\n", offsetof(tg_config, {f}));' for f in fields]
    lines += ['  return 0;', '}']
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([gcc, "-I", os.path.dirname(HEADER), str(src), "-o", str(exe)], check=True)
    out = dict(line.split() for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                       check=True).stdout.splitlines())
    assert int(out["size"]) == ctypes.sizeof(_lib.tg_config)
    for f in fields:
        assert int(out[f]) == getattr(_lib.tg_config, f).offset, f
