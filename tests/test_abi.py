"""The C-ABI library loads, exports every function its headers declare, and
rejects bad arguments with status codes (no GPU work is done here)."""
import ctypes
import re
from pathlib import Path

import pytest

from spacelab_gb300 import _lib

INCLUDE = Path(__file__).resolve().parents[1] / "include"


def _declared_functions():
    names = []
    for h in sorted(INCLUDE.glob("*.h")):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(sl[h]?_\w+)\s*\(", text, flags=re.M):
            names.append(m.group(1))
    return sorted(set(names))


def test_headers_declare_functions():
    names = _declared_functions()
    assert "sl_step" in names and "slh_build_cluster" in names
    assert len(names) >= 20


@pytest.mark.parametrize("name", _declared_functions())
def test_library_exports_declared_symbol(name):
    lib = ctypes.CDLL(str(_lib.LIB_PATH))
    assert hasattr(lib, name), f"{name} declared in include/ but not exported"


def test_binding_covers_all_declared():
    assert set(_declared_functions()) <= set(_lib.EXPORTED_SYMBOLS)


def test_version_and_null_handling():
    lib = _lib.lib()
    assert lib.sl_version() == _lib.API_VERSION
    assert lib.sl_destroy(None) == _lib.SL_OK
    assert lib.sl_step(None, 1, 0, None) == _lib.SL_ERR_ARG
    assert b"null" in lib.sl_last_error()


@pytest.mark.parametrize("n", [0, -5, 46341])
def test_create_rejects_bad_n_without_touching_cuda(n):
    lib = _lib.lib()
    h = ctypes.c_void_p()
    mat = _lib.Material(6.674e-8, 4e-13, 0.3, 1e-5, 1e-5)
    assert lib.sl_create(n, ctypes.byref(mat), 0, ctypes.byref(h)) == _lib.SL_ERR_ARG
    assert not h.value


def test_create_rejects_bad_material_and_mode():
    lib = _lib.lib()
    h = ctypes.c_void_p()
    bad = _lib.Material(6.674e-8, 4e-13, 0.3, 1e-5, 0.0)
    assert lib.sl_create(10, ctypes.byref(bad), 0, ctypes.byref(h)) == _lib.SL_ERR_ARG
    good = _lib.Material(6.674e-8, 4e-13, 0.3, 1e-5, 1e-5)
    assert lib.sl_create(10, ctypes.byref(good), 99, ctypes.byref(h)) == _lib.SL_ERR_UNSUPPORTED
    assert lib.sl_create(10, None, 0, ctypes.byref(h)) == _lib.SL_ERR_ARG


def test_missing_library_fails_loudly(tmp_path):
    with pytest.raises(ImportError, match="no CPU fallback"):
        _lib.load(tmp_path / "nope.so")
