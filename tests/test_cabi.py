"""CPU tests of the C ABI boundary: the library loads and exports every
function include/*.h declares, and reports the absence of a GPU as a
status instead of failing."""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names += re.findall(r"^\s*[A-Za-z_][\w\s\*]*?\b(bsg_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_api():
    names = declared_functions()
    assert "bsg_create" in names and "bsg_run" in names and len(names) >= 25


def test_library_exports_every_declared_symbol():
    from bsglmm_gb300 import _lib
    if not _lib.LIB_PATH.exists():
        pytest.fail(f"{_lib.LIB_PATH} not built (python -m bsglmm_gb300.build)")
    L = C.CDLL(str(_lib.LIB_PATH))
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing
    # and the ctypes signature table covers the header exactly
    assert set(_lib.SIGNATURES) == set(declared_functions())


def test_status_strings():
    from bsglmm_gb300 import _lib
    L = _lib.lib()
    for s in range(0, 9):
        assert L.bsg_status_string(s)
    assert L.bsg_status_string(0) == b"ok"


def test_create_reports_missing_device():
    from bsglmm_gb300 import _lib
    L = _lib.lib()
    h = C.c_void_p()
    st = L.bsg_create(0, C.byref(h))
    if st == 0:
        L.bsg_destroy(h)
        pytest.skip("a GPU is present")
    assert st == 7  # BSG_ERR_NO_DEVICE
    assert L.bsg_create(0, None) == 1
