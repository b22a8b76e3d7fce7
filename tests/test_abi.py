"""The C ABI library loads on a machine without a GPU and exports every entry
point that include/bcx.h declares (no compute calls here)."""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "bcx.h"
LIB = ROOT / "compute_gb300" / "libbcx.so"


def declared_entry_points():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(bcx_\w+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared_entry_points()
    assert "bcx_radix_sort_pairs" in names and "bcx_scan" in names and len(names) >= 20


def test_library_exports_every_declared_symbol():
    if not LIB.exists():
        pytest.skip("libbcx.so not built here")
    lib = ctypes.CDLL(str(LIB))
    missing = [n for n in declared_entry_points() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_the_header():
    from compute_gb300 import _lib
    assert set(declared_entry_points()) <= set(_lib.SIGNATURES), \
        set(declared_entry_points()) - set(_lib.SIGNATURES)


def test_status_codes_mirror_opencl():
    text = HEADER.read_text()
    assert re.search(r"BCX_INVALID_VALUE\s+-30", text)
    assert re.search(r"BCX_BUILD_PROGRAM_FAILURE\s+-11", text)


def test_no_alloc_free_query_protocol_without_gpu():
    """Size queries of the temporary-storage protocol need no device."""
    if not LIB.exists():
        pytest.skip("libbcx.so not built here")
    from compute_gb300 import _lib
    lib = _lib.lib()
    ver = ctypes.c_int(0)
    assert lib.bcx_get_version(ctypes.byref(ver)) == 0 and ver.value >= 10000
    # invalid dtype is rejected before any device work
    tb = ctypes.c_size_t(0)
    rc = lib.bcx_scan(None, 42, 0, 0, None, None, None, 10, 0, None, ctypes.byref(tb))
    assert rc == _lib.INVALID_VALUE
    assert b"dtype" in lib.bcx_last_error_string()
