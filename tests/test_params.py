"""Tuning-parameter table (bcx_param_*): in-memory get/set and the JSON file
under BCX_CACHE_DIR, without a GPU (the table of an unnamed device)."""
import ctypes

import pytest


@pytest.fixture()
def lib():
    from compute_gb300 import _lib
    return _lib.lib()


def test_param_defaults_and_set(lib):
    lib.bcx_param_clear()
    v = ctypes.c_uint(0)
    assert lib.bcx_param_get(b"obj_a", b"p", 42, ctypes.byref(v)) == 0 and v.value == 42
    assert lib.bcx_param_set(b"obj_a", b"p", 7) == 0
    assert lib.bcx_param_get(b"obj_a", b"p", 42, ctypes.byref(v)) == 0 and v.value == 7
    assert lib.bcx_param_set(b'bad"name', b"p", 1) == -30  # CL_INVALID_VALUE
    lib.bcx_param_clear()
    assert lib.bcx_param_get(b"obj_a", b"p", 42, ctypes.byref(v)) == 0 and v.value == 42


def test_param_file_round_trip(lib, tmp_path, monkeypatch):
    monkeypatch.setenv("BCX_CACHE_DIR", str(tmp_path))
    lib.bcx_param_clear()
    try:
        lib.bcx_param_set(b"segmented_sort_k32_v4", b"small_tile", 2048)
        lib.bcx_param_set(b"segmented_sort_k32_v4", b"small_blocks_per_sm", 3)
        lib.bcx_param_set(b"segmented_reduce_float", b"blocks_per_sm", 16)
        assert lib.bcx_param_save() == 0
        files = list((tmp_path / "tune").glob("*.json"))
        assert len(files) == 1
        import json
        table = json.loads(files[0].read_text())
        assert table == {"segmented_reduce_float": {"blocks_per_sm": 16},
                         "segmented_sort_k32_v4": {"small_blocks_per_sm": 3, "small_tile": 2048}}
        lib.bcx_param_clear()
        v = ctypes.c_uint(0)
        assert lib.bcx_param_get(b"segmented_sort_k32_v4", b"small_tile", 0, ctypes.byref(v)) == 0
        assert v.value == 2048
        assert lib.bcx_param_get(b"segmented_reduce_float", b"blocks_per_sm", 0, ctypes.byref(v)) == 0
        assert v.value == 16
    finally:
        monkeypatch.delenv("BCX_CACHE_DIR")
        lib.bcx_param_clear()
