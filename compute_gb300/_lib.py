"""ctypes binding of libbcx.so (the C ABI declared in include/bcx.h).

Loading fails loudly: if the shared library is missing or does not export an
entry point, importing this module raises instead of falling back to anything.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libbcx.so"

# status codes (include/bcx.h)
SUCCESS = 0
DEVICE_NOT_FOUND = -1
MEM_ALLOCATION_FAILURE = -4
OUT_OF_RESOURCES = -5
BUILD_PROGRAM_FAILURE = -11
INVALID_VALUE = -30
INVALID_KERNEL_NAME = -46
INVALID_BUFFER_SIZE = -61
DEVICE_TIMEOUT = -9001
UNSUPPORTED = -9002

DTYPES = {"char": 0, "uchar": 1, "short": 2, "ushort": 3, "int": 4, "uint": 5, "long": 6,
          "ulong": 7, "float": 8, "double": 9}
DTYPE_SIZE = {"char": 1, "uchar": 1, "short": 2, "ushort": 2, "int": 4, "uint": 4, "long": 8,
              "ulong": 8, "float": 4, "double": 8}
OPS = {"plus": 0, "multiplies": 1, "min": 2, "max": 3, "bit_and": 4, "bit_or": 5, "bit_xor": 6,
       "minus": 7, "divides": 8, "modulus": 9}
UNARY_OPS = {"identity": 0, "negate": 1, "abs": 2, "sqrt": 3, "logical_not": 4, "bit_not": 5}

_vp = C.c_void_p
_sz = C.c_size_t
_i = C.c_int
_szp = C.POINTER(C.c_size_t)

# name -> (restype, argtypes); the exported surface of include/bcx.h
SIGNATURES = {
    "bcx_get_version": (_i, [C.POINTER(_i)]),
    "bcx_last_error_string": (C.c_char_p, []),
    "bcx_device_count": (_i, [C.POINTER(_i)]),
    "bcx_set_device": (_i, [_i]),
    "bcx_device_info": (_i, [_i, C.c_char_p, _sz, C.POINTER(_i), _szp]),
    "bcx_stream_create": (_i, [C.POINTER(_vp)]),
    "bcx_stream_destroy": (_i, [_vp]),
    "bcx_stream_synchronize": (_i, [_vp]),
    "bcx_event_create": (_i, [C.POINTER(_vp)]),
    "bcx_event_destroy": (_i, [_vp]),
    "bcx_event_record": (_i, [_vp, _vp]),
    "bcx_event_synchronize": (_i, [_vp]),
    "bcx_event_query": (_i, [_vp, C.POINTER(_i)]),
    "bcx_event_elapsed_ms": (_i, [_vp, _vp, C.POINTER(C.c_float)]),
    "bcx_stream_wait_event": (_i, [_vp, _vp]),
    "bcx_malloc": (_i, [C.POINTER(_vp), _sz]),
    "bcx_free": (_i, [_vp]),
    "bcx_malloc_async": (_i, [C.POINTER(_vp), _sz, _vp]),
    "bcx_free_async": (_i, [_vp, _vp]),
    "bcx_host_register": (_i, [_vp, _sz, _i, C.POINTER(_vp)]),
    "bcx_host_unregister": (_i, [_vp]),
    "bcx_malloc_host": (_i, [C.POINTER(_vp), _sz]),
    "bcx_free_host": (_i, [_vp]),
    "bcx_memcpy_async": (_i, [_vp, _vp, _sz, _vp]),
    "bcx_memset_async": (_i, [_vp, _i, _sz, _vp]),
    "bcx_device_error_check": (_i, [_vp]),
    "bcx_device_error_word": (_i, [C.POINTER(_vp)]),
    "bcx_debug_expire_wait": (_i, [_vp, _i, C.c_uint]),
    "bcx_radix_sort_keys": (_i, [_vp, _i, _vp, _sz, _i, _vp, _szp]),
    "bcx_radix_sort_pairs": (_i, [_vp, _i, _sz, _vp, _vp, _sz, _i, _vp, _szp]),
    "bcx_sort_keys": (_i, [_vp, _i, _vp, _sz, _i, _vp, _szp]),
    "bcx_sort_pairs": (_i, [_vp, _i, _sz, _vp, _vp, _sz, _i, _vp, _szp]),
    "bcx_sort_pairs_host": (_i, [_vp, _i, _sz, _vp, _vp, _sz, _i]),
    "bcx_scan": (_i, [_vp, _i, _i, _i, _vp, _vp, _vp, _sz, _i, _vp, _szp]),
    "bcx_scan_noalloc": (_i, [_vp, _i, _i, _i, _vp, _vp, _vp, _sz, _i]),
    "bcx_reduce": (_i, [_vp, _i, _i, _vp, _sz, _vp, _i, _vp, _szp]),
    "bcx_accumulate": (_i, [_vp, _i, _i, _vp, _sz, _vp, _vp, _i, _vp, _szp]),
    "bcx_transform_unary": (_i, [_vp, _i, _i, _vp, _vp, _sz]),
    "bcx_transform_binary": (_i, [_vp, _i, _i, _vp, _vp, _vp, _sz]),
    "bcx_transform_saxpy": (_i, [_vp, _i, _vp, _vp, _vp, _vp, _sz]),
    "bcx_reduce_by_key": (_i, [_vp, _i, _i, _i, _vp, _vp, _sz, _vp, _vp, _vp, _i, _vp, _szp]),
    "bcx_segmented_scan": (_i, [_vp, _i, _i, _i, _vp, _vp, _vp, _sz, _vp, _sz, _i, _vp, _szp]),
    "bcx_segmented_reduce": (_i, [_vp, _i, _i, _vp, _vp, _sz, _vp, _vp, _i, _vp, _szp]),
    "bcx_segmented_sort_pairs": (_i, [_vp, _i, _sz, _vp, _vp, _sz, _vp, _sz, _i, _vp, _szp]),
    "bcx_server_create": (_i, [C.POINTER(_vp), _i, _sz]),
    "bcx_server_configure": (_i, [_vp, _sz, _sz, _sz]),
    "bcx_server_inject_faults": (_i, [_vp, _sz, _i]),
    "bcx_server_submit": (_i, [_vp, C.c_void_p, C.POINTER(C.c_uint64)]),
    "bcx_server_wait": (_i, [_vp, C.c_uint64, C.POINTER(C.c_double)]),
    "bcx_server_wait_for": (_i, [_vp, C.c_uint64, C.c_double, C.POINTER(C.c_double)]),
    "bcx_server_drain": (_i, [_vp]),
    "bcx_server_stats": (_i, [_vp, C.c_void_p]),
    "bcx_server_reset_stats": (_i, [_vp]),
    "bcx_server_destroy": (_i, [_vp]),
    "bcx_jit_get_kernel": (_i, [C.c_char_p, C.c_char_p, C.c_char_p, C.POINTER(_vp)]),
    "bcx_jit_launch": (_i, [_vp, C.c_uint, C.c_uint, _sz, _vp, C.POINTER(_vp)]),
    "bcx_jit_build_log": (_i, [C.c_char_p, _sz, _szp]),
    "bcx_jit_cache_stats": (_i, [C.POINTER(C.c_uint64)] * 5),
    "bcx_jit_cache_configure": (_i, [_sz, _i]),
    "bcx_device_sm_count": (_i, [C.POINTER(_i)]),
    "bcx_param_get": (_i, [C.c_char_p, C.c_char_p, C.c_uint, C.POINTER(C.c_uint)]),
    "bcx_param_set": (_i, [C.c_char_p, C.c_char_p, C.c_uint]),
    "bcx_param_save": (_i, []),
    "bcx_param_clear": (_i, []),
    "bcx_tune_segmented_sort_pairs": (_i, [_vp, _i, _sz, _vp, _vp, _sz, _vp, _sz, C.c_char_p, _sz]),
    "bcx_tune_segmented_scan": (_i, [_vp, _i, _vp, _sz, _vp, _sz, C.c_char_p, _sz]),
    "bcx_tune_segmented_reduce": (_i, [_vp, _i, _vp, _vp, _sz, C.c_char_p, _sz]),
    "bcx_profile_enable": (_i, [_i]),
    "bcx_profile_reset": (_i, []),
    "bcx_profile_read": (_i, [C.c_char_p, _sz, C.POINTER(C.c_uint64), C.POINTER(C.c_double), _sz, _szp]),
}


class Request(C.Structure):
    """bcx_request (include/bcx.h)."""
    _fields_ = [("kind", C.c_int), ("dtype", C.c_int), ("value_bytes", C.c_size_t), ("n", C.c_size_t),
                ("flags", C.c_int), ("keys", C.c_void_p), ("values", C.c_void_p), ("out", C.c_void_p),
                ("out_values", C.c_void_p)]


class ServerStats(C.Structure):
    """bcx_server_stats_t (include/bcx.h)."""
    _fields_ = [("completed", C.c_uint64), ("batches", C.c_uint64), ("batched_requests", C.c_uint64),
                ("pending", C.c_uint64), ("used_bytes", C.c_size_t), ("p50_ms", C.c_double),
                ("p99_ms", C.c_double), ("max_ms", C.c_double)]


class BcxError(RuntimeError):
    """A libbcx call returned a non-zero status (an OpenCL-style cl_int code)."""

    def __init__(self, status: int, where: str, text: str):
        super().__init__(f"{where} failed with status {status}: {text}")
        self.status = status


def load(path: Path | None = None) -> C.CDLL:
    p = Path(path or os.environ.get("BCX_LIBRARY", LIB_PATH))
    if not p.exists():
        raise ImportError(f"libbcx.so not found at {p}: build it with "
                          "`python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)  # AttributeError if the symbol is missing
        fn.restype = res
        fn.argtypes = args
    return lib


_LIB: C.CDLL | None = None


def lib() -> C.CDLL:
    global _LIB
    if _LIB is None:
        _LIB = load()
    return _LIB


def check(status: int, where: str) -> None:
    if status != SUCCESS:
        text = lib().bcx_last_error_string().decode(errors="replace")
        raise BcxError(status, where, text)
