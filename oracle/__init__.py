"""CPU oracle for the bcx hot path -- TEST INFRASTRUCTURE ONLY.

A ctypes wrapper over oracle/_build/libbcx_oracle.so (built from oracle.cpp by
oracle/Makefile).  Only the test suite, the package smoke check and the
benchmark's CPU-baseline leg use it, always as the checker or the timed CPU
baseline, never as the product path.  The restatement is pinned to the
reference's golden vectors (tests/golden/reference_vectors.json).
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libbcx_oracle.so"

DTYPES = {"char": 0, "uchar": 1, "short": 2, "ushort": 3, "int": 4, "uint": 5, "long": 6,
          "ulong": 7, "float": 8, "double": 9}
NP = {"char": np.int8, "uchar": np.uint8, "short": np.int16, "ushort": np.uint16, "int": np.int32,
      "uint": np.uint32, "long": np.int64, "ulong": np.uint64, "float": np.float32, "double": np.float64}
OPS = {"plus": 0, "multiplies": 1, "min": 2, "max": 3, "bit_and": 4, "bit_or": 5, "bit_xor": 6,
       "minus": 7, "divides": 8, "modulus": 9}


def build() -> Path:
    """Compiles the oracle with the committed Makefile (g++, portable flags)."""
    src = HERE / "oracle.cpp"
    if not LIB.exists() or LIB.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        vp, sz, i = C.c_void_p, C.c_size_t, C.c_int
        L.oracle_radix_keys.argtypes = [i, i, vp, vp, sz]
        L.oracle_radix_sort.argtypes = [i, sz, vp, vp, sz, i]
        L.oracle_insertion_sort.argtypes = [i, sz, vp, vp, sz, i]
        L.oracle_sort.argtypes = [i, vp, sz, i]
        L.oracle_sort_by_key.argtypes = [i, sz, vp, vp, sz, i]
        L.oracle_scan.argtypes = [i, i, i, vp, vp, vp, sz]
        L.oracle_fold.argtypes = [i, i, vp, sz, vp, vp]
        L.oracle_sum_f64.argtypes = [i, vp, sz, C.c_double]
        L.oracle_sum_f64.restype = C.c_double
        L.oracle_prefix_f64.argtypes = [i, i, vp, sz, C.c_double, vp]
        L.oracle_saxpy.argtypes = [i, vp, vp, vp, vp, sz, i]
        L.oracle_transform_binary.argtypes = [i, i, vp, vp, vp, sz]
        L.oracle_reduce_by_key.argtypes = [i, i, i, vp, vp, sz, vp, vp]
        L.oracle_reduce_by_key.restype = sz
        L.oracle_cpu_merge_sort_by_key_u32.argtypes = [vp, vp, sz, i]
        L.oracle_cpu_exclusive_scan_i32.argtypes = [vp, vp, sz, C.c_int32, i]
        L.oracle_cpu_reduce_i32.argtypes = [vp, sz, i]
        L.oracle_cpu_reduce_i32.restype = C.c_int32
        L.oracle_cpu_saxpy_f32.argtypes = [C.c_float, vp, vp, vp, sz, i]
        L.oracle_hardware_threads.restype = i
        _lib = L
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def _scalar(v, dtype):
    return np.array([v], dtype=NP[dtype])


def radix_keys(a: np.ndarray, dtype: str, descending=False) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=NP[dtype])
    out = np.empty(a.size, dtype=np.uint64)
    lib().oracle_radix_keys(DTYPES[dtype], int(descending), _p(a), _p(out), a.size)
    return out


def radix_sort(keys: np.ndarray, dtype: str, values=None, descending=False):
    k = np.array(keys, dtype=NP[dtype], copy=True)
    v = None if values is None else np.array(values, copy=True)
    vb = 0 if v is None else v.nbytes // max(k.size, 1)
    lib().oracle_radix_sort(DTYPES[dtype], vb, _p(k), _p(v), k.size, int(descending))
    return k if v is None else (k, v)


def insertion_sort(keys: np.ndarray, dtype: str, values=None, descending=False):
    k = np.array(keys, dtype=NP[dtype], copy=True)
    v = None if values is None else np.array(values, copy=True)
    vb = 0 if v is None else v.nbytes // max(k.size, 1)
    lib().oracle_insertion_sort(DTYPES[dtype], vb, _p(k), _p(v), k.size, int(descending))
    return k if v is None else (k, v)


def sort(keys, dtype: str, descending=False):
    k = np.array(keys, dtype=NP[dtype], copy=True)
    lib().oracle_sort(DTYPES[dtype], _p(k), k.size, int(descending))
    return k


def sort_by_key(keys, values, dtype: str, descending=False):
    k = np.array(keys, dtype=NP[dtype], copy=True)
    v = np.array(values, copy=True)
    vb = v.nbytes // max(k.size, 1) if k.size else v.itemsize
    lib().oracle_sort_by_key(DTYPES[dtype], vb, _p(k), _p(v), k.size, int(descending))
    return k, v


def scan(a, dtype: str, op="plus", exclusive=False, init=0):
    a = np.ascontiguousarray(a, dtype=NP[dtype])
    out = np.empty_like(a)
    ini = _scalar(init, dtype)
    lib().oracle_scan(DTYPES[dtype], OPS[op], int(exclusive), _p(ini), _p(a), _p(out), a.size)
    return out


def fold(a, dtype: str, op="plus", init=None):
    a = np.ascontiguousarray(a, dtype=NP[dtype])
    out = np.zeros(1, dtype=NP[dtype])
    ini = None if init is None else _scalar(init, dtype)
    lib().oracle_fold(DTYPES[dtype], OPS[op], _p(a), a.size, _p(ini), _p(out))
    return out[0]


def sum_f64(a, dtype: str, init=0.0) -> float:
    a = np.ascontiguousarray(a, dtype=NP[dtype])
    return float(lib().oracle_sum_f64(DTYPES[dtype], _p(a), a.size, float(init)))


def prefix_f64(a, dtype: str, exclusive=False, init=0.0) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=NP[dtype])
    out = np.empty(a.size, dtype=np.float64)
    lib().oracle_prefix_f64(DTYPES[dtype], int(exclusive), _p(a), a.size, float(init), _p(out))
    return out


def saxpy(alpha, x, y, dtype="float", fused=True):
    x = np.ascontiguousarray(x, dtype=NP[dtype])
    y = np.ascontiguousarray(y, dtype=NP[dtype])
    out = np.empty_like(x)
    a = _scalar(alpha, dtype)
    lib().oracle_saxpy(DTYPES[dtype], _p(a), _p(x), _p(y), _p(out), x.size, int(fused))
    return out


def transform_binary(a, b, dtype: str, op: str):
    a = np.ascontiguousarray(a, dtype=NP[dtype])
    b = np.ascontiguousarray(b, dtype=NP[dtype])
    out = np.empty_like(a)
    lib().oracle_transform_binary(DTYPES[dtype], OPS[op], _p(a), _p(b), _p(out), a.size)
    return out


def reduce_by_key(keys, values, key_dtype: str, value_dtype: str, op="plus"):
    k = np.ascontiguousarray(keys, dtype=NP[key_dtype])
    v = np.ascontiguousarray(values, dtype=NP[value_dtype])
    ko = np.empty_like(k)
    vo = np.empty_like(v)
    m = lib().oracle_reduce_by_key(DTYPES[key_dtype], DTYPES[value_dtype], OPS[op], _p(k), _p(v),
                                   k.size, _p(ko), _p(vo))
    return ko[:m], vo[:m]


# ---- CPU-device algorithms (timed CPU baseline) ---------------------------
def cpu_merge_sort_by_key_u32(keys: np.ndarray, values: np.ndarray, threads=0) -> None:
    lib().oracle_cpu_merge_sort_by_key_u32(_p(keys), _p(values), keys.size, int(threads))


def cpu_exclusive_scan_i32(a: np.ndarray, out: np.ndarray, init=0, threads=0) -> None:
    lib().oracle_cpu_exclusive_scan_i32(_p(a), _p(out), a.size, int(init), int(threads))


def cpu_reduce_i32(a: np.ndarray, threads=0) -> int:
    return int(lib().oracle_cpu_reduce_i32(_p(a), a.size, int(threads)))


def cpu_saxpy_f32(alpha, x, y, out, threads=0) -> None:
    lib().oracle_cpu_saxpy_f32(float(alpha), _p(x), _p(y), _p(out), x.size, int(threads))


def hardware_threads() -> int:
    return int(lib().oracle_hardware_threads())
