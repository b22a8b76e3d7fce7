"""compute_gb300 -- GB300-native (sm_103a) data-parallel core with the
Boost.Compute algorithm interface.

The compute path is libbcx.so (hand-written CUDA kernels behind the C ABI in
include/bcx.h).  This module mirrors the reference's algorithm entry points for
device tensors so that Python callers -- and the tests -- use the same names,
argument meaning and error behaviour as ``boost::compute``:

=========================  ==================================================
boost::compute             here (tensors live on the current CUDA device)
=========================  ==================================================
sort(first, last, q)       sort(keys, descending=False)
sort_by_key(k, k+n, v)     sort_by_key(keys, values, descending=False)
stable_sort(_by_key)       stable_sort / stable_sort_by_key (same radix path)
detail::radix_sort         radix_sort(keys, descending) -- radix for any n
exclusive_scan(f, l, r,    exclusive_scan(inp, out=None, init=0, op="plus")
  init, op)
inclusive_scan(f, l, r,    inclusive_scan(inp, out=None, op="plus")
  op)
reduce(f, l, &r, op)       reduce(inp, op="plus", out=None) -> device scalar
accumulate(f, l, init, op) accumulate(inp, init, op="plus") -> host value
transform(f, l, r, op)     transform(inp, op, other=None, out=None)
transform(x, y, r, a*_1+_2) saxpy(alpha, x, y, out=None)
reduce_by_key(...)         reduce_by_key(keys, values, op="plus")
=========================  ==================================================

Failures raise BcxError carrying the library status (OpenCL cl_int codes),
the analogue of boost::compute::opencl_error.  Nothing here falls back to
another implementation: without libbcx.so the import fails.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

from ._lib import (DTYPES, DTYPE_SIZE, OPS, UNARY_OPS, BcxError, check, lib)  # noqa: F401

__all__ = [
    "BcxError", "lib", "sort", "sort_by_key", "stable_sort", "stable_sort_by_key", "radix_sort",
    "radix_sort_by_key", "exclusive_scan", "inclusive_scan", "reduce", "accumulate", "transform",
    "saxpy", "reduce_by_key", "sort_by_key_host", "profile", "device_error_check", "bcx_dtype",
]

_TORCH_TO_BCX = {
    "torch.int8": "char", "torch.uint8": "uchar", "torch.int16": "short", "torch.uint16": "ushort",
    "torch.int32": "int", "torch.uint32": "uint", "torch.int64": "long", "torch.uint64": "ulong",
    "torch.float32": "float", "torch.float64": "double",
}


def bcx_dtype(t, override: Optional[str] = None) -> str:
    """The bcx element type of tensor `t` (or `override`, e.g. "uint" for an
    int32 tensor holding uint32 bit patterns)."""
    if override is not None:
        if override not in DTYPES:
            raise ValueError(f"unknown dtype {override!r}")
        if DTYPE_SIZE[override] != t.element_size():
            raise ValueError(f"dtype {override!r} does not match a {t.element_size()}-byte tensor")
        return override
    name = _TORCH_TO_BCX.get(str(t.dtype))
    if name is None:
        raise TypeError(f"unsupported tensor dtype {t.dtype}")
    return name


def _stream(stream=None) -> int:
    import torch
    if stream is None:
        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


def _ptr(t) -> Optional[int]:
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError("expected a CUDA tensor")
    if not t.is_contiguous():
        raise ValueError("expected a contiguous tensor")
    return t.data_ptr()


def _scalar(value, dtype: str) -> C.Array:
    import struct
    fmt = {"char": "b", "uchar": "B", "short": "h", "ushort": "H", "int": "i", "uint": "I",
           "long": "q", "ulong": "Q", "float": "f", "double": "d"}[dtype]
    if dtype in ("float", "double"):
        raw = struct.pack(fmt, float(value))
    else:
        bits = 8 * DTYPE_SIZE[dtype]
        v = int(value) & ((1 << bits) - 1)
        if fmt.islower() and v >= (1 << (bits - 1)):
            v -= 1 << bits
        raw = struct.pack(fmt, v)
    return (C.c_ubyte * len(raw)).from_buffer_copy(raw)


# ---- sort -----------------------------------------------------------------
def radix_sort(keys, descending: bool = False, dtype: Optional[str] = None, stream=None) -> None:
    """detail::radix_sort: stable LSD radix sort of `keys` in place (any n)."""
    kt = bcx_dtype(keys, dtype)
    check(lib().bcx_radix_sort_keys(_stream(stream), DTYPES[kt], _ptr(keys), keys.numel(),
                                    int(bool(descending)), None, None), "radix_sort")


def radix_sort_by_key(keys, values, descending: bool = False, dtype: Optional[str] = None,
                      stream=None) -> None:
    """detail::radix_sort_by_key: stable; values follow their keys."""
    kt = bcx_dtype(keys, dtype)
    n = keys.numel()
    vb = (values.numel() * values.element_size()) // n if n else values.element_size()
    check(lib().bcx_radix_sort_pairs(_stream(stream), DTYPES[kt], vb, _ptr(keys), _ptr(values),
                                     keys.numel(), int(bool(descending)), None, None),
          "radix_sort_by_key")


def sort(keys, descending: bool = False, dtype: Optional[str] = None, stream=None) -> None:
    """compute::sort with less<T> (or greater<T> when descending)."""
    if not keys.is_cuda:
        raise ValueError("sort: expected a CUDA tensor (use sort_by_key_host for host data)")
    kt = bcx_dtype(keys, dtype)
    check(lib().bcx_sort_keys(_stream(stream), DTYPES[kt], _ptr(keys), keys.numel(),
                              int(bool(descending)), None, None), "sort")


def sort_by_key(keys, values, descending: bool = False, dtype: Optional[str] = None,
                stream=None) -> None:
    """compute::sort_by_key (stable on the radix path)."""
    kt = bcx_dtype(keys, dtype)
    n = keys.numel()
    vb = (values.numel() * values.element_size()) // n if n else values.element_size()
    check(lib().bcx_sort_pairs(_stream(stream), DTYPES[kt], vb, _ptr(keys), _ptr(values), n,
                               int(bool(descending)), None, None), "sort_by_key")


stable_sort = sort
stable_sort_by_key = sort_by_key


def sort_by_key_host(keys, values, descending: bool = False, dtype: Optional[str] = None,
                     stream=None) -> None:
    """sort_by_key on host (CPU, ideally pinned) tensors: copy in, sort on the
    device, copy back, synchronize."""
    kt = bcx_dtype(keys, dtype)
    n = keys.numel()
    vb = (values.numel() * values.element_size()) // n if n else values.element_size()
    check(lib().bcx_sort_pairs_host(_stream(stream), DTYPES[kt], vb, keys.data_ptr(),
                                    values.data_ptr(), n, int(bool(descending))), "sort_by_key_host")


# ---- scan -----------------------------------------------------------------
def _scan(inp, out, exclusive: bool, init, op: str, compensated: bool, dtype, stream):
    import torch
    t = bcx_dtype(inp, dtype)
    if out is None:
        out = torch.empty_like(inp)
    init_buf = _scalar(init, t)
    check(lib().bcx_scan(_stream(stream), DTYPES[t], OPS[op], int(exclusive), init_buf, _ptr(inp),
                         _ptr(out), inp.numel(), int(bool(compensated)), None, None),
          "exclusive_scan" if exclusive else "inclusive_scan")
    return out


def exclusive_scan(inp, out=None, init=0, op: str = "plus", compensated: bool = False,
                   dtype: Optional[str] = None, stream=None):
    """compute::exclusive_scan: out[0] = init, out[i] = out[i-1] op in[i-1]."""
    return _scan(inp, out, True, init, op, compensated, dtype, stream)


def inclusive_scan(inp, out=None, op: str = "plus", compensated: bool = False,
                   dtype: Optional[str] = None, stream=None):
    """compute::inclusive_scan: out[i] = in[0] op ... op in[i]."""
    return _scan(inp, out, False, 0, op, compensated, dtype, stream)


# ---- reduce / accumulate --------------------------------------------------
def reduce(inp, op: str = "plus", out=None, compensated: bool = False,
           dtype: Optional[str] = None, stream=None):
    """compute::reduce into a one-element device tensor (returned)."""
    import torch
    t = bcx_dtype(inp, dtype)
    if out is None:
        out = torch.zeros(1, dtype=inp.dtype, device=inp.device)
    check(lib().bcx_reduce(_stream(stream), DTYPES[t], OPS[op], _ptr(inp), inp.numel(), _ptr(out),
                           int(bool(compensated)), None, None), "reduce")
    return out


def accumulate(inp, init, op: str = "plus", compensated: bool = True,
               dtype: Optional[str] = None, stream=None):
    """compute::accumulate: returns init op reduce(inp) as a host scalar
    (blocks, like the reference)."""
    import torch
    t = bcx_dtype(inp, dtype)
    out = torch.zeros(1, dtype=inp.dtype, device=inp.device)
    check(lib().bcx_accumulate(_stream(stream), DTYPES[t], OPS[op], _ptr(inp), inp.numel(),
                               _scalar(init, t), _ptr(out), int(bool(compensated)), None, None),
          "accumulate")
    return out.item()


# ---- transform ------------------------------------------------------------
def transform(inp, op: str, other=None, out=None, dtype: Optional[str] = None, stream=None):
    """compute::transform with a built-in functor: unary when `other` is None,
    binary (zip + unpack) otherwise."""
    import torch
    t = bcx_dtype(inp, dtype)
    if out is None:
        out = torch.empty_like(inp)
    if other is None:
        check(lib().bcx_transform_unary(_stream(stream), DTYPES[t], UNARY_OPS[op], _ptr(inp),
                                        _ptr(out), inp.numel()), "transform")
    else:
        check(lib().bcx_transform_binary(_stream(stream), DTYPES[t], OPS[op], _ptr(inp), _ptr(other),
                                         _ptr(out), inp.numel()), "transform")
    return out


def saxpy(alpha, x, y, out=None, stream=None):
    """compute::transform(x, x+n, y, out, alpha * _1 + _2) for float/double."""
    import torch
    t = bcx_dtype(x)
    if out is None:
        out = torch.empty_like(x)
    check(lib().bcx_transform_saxpy(_stream(stream), DTYPES[t], _scalar(alpha, t), _ptr(x), _ptr(y),
                                    _ptr(out), x.numel()), "saxpy")
    return out


# ---- reduce_by_key --------------------------------------------------------
def reduce_by_key(keys, values, op: str = "plus", compensated: bool = True,
                  key_dtype: Optional[str] = None, value_dtype: Optional[str] = None, stream=None):
    """compute::reduce_by_key with equal_to: returns (keys_out, values_out)
    trimmed to the number of runs."""
    import torch
    kt, vt = bcx_dtype(keys, key_dtype), bcx_dtype(values, value_dtype)
    n = keys.numel()
    keys_out = torch.empty_like(keys)
    vals_out = torch.empty_like(values)
    count = torch.zeros(1, dtype=torch.int64, device=keys.device)
    check(lib().bcx_reduce_by_key(_stream(stream), DTYPES[kt], DTYPES[vt], OPS[op], _ptr(keys),
                                  _ptr(values), n, _ptr(keys_out), _ptr(vals_out), _ptr(count),
                                  int(bool(compensated)), None, None), "reduce_by_key")
    m = int(count.item())
    return keys_out[:m], vals_out[:m]


# ---- profiling / errors ---------------------------------------------------
def device_error_check(stream=None) -> None:
    """Synchronize and raise if a bounded device-side wait expired."""
    check(lib().bcx_device_error_check(_stream(stream)), "device_error_check")


class profile:
    """Context manager: per-kernel launch counts and CUDA-event milliseconds of
    every libbcx kernel launched inside the block."""

    def __enter__(self):
        check(lib().bcx_profile_reset(), "profile_reset")
        check(lib().bcx_profile_enable(1), "profile_enable")
        self.kernels = {}
        return self

    def __exit__(self, *exc):
        check(lib().bcx_profile_enable(0), "profile_enable")
        self.kernels = read_profile()
        return False


def read_profile() -> dict:
    cap, stride = 64, 64
    names = C.create_string_buffer(cap * stride)
    launches = (C.c_uint64 * cap)()
    ms = (C.c_double * cap)()
    count = C.c_size_t(0)
    check(lib().bcx_profile_read(names, stride, launches, ms, cap, C.byref(count)), "profile_read")
    out = {}
    for i in range(min(count.value, cap)):
        name = names.raw[i * stride:(i + 1) * stride].split(b"\0", 1)[0].decode()
        out[name] = {"launches": int(launches[i]), "ms": float(ms[i])}
    return out
