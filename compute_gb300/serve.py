"""Python handle on the continuous-batching request server (bcx_server_* in
include/bcx.h).  Requests reference host buffers (numpy arrays or pinned torch
tensors) or, with device=True, CUDA tensors; either must stay alive until the
request's ticket has been waited for."""
from __future__ import annotations

import ctypes as C

from ._lib import DTYPES, Request, ServerStats, check, lib

KINDS = {"sort_by_key": 0, "exclusive_scan": 1, "reduce": 2}


def _addr(a) -> int:
    if a is None:
        return 0
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    return a.ctypes.data


class Server:
    def __init__(self, slots: int = 8, memory_budget_bytes: int = 0, small_limit: int | None = None,
                 batch_elems: int = 0, batch_count: int = 0):
        self._h = C.c_void_p()
        check(lib().bcx_server_create(C.byref(self._h), slots, memory_budget_bytes), "server_create")
        if small_limit is not None or batch_elems or batch_count:
            check(lib().bcx_server_configure(self._h, small_limit if small_limit is not None else 1 << 18,
                                             batch_elems, batch_count), "server_configure")
        self._keep = {}

    def submit(self, kind: str, dtype: str, keys, values=None, out=None, out_values=None,
               n: int | None = None, device: bool = False) -> int:
        """Queue one request; sorts write to out/out_values (default: in place)."""
        if n is None:
            n = int(keys.size if hasattr(keys, "size") and not callable(keys.size) else keys.numel())
        vb = 0
        if values is not None:
            vb = int(values.itemsize if hasattr(values, "itemsize") else values.element_size())
        if kind == "sort_by_key":
            out = keys if out is None else out
            out_values = values if out_values is None else out_values
        req = Request(KINDS[kind], DTYPES[dtype], vb, n, 1 if device else 0, _addr(keys), _addr(values),
                      _addr(out), _addr(out_values))
        t = C.c_uint64(0)
        check(lib().bcx_server_submit(self._h, C.byref(req), C.byref(t)), "server_submit")
        self._keep[t.value] = (keys, values, out, out_values)
        return t.value

    def submit_request(self, req: Request) -> int:
        """Queue a prepared bcx_request; its buffers are the caller's to keep alive."""
        t = C.c_uint64(0)
        check(lib().bcx_server_submit(self._h, C.byref(req), C.byref(t)), "server_submit")
        return t.value

    def wait(self, ticket: int, timeout: float | None = None) -> float:
        """Latency of the request in ms; with `timeout` (seconds) raises BcxError
        (BCX_DEVICE_TIMEOUT) if it has not finished by then."""
        ms = C.c_double(0)
        limit = -1.0 if timeout is None else float(timeout) * 1e3
        rc = lib().bcx_server_wait_for(self._h, C.c_uint64(ticket), limit, C.byref(ms))
        if rc != -9001:
            self._keep.pop(ticket, None)
        check(rc, "server_wait")
        return ms.value

    def inject_faults(self, fake_free_bytes: int = 0, fail_allocations: int = 0) -> None:
        """Test hook: admission sees `fake_free_bytes` of free device memory (0 =
        the measured figure); the next `fail_allocations` batches fail as if
        their device allocation had failed."""
        check(lib().bcx_server_inject_faults(self._h, int(fake_free_bytes), int(fail_allocations)),
              "server_inject_faults")

    def drain(self) -> None:
        check(lib().bcx_server_drain(self._h), "server_drain")

    def stats(self) -> dict:
        st = ServerStats()
        check(lib().bcx_server_stats(self._h, C.byref(st)), "server_stats")
        return {f: getattr(st, f) for f, _ in ServerStats._fields_}

    def reset_stats(self) -> None:
        check(lib().bcx_server_reset_stats(self._h), "server_reset_stats")

    def close(self) -> None:
        if self._h:
            lib().bcx_server_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
        return False
