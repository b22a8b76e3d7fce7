"""bcx_scan_noalloc: the scan entry point that allocates nothing.

Some callers cannot call cudaMalloc when they need a scan: an application
whose own pool owns every byte of device memory and forbids libraries from
allocating, or a latency-critical path that must not risk the device
synchronization an allocation can cause.  This entry point keeps its
look-back scratch and its error word in one fixed array inside libbcx, so the
caller passes only input and output.

The tests call it through the C ABI, each case twice in a row (the second
call reuses the array the first one left behind), and compare every result
with the CPU oracle -- integers bit for bit, floats within the FP64-oracle
tolerance of the float scan tests -- and with the allocating bcx_scan.  They
cover every element width, float/double plain and compensated, aligned and
unaligned pointers, one tile and many, the exact per-call limits and one
element past them, and a fresh process in which the no-alloc scan is the first
library call (no library device state is set up, no memory changes hands).
This file is collected last, so a failure here leaves every other test
already run.
"""
import ctypes
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

import oracle
from golden_cases import NP

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TORCH_NP = {"char": np.int8, "uchar": np.uint8, "short": np.int16, "ushort": np.int16, "int": np.int32,
            "uint": np.int32, "long": np.int64, "ulong": np.int64, "float": np.float32, "double": np.float64}
CTYPE = {"char": ctypes.c_int8, "uchar": ctypes.c_uint8, "short": ctypes.c_int16, "ushort": ctypes.c_uint16,
         "int": ctypes.c_int32, "uint": ctypes.c_uint32, "long": ctypes.c_int64, "ulong": ctypes.c_uint64,
         "float": ctypes.c_float, "double": ctypes.c_double}
# Per-call limits of bcx_scan_noalloc, by the carry between tiles.
LIMIT = {"narrow": 1 << 30, "wide": 1 << 28, "comp_double": 1 << 27}


def _lib():
    from compute_gb300 import _lib as L
    return L, L.lib()


def _values(rng, dtype, n):
    if dtype in ("float", "double"):
        return (rng.standard_normal(n) * 1000.0).astype(NP[dtype])
    info = np.iinfo(NP[dtype])
    return rng.integers(info.min, info.max, size=n, endpoint=True, dtype=NP[dtype])


def _check(got, a, dtype, exclusive, init, compensated):
    """Integers bit for bit; floats within the per-prefix bound of the float
    scan tests: (i+1) eps sum|prefix| plain, 4 eps sum|prefix| compensated."""
    if dtype not in ("float", "double"):
        ref = oracle.scan(a, dtype, exclusive=bool(exclusive), init=init)
        assert np.array_equal(got.view(NP[dtype]), ref), f"{dtype} differs from the oracle"
        return
    eps = float(np.finfo(NP[dtype]).eps)
    ref = oracle.prefix_f64(a, dtype, exclusive=bool(exclusive), init=float(init))
    mag = np.cumsum(np.abs(a.astype(np.float64)))
    if exclusive:
        mag = np.concatenate([[abs(init)], abs(init) + mag[:-1]])
    n = a.size
    bound = (4.0 * eps * mag) if compensated else (np.arange(1, n + 1) * eps * mag)
    err = np.abs(got.view(NP[dtype]).astype(np.float64) - ref)
    assert (err <= bound + 1e-30).all(), f"{dtype} max error {err.max()}"


CASES = [("char", 0), ("uchar", 0), ("short", 0), ("ushort", 0), ("int", 0), ("uint", 0), ("long", 0),
         ("ulong", 0), ("float", 0), ("float", 1), ("double", 0), ("double", 1)]


@pytest.mark.parametrize("dtype,compensated", CASES, ids=[f"{d}{'-comp' if c else ''}" for d, c in CASES])
@pytest.mark.parametrize("in_off,out_off", [(0, 0), (1, 1), (1, 0)], ids=["aligned", "same-offset", "mixed"])
def test_scan_noalloc_matches_oracle_twice(cuda, dtype, compensated, in_off, out_off):
    """Many tiles (look-back through the fixed array) and one tile; inclusive
    and exclusive with an init; pointers 16-byte aligned, offset by one element
    alike (the unaligned head), and offset differently (the scalar path)."""
    torch = cuda
    L, lib = _lib()
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(1000 + L.DTYPES[dtype] * 7 + compensated + 3 * in_off + 5 * out_off)
    esz = np.dtype(NP[dtype]).itemsize
    for n, exclusive, init in [(200_003, 1, 7), (200_003, 0, 0), (1000, 1, 3)]:
        a = _values(rng, dtype, n)
        dev_in = torch.from_numpy(np.concatenate([np.zeros(in_off, NP[dtype]), a]).view(TORCH_NP[dtype])).cuda()
        dev_out = torch.empty(n + out_off, dtype=dev_in.dtype, device="cuda")
        dev_ref = torch.empty(n + out_off, dtype=dev_in.dtype, device="cuda")
        pin = dev_in.data_ptr() + in_off * esz
        pout = dev_out.data_ptr() + out_off * esz
        pref = dev_ref.data_ptr() + out_off * esz
        init_v = CTYPE[dtype](init)
        rc = lib.bcx_scan(stream, L.DTYPES[dtype], L.OPS["plus"], exclusive, ctypes.byref(init_v), pin, pref, n,
                          compensated, None, None)
        assert rc == 0, lib.bcx_last_error_string()
        ref = dev_ref[out_off:].cpu().numpy()
        _check(ref, a, dtype, exclusive, init, compensated)
        for _ in range(2):
            dev_out.fill_(0x5A)
            rc = lib.bcx_scan_noalloc(stream, L.DTYPES[dtype], L.OPS["plus"], exclusive, ctypes.byref(init_v),
                                      pin, pout, n, compensated)
            assert rc == 0, lib.bcx_last_error_string()
            got = dev_out[out_off:].cpu().numpy()
            _check(got, a, dtype, exclusive, init, compensated)
            if dtype not in ("float", "double"):
                assert np.array_equal(got, ref), "differs from bcx_scan"
    assert lib.bcx_device_error_check(stream) == 0, lib.bcx_last_error_string()


def test_scan_noalloc_other_functors(cuda):
    """max and bit_xor on int32, min on float, twice each, against the oracle."""
    torch = cuda
    L, lib = _lib()
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(5)
    for dtype, op in [("int", "max"), ("int", "bit_xor"), ("float", "min")]:
        n = 100_001
        a = _values(rng, dtype, n)
        d = torch.from_numpy(a.view(TORCH_NP[dtype])).cuda()
        out = torch.empty_like(d)
        for _ in range(2):
            out.fill_(0)
            rc = lib.bcx_scan_noalloc(stream, L.DTYPES[dtype], L.OPS[op], 0, None, d.data_ptr(), out.data_ptr(),
                                      n, 0)
            assert rc == 0, lib.bcx_last_error_string()
            got = out.cpu().numpy().view(NP[dtype])
            ref = oracle.scan(a, dtype, op=op, exclusive=False)
            assert np.array_equal(got.view(np.uint8), ref.view(np.uint8)), (dtype, op)


def test_scan_noalloc_at_its_limits(cuda):
    """n at the documented limit runs (int32 at 2^30, with both pointers one
    element off 16-byte alignment: the worst case for the array); one element
    more is rejected with BCX_INVALID_BUFFER_SIZE for each carry width.  The
    rejected calls get real buffers of n elements, so nothing could go out of
    bounds even if the size check were missing."""
    torch = cuda
    L, lib = _lib()
    stream = torch.cuda.current_stream().cuda_stream
    n = LIMIT["narrow"]
    a = torch.ones(n + 1, dtype=torch.int32, device="cuda")
    out = torch.empty(n + 1, dtype=torch.int32, device="cuda")
    init_v = ctypes.c_int32(-5)
    rc = lib.bcx_scan_noalloc(stream, L.DTYPES["int"], L.OPS["plus"], 1, ctypes.byref(init_v), a.data_ptr() + 4,
                              out.data_ptr() + 4, n, 0)
    assert rc == 0, lib.bcx_last_error_string()
    expect = torch.arange(n, dtype=torch.int64, device="cuda") - 5
    assert torch.equal(out[1:].to(torch.int64), expect)
    del expect
    rc = lib.bcx_scan_noalloc(stream, L.DTYPES["int"], L.OPS["plus"], 0, None, a.data_ptr(), out.data_ptr(), n + 1, 0)
    assert rc == L.INVALID_BUFFER_SIZE
    assert b"limit" in lib.bcx_last_error_string()
    del a, out
    torch.cuda.empty_cache()
    for dtype, comp, key in [("long", 0, "wide"), ("float", 1, "wide"), ("double", 1, "comp_double")]:
        m = LIMIT[key] + 1
        tdt = torch.int64 if dtype == "long" else (torch.float32 if dtype == "float" else torch.float64)
        a = torch.zeros(m, dtype=tdt, device="cuda")
        out = torch.empty_like(a)
        rc = lib.bcx_scan_noalloc(stream, L.DTYPES[dtype], L.OPS["plus"], 0, None, a.data_ptr(), out.data_ptr(), m,
                                  comp)
        assert rc == L.INVALID_BUFFER_SIZE, (dtype, comp)
        del a, out
        torch.cuda.empty_cache()
    assert lib.bcx_device_error_check(stream) == 0


FRESH = textwrap.dedent(r"""
    import ctypes, sys
    import numpy as np
    import torch
    sys.path.insert(0, sys.argv[1])
    from compute_gb300 import _lib as L
    lib = L.lib()
    torch.cuda.init()
    n = 300_007
    a = torch.randint(-100, 100, (n,), dtype=torch.int32, device="cuda")
    out = torch.empty_like(a)
    ref = torch.cumsum(a.to(torch.int64), 0).to(torch.int32)
    torch.cuda.synchronize()
    cu = ctypes.CDLL("libcuda.so.1")
    dev = ctypes.c_int()
    assert cu.cuDeviceGet(ctypes.byref(dev), torch.cuda.current_device()) == 0
    pool = ctypes.c_void_p()
    assert cu.cuDeviceGetDefaultMemPool(ctypes.byref(pool), dev) == 0

    def threshold():
        v = ctypes.c_uint64()
        assert cu.cuMemPoolGetAttribute(pool, 4, ctypes.byref(v)) == 0  # CU_MEMPOOL_ATTR_RELEASE_THRESHOLD
        return v.value

    t0 = threshold()
    stream = torch.cuda.current_stream().cuda_stream
    free = []
    for _ in range(3):
        out.zero_()
        rc = lib.bcx_scan_noalloc(stream, L.DTYPES["int"], L.OPS["plus"], 0, None, a.data_ptr(), out.data_ptr(),
                                  n, 0)
        assert rc == 0, lib.bcx_last_error_string()
        torch.cuda.synchronize()
        assert torch.equal(out, ref)
        free.append(torch.cuda.mem_get_info()[0])
    assert lib.bcx_device_error_check(stream) == 0
    assert threshold() == t0, "the no-alloc scan set up the library's device state (pool threshold changed)"
    assert free[0] == free[1] == free[2], f"device memory changed between calls: {free}"
    # control: any other entry point sets the device state up, which the
    # check above would have seen
    rc = lib.bcx_scan(stream, L.DTYPES["int"], L.OPS["plus"], 0, None, a.data_ptr(), out.data_ptr(), n, 0,
                      None, None)
    assert rc == 0
    assert threshold() != t0
    print("fresh-process no-alloc ok")
""")


def test_scan_noalloc_first_call_in_fresh_process(cuda):
    """A process whose first libbcx call is the no-alloc scan: three calls in
    a row give the right result, leave the library's per-device state unset
    (the default pool's release threshold, which that state changes, stays as
    it was), and change no free device memory between calls."""
    r = subprocess.run([sys.executable, "-c", FRESH, ROOT], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "fresh-process no-alloc ok" in r.stdout
