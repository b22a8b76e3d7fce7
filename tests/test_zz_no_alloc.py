"""bcx_scan_noalloc: the scan entry point that allocates nothing.

Callers that cannot call cudaMalloc at scan time (an application whose own
pool owns all device memory, or a latency-critical path that must not risk an
allocation's device synchronization) use this variant: its look-back scratch
is a fixed array inside libbcx.  The test calls it through the C ABI twice in
a row -- the second call reuses the array the first one left behind -- and
checks each result against the allocating bcx_scan bit for bit (integer
results are exact).  This file is collected last so that a failure here
leaves every other test already run.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_scan_noalloc_matches_scan_twice(cuda):
    torch = cuda
    from compute_gb300 import _lib
    lib = _lib.lib()
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(99)
    # sizes: many tiles (look-back through the fixed scratch), then a single tile
    for n, exclusive, init in [(3_000_017, 1, 7), (3_000_017, 0, 0), (1000, 1, -3)]:
        a = torch.from_numpy(rng.integers(-1000, 1000, size=n).astype(np.int32)).cuda()
        ref = torch.empty_like(a)
        init_v = ctypes.c_int32(init)
        rc = lib.bcx_scan(stream, _lib.DTYPES["int"], _lib.OPS["plus"], exclusive, ctypes.byref(init_v),
                          a.data_ptr(), ref.data_ptr(), n, 0, None, None)
        assert rc == 0, lib.bcx_last_error_string()
        for _ in range(2):
            out = torch.full_like(a, 12345)
            rc = lib.bcx_scan_noalloc(stream, _lib.DTYPES["int"], _lib.OPS["plus"], exclusive,
                                      ctypes.byref(init_v), a.data_ptr(), out.data_ptr(), n, 0)
            assert rc == 0, lib.bcx_last_error_string()
            torch.cuda.synchronize()
            assert torch.equal(out, ref)
    assert lib.bcx_device_error_check(stream) == 0


def test_scan_noalloc_rejects_sizes_beyond_its_scratch(cuda):
    torch = cuda
    from compute_gb300 import _lib
    lib = _lib.lib()
    n = (1 << 30) + (1 << 26)  # int32: more tiles than the fixed array holds
    # real buffers of n elements, so nothing could go out of bounds even if
    # the size check did not reject the call
    a = torch.empty(n, dtype=torch.int32, device="cuda")
    out = torch.empty_like(a)
    rc = lib.bcx_scan_noalloc(torch.cuda.current_stream().cuda_stream, _lib.DTYPES["int"], _lib.OPS["plus"],
                              0, None, a.data_ptr(), out.data_ptr(), n, 0)
    assert rc == _lib.INVALID_BUFFER_SIZE
    assert b"at most" in lib.bcx_last_error_string()
    del a, out
    torch.cuda.empty_cache()
