"""Failure detection without a GPU fault: every bounded device-side wait of
the library gives up after its poll limit, the kernel returns normally, and the
host learns of it through bcx_device_error_check (BCX_DEVICE_TIMEOUT, then
cleared), with the context still usable for correct work afterwards.

bcx_debug_expire_wait runs the library's own wait routines -- the onesweep
digit look-back, the scan tile look-back and the bulk-copy mbarrier wait --
against a status word or barrier that nothing ever publishes, with a poll
limit of a few hundred polls instead of the production 2^22."""
import ctypes

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("which,word", [(0, 0x1), (1, 0x1), (2, 0x2)],
                         ids=["onesweep-lookback", "scan-lookback", "bulk-copy-wait"])
def test_expired_wait_is_reported_and_cleared(cuda, which, word):
    torch = cuda
    from compute_gb300 import _lib
    lib = _lib.lib()
    stream = torch.cuda.current_stream().cuda_stream
    assert lib.bcx_device_error_check(stream) == 0, lib.bcx_last_error_string()
    assert lib.bcx_debug_expire_wait(stream, which, 500) == 0, lib.bcx_last_error_string()
    rc = lib.bcx_device_error_check(stream)
    assert rc == _lib.DEVICE_TIMEOUT
    assert f"0x{word:x}".encode() in lib.bcx_last_error_string()
    assert lib.bcx_device_error_check(stream) == 0  # cleared by the first check
    # the context still computes correctly
    import compute_gb300 as bc
    rng = np.random.default_rng(which)
    keys = rng.integers(0, 2**32, size=70_001, dtype=np.uint64).astype(np.uint32)
    d = torch.from_numpy(keys.view(np.int32).copy()).cuda()
    bc.sort(d, dtype="uint")
    assert np.array_equal(d.cpu().numpy().view(np.uint32), oracle.sort(keys, "uint"))
    assert lib.bcx_device_error_check(stream) == 0


def test_expire_wait_rejects_bad_arguments(cuda):
    from compute_gb300 import _lib
    lib = _lib.lib()
    assert lib.bcx_debug_expire_wait(None, 3, 10) == _lib.INVALID_VALUE
    assert lib.bcx_debug_expire_wait(None, 0, 0) == _lib.INVALID_VALUE
