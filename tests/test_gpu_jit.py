"""Run-time compiled kernels and their cache (program_cache / offline cache
analogue, the reference's test/test_program_cache.cpp): hits, misses and LRU
eviction of compiled modules, the on-disk cubin cache under BCX_CACHE_DIR, a
build failure with its log, and a compiled kernel's output."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SRC = r'''
extern "C" __global__ void k_fill(int *out, int n, int v) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = v + i * %d;
}
'''


def stats(lib):
    v = [C.c_uint64(0) for _ in range(5)]
    assert lib.bcx_jit_cache_stats(*[C.byref(x) for x in v]) == 0
    return dict(zip(["hits", "misses", "compiles", "disk_hits", "entries"], [x.value for x in v]))


def get(lib, src, name="k_fill"):
    k = C.c_void_p()
    rc = lib.bcx_jit_get_kernel(src.encode(), name.encode(), b"", C.byref(k))
    return rc, k


@pytest.fixture()
def lib(cuda, monkeypatch):
    from compute_gb300 import _lib
    monkeypatch.delenv("BCX_CACHE_DIR", raising=False)
    L = _lib.lib()
    assert L.bcx_jit_cache_configure(2, 1) == 0
    yield L
    L.bcx_jit_cache_configure(256, 1)


def test_lru_hits_misses_and_eviction(lib):
    s0 = stats(lib)
    for m in (1, 2, 3):
        rc, _ = get(lib, SRC % m)
        assert rc == 0
    s1 = stats(lib)
    assert s1["compiles"] - s0["compiles"] == 3 and s1["misses"] - s0["misses"] == 3
    assert s1["entries"] == 2  # capacity 2: the module of multiplier 1 was evicted
    assert get(lib, SRC % 3)[0] == 0
    s2 = stats(lib)
    assert s2["hits"] == s1["hits"] + 1 and s2["compiles"] == s1["compiles"]
    assert get(lib, SRC % 1)[0] == 0  # evicted: compiled again
    assert stats(lib)["compiles"] == s2["compiles"] + 1


def test_compiled_kernel_runs(lib, cuda):
    rc, k = get(lib, SRC % 7)
    assert rc == 0
    n = 1000
    out = cuda.zeros(n, dtype=cuda.int32, device="cuda")
    p, nn, v = C.c_void_p(out.data_ptr()), C.c_int(n), C.c_int(5)
    args = (C.c_void_p * 3)(*[C.cast(C.pointer(x), C.c_void_p) for x in (p, nn, v)])
    stream = cuda.cuda.current_stream().cuda_stream
    assert lib.bcx_jit_launch(k, (n + 127) // 128, 128, 0, stream, args) == 0
    np.testing.assert_array_equal(out.cpu().numpy(), 5 + 7 * np.arange(n, dtype=np.int32))


def test_disk_cache_serves_a_cleared_process_cache(lib, tmp_path, monkeypatch):
    monkeypatch.setenv("BCX_CACHE_DIR", str(tmp_path))
    src = SRC % 11
    assert get(lib, src)[0] == 0
    assert any(tmp_path.rglob("*")), "no cubin written"
    lib.bcx_jit_cache_configure(0, 1)  # drop every loaded module
    s0 = stats(lib)
    assert get(lib, src)[0] == 0
    s1 = stats(lib)
    assert s1["disk_hits"] == s0["disk_hits"] + 1 and s1["compiles"] == s0["compiles"]


def test_build_failure_reports_log(lib):
    rc, _ = get(lib, 'extern "C" __global__ void broken(int *o) { o[0] = ; }', "broken")
    assert rc == -11  # CL_BUILD_PROGRAM_FAILURE
    need = C.c_size_t(0)
    assert lib.bcx_jit_build_log(None, 0, C.byref(need)) == 0 and need.value > 1
    buf = C.create_string_buffer(need.value)
    assert lib.bcx_jit_build_log(buf, need.value, None) == 0
    assert b"error" in buf.value
