"""Segmented scan / reduce (one launch each) against per-segment oracle calls.

Segments are CSR offsets; the equivalent reference code is one plain call
per segment, so each segment's result must equal the oracle on that slice
(bit-exact for integers, FP64-oracle tolerance for compensated floats)."""
import ctypes

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

NP = {"int": np.int32, "uint": np.uint32, "long": np.int64, "ulong": np.uint64, "float": np.float32,
      "double": np.float64}
TORCH_NP = {"int": np.int32, "uint": np.int32, "long": np.int64, "ulong": np.int64, "float": np.float32,
            "double": np.float64, "uchar": np.uint8}


def log_uniform_offsets(rng, nseg, lo, hi, empty_frac=0.0):
    sizes = np.exp(rng.uniform(np.log(lo), np.log(hi), size=nseg)).astype(np.int64)
    if empty_frac:
        sizes[rng.random(nseg) < empty_frac] = 0
    return np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)


def run_seg_scan(torch, x, dtype, op, exclusive, init, offsets):
    from compute_gb300 import _lib
    lib = _lib.lib()
    d = torch.from_numpy(x.view(TORCH_NP[dtype]).copy()).cuda()
    out = torch.empty_like(d)
    offs = torch.from_numpy(offsets.view(np.int64).copy()).cuda()
    init_b = np.array([init], dtype=NP[dtype])
    rc = lib.bcx_segmented_scan(torch.cuda.current_stream().cuda_stream, _lib.DTYPES[dtype], _lib.OPS[op],
                                int(exclusive), init_b.ctypes.data_as(ctypes.c_void_p), d.data_ptr(),
                                out.data_ptr(), x.size, offs.data_ptr(), offsets.size - 1, 1, None, None)
    assert rc == 0, lib.bcx_last_error_string()
    return out.cpu().numpy().view(NP[dtype])


@pytest.mark.parametrize("dtype", ["int", "uint", "long", "float"])
@pytest.mark.parametrize("op", ["plus", "max"])
@pytest.mark.parametrize("exclusive", [False, True])
def test_segmented_scan_matches_per_segment(cuda, dtype, op, exclusive):
    rng = np.random.default_rng(3)
    offsets = log_uniform_offsets(rng, 700, 1, 20000, empty_frac=0.05)
    n = int(offsets[-1])
    if dtype == "float":
        x = rng.integers(-100, 100, size=n).astype(np.float32)  # exact in FP32: order does not matter
    else:
        x = rng.integers(0, 1000, size=n).astype(NP[dtype])
    init = 5
    got = run_seg_scan(cuda, x, dtype, op, exclusive, init, offsets)
    for s in range(offsets.size - 1):
        a, b = int(offsets[s]), int(offsets[s + 1])
        if a == b:
            continue
        ref = oracle.scan(x[a:b], dtype, op=op, exclusive=exclusive, init=init)
        np.testing.assert_array_equal(got[a:b], ref, err_msg=f"segment {s} [{a},{b})")


def test_segmented_scan_float_compensated_accuracy(cuda):
    rng = np.random.default_rng(8)
    offsets = log_uniform_offsets(rng, 60, 16, 1 << 18)
    n = int(offsets[-1])
    x = rng.standard_normal(n).astype(np.float32)
    got = run_seg_scan(cuda, x, "float", "plus", False, 0, offsets).astype(np.float64)
    for s in range(offsets.size - 1):
        a, b = int(offsets[s]), int(offsets[s + 1])
        ref = oracle.prefix_f64(x[a:b], "float")
        bound = np.cumsum(np.abs(x[a:b]).astype(np.float64)) * 2.0 ** -23 * 2 + 1e-30
        assert (np.abs(got[a:b] - ref) <= bound).all(), s


@pytest.mark.parametrize("dtype", ["int", "ulong", "float", "double"])
@pytest.mark.parametrize("op", ["plus", "min"])
def test_segmented_reduce_matches_per_segment(cuda, dtype, op):
    from compute_gb300 import _lib
    lib = _lib.lib()
    torch = cuda
    rng = np.random.default_rng(4)
    offsets = log_uniform_offsets(rng, 2000, 1, 1 << 16, empty_frac=0.02)
    n = int(offsets[-1])
    x = rng.integers(-1000, 1000, size=n).astype(NP[dtype]) if dtype not in ("ulong",) else \
        rng.integers(0, 1000, size=n).astype(np.uint64)
    d = torch.from_numpy(x.view(TORCH_NP[dtype]).copy()).cuda()
    offs = torch.from_numpy(offsets.view(np.int64).copy()).cuda()
    out = torch.empty(offsets.size - 1, dtype=d.dtype, device="cuda")
    init = np.array([7 if op == "plus" else 10**6], dtype=NP[dtype])
    rc = lib.bcx_segmented_reduce(torch.cuda.current_stream().cuda_stream, _lib.DTYPES[dtype], _lib.OPS[op],
                                  d.data_ptr(), offs.data_ptr(), offsets.size - 1,
                                  init.ctypes.data_as(ctypes.c_void_p), out.data_ptr(), 1, None, None)
    assert rc == 0, lib.bcx_last_error_string()
    got = out.cpu().numpy().view(NP[dtype])
    for s in range(offsets.size - 1):
        a, b = int(offsets[s]), int(offsets[s + 1])
        ref = oracle.fold(x[a:b], dtype, op=op, init=init[0])
        if dtype in ("float", "double") and op == "plus":
            assert got[s] == NP[dtype](oracle.sum_f64(x[a:b], dtype, init=float(init[0]))), s
        else:
            assert got[s] == ref, (s, got[s], ref)


def run_seg_sort(torch, keys, vals, kt, offsets, descending=False):
    from compute_gb300 import _lib
    lib = _lib.lib()
    dk = torch.from_numpy(keys.view(TORCH_NP.get(kt, keys.dtype)).copy()).cuda()
    dv = torch.from_numpy(vals.copy()).cuda() if vals is not None else None
    offs = torch.from_numpy(offsets.view(np.int64).copy()).cuda()
    vb = vals.dtype.itemsize if vals is not None else 0
    rc = lib.bcx_segmented_sort_pairs(torch.cuda.current_stream().cuda_stream, _lib.DTYPES[kt], vb, dk.data_ptr(),
                                      dv.data_ptr() if dv is not None else None, keys.size, offs.data_ptr(),
                                      offsets.size - 1, int(descending), None, None)
    assert rc == 0, lib.bcx_last_error_string()
    assert lib.bcx_device_error_check(torch.cuda.current_stream().cuda_stream) == 0
    return dk.cpu().numpy().view(keys.dtype), (dv.cpu().numpy() if dv is not None else None)


@pytest.mark.parametrize("kt", ["uint", "int", "float", "ulong"])
@pytest.mark.parametrize("descending", [False, True])
def test_segmented_sort_pairs_matches_per_segment(cuda, kt, descending):
    rng = np.random.default_rng(11)
    # log-uniform sizes from 1 to 3e5: both the shared-memory and the onesweep paths
    offsets = log_uniform_offsets(rng, 300, 1, 300_000, empty_frac=0.03)
    n = int(offsets[-1])
    if kt == "float":
        keys = (rng.standard_normal(n) * 100).astype(np.float32)
        keys[rng.integers(0, n, size=n // 50)] = -0.0
    elif kt == "ulong":
        keys = rng.integers(0, 2**63, size=n, dtype=np.int64).astype(np.uint64) * 2
    else:
        keys = rng.integers(0, 1 << 20, size=n).astype(NP[kt])  # many equal keys: stability matters
    vals = np.arange(n, dtype=np.uint32)
    gk, gv = run_seg_sort(cuda, keys, vals, kt, offsets, descending)
    for s in range(offsets.size - 1):
        a, b = int(offsets[s]), int(offsets[s + 1])
        rk, rv = oracle.radix_sort(keys[a:b], kt, values=vals[a:b], descending=descending)
        np.testing.assert_array_equal(gk[a:b].view(np.uint8), rk.view(np.uint8), err_msg=f"keys seg {s} [{a},{b})")
        np.testing.assert_array_equal(gv[a:b], rv, err_msg=f"values seg {s} [{a},{b})")


def test_segmented_sort_keys_only_and_8bit(cuda):
    rng = np.random.default_rng(12)
    offsets = log_uniform_offsets(rng, 80, 1, 50_000)
    n = int(offsets[-1])
    keys = rng.integers(0, 256, size=n).astype(np.uint8)
    gk, _ = run_seg_sort(cuda, keys, None, "uchar", offsets)
    for s in range(offsets.size - 1):
        a, b = int(offsets[s]), int(offsets[s + 1])
        np.testing.assert_array_equal(gk[a:b], np.sort(keys[a:b], kind="stable"))


def _set_param(obj, param, value):
    from compute_gb300 import _lib
    assert _lib.lib().bcx_param_set(obj.encode(), param.encode(), value) == 0


@pytest.mark.parametrize("tile", [1024, 2048, 4096])
@pytest.mark.parametrize("per_sm", [0, 1, 8])
def test_segmented_sort_every_small_tile(cuda, tile, per_sm):
    """Every compiled shared-memory tile and grid the autotuner may choose gives
    the same stable per-segment order (segments straddle each tile size)."""
    rng = np.random.default_rng(tile + per_sm)
    offsets = log_uniform_offsets(rng, 400, 1, 12_000)
    n = int(offsets[-1])
    keys = rng.integers(0, 1 << 12, size=n).astype(np.uint32)
    vals = np.arange(n, dtype=np.uint32)
    _set_param("segmented_sort_k32_v4", "small_tile", tile)
    _set_param("segmented_sort_k32_v4", "small_blocks_per_sm", per_sm)
    try:
        gk, gv = run_seg_sort(cuda, keys, vals, "uint", offsets)
    finally:
        from compute_gb300 import _lib
        _lib.lib().bcx_param_clear()
    for s in range(offsets.size - 1):
        a, b = int(offsets[s]), int(offsets[s + 1])
        rk, rv = oracle.radix_sort(keys[a:b], "uint", values=vals[a:b])
        np.testing.assert_array_equal(gk[a:b], rk, err_msg=f"keys seg {s}")
        np.testing.assert_array_equal(gv[a:b], rv, err_msg=f"values seg {s}")


@pytest.mark.parametrize("dtype,items", [("int", 32), ("int", 64), ("long", 8), ("long", 16), ("float", 64)])
def test_segmented_scan_every_tile(cuda, dtype, items):
    rng = np.random.default_rng(items)
    offsets = log_uniform_offsets(rng, 500, 1, 30_000, empty_frac=0.05)
    n = int(offsets[-1])
    x = rng.integers(-100, 100, size=n).astype(NP[dtype])
    _set_param(f"segmented_scan_{dtype}", "items_per_thread", items)
    try:
        got = run_seg_scan(cuda, x, dtype, "plus", True, 3, offsets)
    finally:
        from compute_gb300 import _lib
        _lib.lib().bcx_param_clear()
    for s in range(offsets.size - 1):
        a, b = int(offsets[s]), int(offsets[s + 1])
        if a < b:
            np.testing.assert_array_equal(got[a:b], oracle.scan(x[a:b], dtype, exclusive=True, init=3))


def test_autotuner_records_fastest(cuda, tmp_path, monkeypatch):
    """The tuners time each candidate, store one of them and write the table."""
    from compute_gb300 import _lib
    lib = _lib.lib()
    monkeypatch.setenv("BCX_CACHE_DIR", str(tmp_path))
    lib.bcx_param_clear()
    rng = np.random.default_rng(5)
    offsets = log_uniform_offsets(rng, 2000, 16, 1 << 14)
    n = int(offsets[-1])
    keys = cuda.randint(0, 2**31 - 1, (n,), dtype=cuda.int32, device="cuda")
    before = keys.clone()
    vals = cuda.arange(n, dtype=cuda.int32, device="cuda")
    offs = cuda.from_numpy(offsets.view(np.int64).copy()).cuda()
    s = cuda.cuda.current_stream().cuda_stream
    buf = ctypes.create_string_buffer(8192)
    try:
        rc = lib.bcx_tune_segmented_sort_pairs(s, _lib.DTYPES["uint"], 4, keys.data_ptr(), vals.data_ptr(), n,
                                               offs.data_ptr(), offsets.size - 1, buf, len(buf))
        assert rc == 0, lib.bcx_last_error_string()
        report = buf.value.decode()
        assert "segmented_sort_k32_v4.small_tile=1024" in report and "-> " in report
        rc = lib.bcx_tune_segmented_scan(s, _lib.DTYPES["int"], keys.data_ptr(), n, offs.data_ptr(),
                                         offsets.size - 1, buf, len(buf))
        assert rc == 0, lib.bcx_last_error_string()
        rc = lib.bcx_tune_segmented_reduce(s, _lib.DTYPES["int"], keys.data_ptr(), offs.data_ptr(),
                                           offsets.size - 1, buf, len(buf))
        assert rc == 0, lib.bcx_last_error_string()
        assert cuda.equal(keys, before)  # trial runs worked on copies
        files = list((tmp_path / "tune").glob("*.json"))
        assert len(files) == 1
        text = files[0].read_text()
        for key in ("segmented_sort_k32_v4", "small_tile", "segmented_scan_int", "segmented_reduce_int"):
            assert key in text
        v = ctypes.c_uint(0)
        lib.bcx_param_clear()  # re-read from the file
        assert lib.bcx_param_get(b"segmented_sort_k32_v4", b"small_tile", 7, ctypes.byref(v)) == 0
        assert v.value in (1024, 2048, 4096)
    finally:
        monkeypatch.delenv("BCX_CACHE_DIR")
        lib.bcx_param_clear()
