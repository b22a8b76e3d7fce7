"""Full-size parity through size-independent properties, at the sizes the
benchmark is quoted on (the oracle covers the same kernels element by element
at smaller sizes):

* sort_by_key of 2^28 uint32 pairs: keys non-decreasing, equal keys keep
  increasing values (stability), values a permutation that maps the input keys
  onto the output keys;
* exclusive / inclusive scan and reduce of 2^30 int32: inclusive - exclusive
  equals the input, the last inclusive element equals the reduction, which
  equals the exact sum modulo 2^32;
* compensated accumulate / inclusive scan of 2^30 float32 N(1000, 1) within
  their stated FP64-reference tolerances;
* the 10,000-segment workload (9.5·10^8 elements): segmented scan restarts at
  every segment start and otherwise differences to its input; segmented
  sort_by_key is sorted and stable inside every segment and keeps every
  segment's key sum."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def bc(cuda):
    import compute_gb300
    return compute_gb300


def test_sort_by_key_2p28_properties(bc, cuda):
    torch = cuda
    n = 1 << 28
    g = torch.Generator(device="cuda").manual_seed(20261203)
    keys = torch.randint(-2**31, 2**31, (n,), dtype=torch.int32, device="cuda", generator=g)
    orig = keys.clone()
    vals = torch.arange(n, dtype=torch.int32, device="cuda")
    bc.sort_by_key(keys, vals, dtype="uint")
    u = keys.to(torch.int64) & 0xFFFFFFFF
    assert bool((u[1:] >= u[:-1]).all())
    eq = u[1:] == u[:-1]
    assert bool((vals[1:][eq] > vals[:-1][eq]).all())
    del u, eq
    assert bool((orig[vals.long()] == keys).all())  # values are the permutation
    assert int(vals.to(torch.int64).sum().item()) == n * (n - 1) // 2
    bc.device_error_check()


def test_scan_reduce_2p30_linearity(bc, cuda):
    torch = cuda
    n = 1 << 30
    g = torch.Generator(device="cuda").manual_seed(1)
    a = torch.randint(0, 100, (n,), dtype=torch.int32, device="cuda", generator=g)
    ex = bc.exclusive_scan(a)
    inc = bc.inclusive_scan(a)
    assert bool((inc - ex == a).all())
    assert int(ex[0].item()) == 0
    del ex
    total = int(bc.reduce(a).item())
    assert int(inc[-1].item()) == total
    exact = int(a.sum(dtype=torch.int64).item()) & 0xFFFFFFFF
    assert total & 0xFFFFFFFF == exact
    bc.device_error_check()


def test_compensated_2p30_float_accuracy(bc, cuda):
    torch = cuda
    n = 1 << 30
    g = torch.Generator(device="cuda").manual_seed(2)
    x = torch.randn(n, dtype=torch.float32, device="cuda", generator=g) + 1000.0
    ref = float(x.double().sum().item())
    got = bc.accumulate(x, 0.0, compensated=True)
    ulp = float(np.spacing(np.float32(ref)))
    assert abs(got - float(np.float32(ref))) <= ulp, (got, ref)  # within 1 ulp of the FP32-rounded sum
    y = bc.inclusive_scan(x, compensated=True)
    pref = torch.cumsum(x.double(), 0)
    rel = ((y.double() - pref).abs() / pref.abs()).max().item()
    assert rel <= 2.0 ** -23, rel  # every prefix within 1 ulp of the FP64 prefix
    bc.device_error_check()


def _segments(torch, nseg=10_000, seed=20261205):
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(16), np.log(1 << 20), size=nseg)).astype(np.int64)
    offsets = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    seg_id = torch.repeat_interleave(torch.arange(nseg, device="cuda"), torch.from_numpy(sizes).cuda())
    return offsets, seg_id


def test_segmented_scan_10000_segments(bc, cuda):
    import ctypes
    from compute_gb300 import _lib
    torch = cuda
    offsets, seg_id = _segments(torch)
    n = int(offsets[-1])
    g = torch.Generator(device="cuda").manual_seed(3)
    x = torch.randint(0, 100, (n,), dtype=torch.int32, device="cuda", generator=g)
    out = torch.empty_like(x)
    offs = torch.from_numpy(offsets).cuda()
    init = np.array([7], dtype=np.int32)
    rc = _lib.lib().bcx_segmented_scan(torch.cuda.current_stream().cuda_stream, _lib.DTYPES["int"], _lib.OPS["plus"],
                                       1, init.ctypes.data_as(ctypes.c_void_p), x.data_ptr(), out.data_ptr(), n,
                                       offs.data_ptr(), offsets.size - 1, 0, None, None)
    assert rc == 0, _lib.lib().bcx_last_error_string()
    start = torch.zeros(n, dtype=torch.bool, device="cuda")
    start[offs[:-1]] = True
    assert bool((out[start] == 7).all())  # every segment restarts at init
    cont = ~start[1:]
    assert bool(((out[1:] - out[:-1])[cont] == x[:-1][cont]).all())
    bc.device_error_check()


def test_segmented_sort_10000_segments(bc, cuda):
    from compute_gb300 import _lib
    torch = cuda
    offsets, seg_id = _segments(torch)
    n = int(offsets[-1])
    g = torch.Generator(device="cuda").manual_seed(4)
    keys = torch.randint(0, 1 << 16, (n,), dtype=torch.int32, device="cuda", generator=g)  # many ties
    vals = torch.arange(n, dtype=torch.int32, device="cuda")
    seg_sum = torch.zeros(offsets.size - 1, dtype=torch.int64, device="cuda").index_add_(0, seg_id, keys.to(torch.int64))
    offs = torch.from_numpy(offsets).cuda()
    rc = _lib.lib().bcx_segmented_sort_pairs(torch.cuda.current_stream().cuda_stream, _lib.DTYPES["uint"], 4,
                                             keys.data_ptr(), vals.data_ptr(), n, offs.data_ptr(), offsets.size - 1, 0,
                                             None, None)
    assert rc == 0, _lib.lib().bcx_last_error_string()
    same_seg = seg_id[1:] == seg_id[:-1]
    assert bool((keys[1:] >= keys[:-1])[same_seg].all())
    tie = same_seg & (keys[1:] == keys[:-1])
    assert bool((vals[1:] > vals[:-1])[tie].all())  # stable inside segments
    assert bool((seg_id[vals.long()] == seg_id).all())  # values stay in their segment
    after = torch.zeros_like(seg_sum).index_add_(0, seg_id, keys.to(torch.int64))
    assert bool((after == seg_sum).all())
    bc.device_error_check()
