"""Bit-for-bit parity with the oracle at the sizes of the benchmark
configurations (the smaller oracle tests in test_gpu_parity.py cover every
type and functor; these pin the configurations themselves):

* the README example: compute::sort of 2^20 float32 values, each a uniform
  integer in [0, 2^31 - 1] cast to float -- equal to the oracle's sort;
* float32 sort of 2^27 keys mixing 1 % NaN of both signs with random
  payloads, +-0.0, denormals and +-inf among U(-1e6, 1e6) values -- every bit
  pattern in the oracle's (the reference radix) order;
* uint64 sorts of 2^27 keys: Zipf(1.1), all equal, presorted and 8
  significant bits -- equal to the oracle;
* sort_by_key of 2^28 uint32 keys with iota values -- keys and values equal to
  the oracle's stable sort;
* sort_by_key of 2^30 + 5 uint32 pairs (beyond the 30-bit counts an earlier
  status-word layout was limited to) -- sorted, stable and a permutation.

Inputs are seeded synthetic data with the configurations' shapes and value
distributions; the oracle (a stable sort by the reference's radix() key)
runs on the host in seconds to a minute at these sizes.
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def bc(cuda):
    import compute_gb300
    return compute_gb300


def _bits(torch_tensor, np_type):
    return torch_tensor.cpu().numpy().view(np_type)


def test_readme_float_sort_2p20_equals_oracle(bc, cuda):
    torch = cuda
    rng = np.random.default_rng(20261203)
    n = 1 << 20
    keys = rng.integers(0, 2**31 - 1, size=n, endpoint=True).astype(np.float32)
    d = torch.from_numpy(keys.copy()).cuda()
    bc.sort(d, dtype="float")
    ref = oracle.sort(keys, "float")
    np.testing.assert_array_equal(_bits(d, np.uint32), ref.view(np.uint32))


def _f32_specials(rng, n):
    v = rng.uniform(-1e6, 1e6, size=n).astype(np.float32)
    r = rng.random(n)
    bits = v.view(np.uint32)
    nan = r < 0.01
    payload = rng.integers(1, 1 << 22, size=int(nan.sum()), dtype=np.uint32)
    sign = rng.integers(0, 2, size=int(nan.sum()), dtype=np.uint32) << 31
    bits[nan] = sign | np.uint32(0x7F800000) | np.uint32(1 << 22) * rng.integers(0, 2, size=int(nan.sum()),
                                                                                  dtype=np.uint32) | payload
    bits[(r >= 0.01) & (r < 0.02)] = 0x00000000  # +0.0
    bits[(r >= 0.02) & (r < 0.03)] = 0x80000000  # -0.0
    den = (r >= 0.03) & (r < 0.05)
    bits[den] = rng.integers(1, 1 << 23, size=int(den.sum()), dtype=np.uint32) | \
        (rng.integers(0, 2, size=int(den.sum()), dtype=np.uint32) << 31)
    bits[(r >= 0.05) & (r < 0.055)] = 0x7F800000  # +inf
    bits[(r >= 0.055) & (r < 0.06)] = 0xFF800000  # -inf
    return v


@pytest.mark.parametrize("desc", [False, True])
def test_float_sort_2p27_specials_bits(bc, cuda, desc):
    torch = cuda
    rng = np.random.default_rng(20261206 + int(desc))
    n = 1 << 27
    keys = _f32_specials(rng, n)
    assert np.isnan(keys).sum() > n // 200
    d = torch.from_numpy(keys.view(np.int32).copy()).cuda()
    bc.sort(d, descending=desc, dtype="float")
    got = _bits(d, np.uint32)
    del d
    ref = oracle.sort(keys, "float", descending=desc)
    np.testing.assert_array_equal(got, ref.view(np.uint32))


def _u64(kind, rng, n):
    if kind == "zipf":
        return rng.zipf(1.1, size=n).astype(np.uint64)
    if kind == "equal":
        return np.full(n, 0x123456789, dtype=np.uint64)
    if kind == "sorted":
        return np.arange(n, dtype=np.uint64) * np.uint64(3)
    return rng.integers(0, 256, size=n, dtype=np.uint64)


@pytest.mark.parametrize("kind", ["zipf", "equal", "sorted", "8bit"])
def test_u64_sort_2p27_distributions(bc, cuda, kind):
    torch = cuda
    rng = np.random.default_rng(20261207)
    n = 1 << 27
    keys = _u64(kind, rng, n)
    d = torch.from_numpy(keys.view(np.int64).copy()).cuda()
    bc.sort(d, dtype="ulong")
    got = _bits(d, np.uint64)
    del d
    ref = oracle.sort(keys, "ulong")
    np.testing.assert_array_equal(got, ref)


def test_sort_by_key_2p28_equals_oracle(bc, cuda):
    torch = cuda
    rng = np.random.default_rng(20261203)
    n = 1 << 28
    keys = rng.integers(0, 2**32, size=n, dtype=np.uint32)
    vals = np.arange(n, dtype=np.uint32)
    dk = torch.from_numpy(keys.view(np.int32).copy()).cuda()
    dv = torch.from_numpy(vals.view(np.int32).copy()).cuda()
    bc.sort_by_key(dk, dv, dtype="uint")
    gk, gv = _bits(dk, np.uint32), _bits(dv, np.uint32)
    del dk, dv
    rk, rv = oracle.sort_by_key(keys, vals, "uint")
    np.testing.assert_array_equal(gk, rk)
    np.testing.assert_array_equal(gv, rv)


def test_sort_by_key_beyond_2p30_properties(bc, cuda):
    torch = cuda
    n = (1 << 30) + 5
    g = torch.Generator(device="cuda").manual_seed(77)
    keys = torch.randint(-2**31, 2**31, (n,), dtype=torch.int32, device="cuda", generator=g)
    keys[: n // 4] = 12345  # a quarter of equal keys: stability across > 2^30 elements
    orig = keys.clone()
    vals = torch.arange(n, dtype=torch.int32, device="cuda")
    bc.sort_by_key(keys, vals, dtype="uint")
    bc.device_error_check()
    u = keys.to(torch.int64) & 0xFFFFFFFF
    assert bool((u[1:] >= u[:-1]).all())
    eq = u[1:] == u[:-1]
    del u
    assert bool((vals[1:][eq] > vals[:-1][eq]).all())
    del eq
    assert bool((orig[vals.long()] == keys).all())
    assert int(vals.to(torch.int64).sum().item()) == n * (n - 1) // 2
