"""Parity of the CUDA path (libbcx through its C ABI) with the reference.

Small inputs are compared with the reference's golden vectors and with the CPU
oracle bit for bit; integer/byte/index work must be bit-exact, float sort is
compared as bit patterns (the reference radix order), float sums against the
FP64 oracle with the tolerance written in each test.  Large inputs are checked
through size-independent properties (sortedness, stability, multiset
checksums, scan/reduce consistency).
"""
import numpy as np
import pytest

import oracle
from golden_cases import NP, arr, cases, ids, scalar

pytestmark = pytest.mark.gpu

# numpy type of a torch-supported tensor with the same width as each bcx type
TORCH_NP = {"char": np.int8, "uchar": np.uint8, "short": np.int16, "ushort": np.int16, "int": np.int32,
            "uint": np.int32, "long": np.int64, "ulong": np.int64, "float": np.float32,
            "double": np.float64}


@pytest.fixture(scope="module")
def bc(cuda):
    import compute_gb300
    return compute_gb300


def to_dev(torch, a: np.ndarray, dtype: str):
    """numpy array -> CUDA tensor holding the same bytes (unsigned types ride
    in signed tensors with the same width)."""
    t = torch.from_numpy(np.ascontiguousarray(a, dtype=NP[dtype]).view(TORCH_NP[dtype]).copy())
    return t.cuda()


def to_np(t, dtype: str) -> np.ndarray:
    return t.cpu().numpy().view(NP[dtype])


def bits(a: np.ndarray) -> np.ndarray:
    return a.view({1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}[a.itemsize])


# ---- golden vectors ---------------------------------------------------------
SORT_CASES = cases("radix_sort", "radix_sort_range", "sort", "insertion_sort")


@pytest.mark.parametrize("case", SORT_CASES, ids=ids(SORT_CASES))
def test_sort_golden(bc, cuda, case):
    t = case["dtype"]
    data = arr(case["inputs"][0], t)
    exp = arr(case["expected"][0], t)
    d = to_dev(cuda, data, t)
    desc = case["descending"]
    if case["kind"] == "radix_sort":
        bc.radix_sort(d, descending=desc, dtype=t)
    elif case["kind"] == "radix_sort_range":
        a, b = case["range"]
        bc.radix_sort(d[a:b], descending=desc, dtype=t)
    else:  # public sort dispatch (insertion sort for these sizes)
        bc.sort(d, descending=desc, dtype=t)
    got = to_np(d, t)
    np.testing.assert_array_equal(got, exp)
    # bit patterns must match the oracle (sign of zero included)
    if case["kind"] == "radix_sort":
        ref = oracle.radix_sort(data, t, descending=desc)
    elif case["kind"] == "radix_sort_range":
        ref = data.copy()
        ref[a:b] = oracle.radix_sort(data[a:b], t, descending=desc)
    else:
        ref = oracle.sort(data, t, descending=desc)
    np.testing.assert_array_equal(bits(got), bits(ref))


PAIR_CASES = cases("radix_sort_by_key", "sort_by_key")


@pytest.mark.parametrize("case", PAIR_CASES, ids=ids(PAIR_CASES))
def test_sort_by_key_golden(bc, cuda, case):
    kt, vt = case["dtype"], case["value_dtype"]
    keys = arr(case["inputs"][0], kt)
    vals = arr(case["inputs"][1], vt)
    dk = to_dev(cuda, keys, kt)
    dv = cuda.from_numpy(vals.copy()).cuda()
    if case["kind"] == "radix_sort_by_key":
        bc.radix_sort_by_key(dk, dv, descending=case["descending"], dtype=kt)
    else:
        bc.sort_by_key(dk, dv, descending=case["descending"], dtype=kt)
    np.testing.assert_array_equal(to_np(dk, kt), arr(case["expected"][0], kt))
    np.testing.assert_array_equal(dv.cpu().numpy(), arr(case["expected"][1], vt))


SCAN_CASES = cases("scan")


@pytest.mark.parametrize("case", SCAN_CASES, ids=ids(SCAN_CASES))
@pytest.mark.parametrize("inplace", [False, True])
def test_scan_golden(bc, cuda, case, inplace):
    t = case["dtype"]
    d = to_dev(cuda, arr(case["inputs"][0], t), t)
    out = d if inplace else None
    if case["exclusive"]:
        r = bc.exclusive_scan(d, out=out, init=case.get("init", 0), op=case["op"], dtype=t)
    else:
        r = bc.inclusive_scan(d, out=out, op=case["op"], dtype=t)
    np.testing.assert_array_equal(to_np(r, t), arr(case["expected"][0], t))


FOLD_CASES = cases("fold")


@pytest.mark.parametrize("case", FOLD_CASES, ids=ids(FOLD_CASES))
def test_fold_golden(bc, cuda, case):
    t = case["dtype"]
    d = to_dev(cuda, arr(case["inputs"][0], t), t)
    for chk in case["checks"]:
        if chk["init"] is None:
            got = to_np(bc.reduce(d, op=chk["op"], dtype=t), t)[0]
        else:
            got = NP[t](bc.accumulate(d, scalar(chk["init"], t), op=chk["op"], dtype=t))
        assert got == NP[t](chk["expected"]), (chk, got)


def test_accumulate_iota_golden(bc, cuda):
    (case,) = cases("fold_iota")
    for size, chk in zip(case["sizes"], case["checks"]):
        d = cuda.arange(size, dtype=cuda.int32, device="cuda")
        assert bc.accumulate(d, chk["init"], op=chk["op"]) == chk["expected"]


def test_reduce_empty_writes_nothing(bc, cuda):
    d = cuda.empty(0, dtype=cuda.int16, device="cuda")
    out = cuda.full((1,), 7, dtype=cuda.int16, device="cuda")
    bc.reduce(d, out=out)
    assert out.item() == 7  # test/test_reduce.cpp:42-49 leaves the result untouched


TF_CASES = cases("transform_binary", "transform_unary")


@pytest.mark.parametrize("case", TF_CASES, ids=ids(TF_CASES))
def test_transform_golden(bc, cuda, case):
    t = case["dtype"]
    a = to_dev(cuda, arr(case["inputs"][0], t), t)
    if case["kind"] == "transform_unary":
        r = bc.transform(a, case["op"], out=a, dtype=t)  # in place like the reference test
    else:
        b = to_dev(cuda, arr(case["inputs"][1], t), t)
        r = bc.transform(a, case["op"], other=b, dtype=t)
    np.testing.assert_array_equal(to_np(r, t), arr(case["expected"][0], t))


# ---- random parity vs the oracle ------------------------------------------------
SIZES = [0, 1, 2, 3, 31, 32, 33, 255, 256, 257, 4095, 4096, 4097, 8191, 12289, 65537, 1 << 20]
KEY_TYPES = ["char", "uchar", "short", "ushort", "int", "uint", "long", "ulong", "float", "double"]


def random_keys(rng, dtype, n, special=False):
    if dtype in ("float", "double"):
        a = rng.standard_normal(n).astype(NP[dtype]) * NP[dtype](1000)
        if special and n >= 16:
            sp = np.array([np.nan, -np.nan, np.inf, -np.inf, 0.0, -0.0, 1e-45, -1e-45, 1e-310, -1e-310],
                          dtype=NP[dtype])
            idx = rng.integers(0, n, size=max(n // 20, 10))
            a[idx] = sp[rng.integers(0, sp.size, size=idx.size)]
            # NaNs with payloads and both signs
            nan_idx = rng.integers(0, n, size=max(n // 100, 2))
            w = a.view(bits(a).dtype)
            if dtype == "float":
                w[nan_idx] = (rng.integers(0, 2, size=nan_idx.size, dtype=np.uint32) << 31) | 0x7F800000 | \
                    rng.integers(1, 1 << 22, size=nan_idx.size, dtype=np.uint32)
            else:
                w[nan_idx] = (rng.integers(0, 2, size=nan_idx.size, dtype=np.uint64) << np.uint64(63)) | \
                    np.uint64(0x7FF0000000000000) | rng.integers(1, 1 << 50, size=nan_idx.size, dtype=np.uint64)
        return a
    info = np.iinfo(NP[dtype])
    a = rng.integers(info.min, info.max, size=n, endpoint=True, dtype=NP[dtype])
    if special and n >= 4:
        a[rng.integers(0, n, size=4)] = info.min
        a[rng.integers(0, n, size=4)] = info.max
    return a


@pytest.mark.parametrize("dtype", KEY_TYPES)
@pytest.mark.parametrize("desc", [False, True])
def test_radix_sort_keys_random(bc, cuda, dtype, desc):
    rng = np.random.default_rng(KEY_TYPES.index(dtype) * 2 + int(desc))
    for n in SIZES:
        keys = random_keys(rng, dtype, n, special=True)
        d = to_dev(cuda, keys, dtype)
        bc.radix_sort(d, descending=desc, dtype=dtype)
        ref = oracle.radix_sort(keys, dtype, descending=desc)
        np.testing.assert_array_equal(bits(to_np(d, dtype)), bits(ref), err_msg=f"n={n}")


@pytest.mark.parametrize("dtype", ["int", "uint", "float", "ulong", "double", "short", "uchar"])
@pytest.mark.parametrize("vbytes", [1, 2, 4, 8, 16])
def test_radix_sort_pairs_random_stable(bc, cuda, dtype, vbytes):
    rng = np.random.default_rng(7 + vbytes)
    for n in [0, 1, 33, 4097, 12289, 100_003]:
        # few distinct keys -> long runs of equal keys exercise stability
        keys = random_keys(rng, dtype, n, special=True)
        if n > 10:
            keys[rng.integers(0, n, size=n // 2)] = keys[0]
        vals = rng.integers(0, 256, size=n * vbytes, dtype=np.uint8)
        dk = to_dev(cuda, keys, dtype)
        dv = cuda.from_numpy(vals.copy()).cuda()
        bc.radix_sort_by_key(dk, dv, dtype=dtype)
        rk, rv = oracle.radix_sort(keys, dtype, values=vals.reshape(n, vbytes) if n else vals)
        np.testing.assert_array_equal(bits(to_np(dk, dtype)), bits(rk), err_msg=f"n={n}")
        np.testing.assert_array_equal(dv.cpu().numpy(), np.asarray(rv).reshape(-1), err_msg=f"n={n}")


@pytest.mark.parametrize("dtype", KEY_TYPES)
@pytest.mark.parametrize("desc", [False, True])
def test_public_sort_dispatch_random(bc, cuda, dtype, desc):
    """compute::sort: n <= 32 takes the insertion sort with typed compares (NaN
    placement differs from the radix order there), larger n the radix sort."""
    rng = np.random.default_rng(3)
    for n in [2, 5, 17, 31, 32, 33, 64, 1000]:
        keys = random_keys(rng, dtype, n, special=True)
        d = to_dev(cuda, keys, dtype)
        bc.sort(d, descending=desc, dtype=dtype)
        np.testing.assert_array_equal(bits(to_np(d, dtype)), bits(oracle.sort(keys, dtype, descending=desc)),
                                      err_msg=f"n={n}")
        vals = np.arange(n, dtype=np.int32)
        dk, dv = to_dev(cuda, keys, dtype), cuda.from_numpy(vals.copy()).cuda()
        bc.sort_by_key(dk, dv, descending=desc, dtype=dtype)
        rk, rv = oracle.sort_by_key(keys, vals, dtype, descending=desc)
        np.testing.assert_array_equal(bits(to_np(dk, dtype)), bits(rk), err_msg=f"pairs n={n}")
        np.testing.assert_array_equal(dv.cpu().numpy(), rv, err_msg=f"pairs n={n}")


def test_sort_distributions_u64(bc, cuda):
    """uint64 keys: all-equal, pre-sorted, 8 significant bits, Zipf-like."""
    rng = np.random.default_rng(11)
    n = 300_001
    dists = {
        "equal": np.full(n, 0xDEADBEEFCAFEF00D, dtype=np.uint64),
        "sorted": np.arange(n, dtype=np.uint64),
        "bits8": rng.integers(0, 256, size=n, dtype=np.uint64),
        "zipf": rng.zipf(1.1, size=n).astype(np.uint64),
    }
    for name, keys in dists.items():
        vals = np.arange(n, dtype=np.uint32)
        dk, dv = to_dev(cuda, keys, "ulong"), cuda.from_numpy(vals.copy()).cuda()
        bc.sort_by_key(dk, dv, dtype="ulong")
        rk, rv = oracle.radix_sort(keys, "ulong", values=vals)
        np.testing.assert_array_equal(to_np(dk, "ulong"), rk, err_msg=name)
        np.testing.assert_array_equal(dv.cpu().numpy(), rv, err_msg=name)


SCAN_TYPES = ["char", "uchar", "short", "ushort", "int", "uint", "long", "ulong"]
SCAN_OPS = ["plus", "multiplies", "min", "max", "bit_and", "bit_or", "bit_xor"]


@pytest.mark.parametrize("dtype", SCAN_TYPES)
@pytest.mark.parametrize("op", SCAN_OPS)
def test_scan_integer_random(bc, cuda, dtype, op):
    rng = np.random.default_rng(5)
    for n in [1, 2, 17, 4096, 4097, 16385, 262_147]:
        a = random_keys(rng, dtype, n)
        if op == "multiplies":
            a = rng.integers(1, 4, size=n).astype(NP[dtype])
        d = to_dev(cuda, a, dtype)
        for exclusive in (False, True):
            init = NP[dtype](rng.integers(0, 50))
            r = bc.exclusive_scan(d, init=init, op=op, dtype=dtype) if exclusive else \
                bc.inclusive_scan(d, op=op, dtype=dtype)
            ref = oracle.scan(a, dtype, op=op, exclusive=exclusive, init=init)
            np.testing.assert_array_equal(to_np(r, dtype), ref, err_msg=f"n={n} exclusive={exclusive}")


# Tiles of the aligned (bulk-copy) scan: 64 KB, 96 KB for 8-byte elements.
STAGED_TILE = {"uchar": 65536, "short": 32768, "int": 16384, "long": 12288}


@pytest.mark.parametrize("dtype", list(STAGED_TILE))
def test_scan_staged_ragged_tails(bc, cuda, dtype):
    """Aligned inputs of several tiles whose last tile is whole, one element,
    or a bulk-copied part plus a few trailing elements (under 16 bytes), in
    place and out of place, against the oracle bit for bit."""
    rng = np.random.default_rng(11)
    t = STAGED_TILE[dtype]
    w = np.dtype(NP[dtype]).itemsize
    for n in [2 * t, 2 * t + 1, 3 * t + 1003 * (16 // w) + 3, 5 * t - 1]:
        a = random_keys(rng, dtype, n)
        for exclusive in (False, True):
            d = to_dev(cuda, a, dtype)
            if exclusive:
                bc.exclusive_scan(d, out=d, init=NP[dtype](7), dtype=dtype)
            else:
                bc.inclusive_scan(d, out=d, dtype=dtype)
            ref = oracle.scan(a, dtype, exclusive=exclusive, init=NP[dtype](7))
            np.testing.assert_array_equal(to_np(d, dtype), ref, err_msg=f"n={n} exclusive={exclusive}")
    x = rng.normal(1000.0, 1.0, size=3 * 16384 + 1003 * 4 + 3).astype(np.float32)
    got = to_np(bc.inclusive_scan(to_dev(cuda, x, "float"), compensated=True), "float").astype(np.float64)
    ref = oracle.prefix_f64(x, "float")
    assert (np.abs(got - ref) / np.abs(ref)).max() <= 2.0 ** -23


@pytest.mark.parametrize("offset", [0, 1, 2, 3])
def test_scan_misaligned_and_inplace(bc, cuda, offset):
    rng = np.random.default_rng(offset)
    n = 100_000 + offset
    a = rng.integers(0, 100, size=n + 8).astype(np.int32)
    d = to_dev(cuda, a, "int")
    view = d[offset:offset + n]
    bc.exclusive_scan(view, out=view, init=3)
    ref = oracle.scan(a[offset:offset + n], "int", exclusive=True, init=3)
    got = to_np(d, "int")
    np.testing.assert_array_equal(got[offset:offset + n], ref)
    np.testing.assert_array_equal(got[:offset], a[:offset])  # untouched around the view
    np.testing.assert_array_equal(got[offset + n:], a[offset + n:])
    # input and output with different 16-byte phase
    src = to_dev(cuda, a, "int")
    dst = cuda.zeros(n + 8, dtype=cuda.int32, device="cuda")
    bc.inclusive_scan(src[offset:offset + n], out=dst[(offset + 1) % 4:(offset + 1) % 4 + n])
    np.testing.assert_array_equal(to_np(dst, "int")[(offset + 1) % 4:(offset + 1) % 4 + n],
                                  oracle.scan(a[offset:offset + n], "int"))


@pytest.mark.parametrize("dtype", SCAN_TYPES + ["float", "double"])
@pytest.mark.parametrize("op", ["plus", "multiplies", "min", "max", "bit_xor"])
def test_reduce_random(bc, cuda, dtype, op):
    if op == "bit_xor" and dtype in ("float", "double"):
        pytest.skip("no bitwise functor on floats")
    rng = np.random.default_rng(9)
    for n in [1, 3, 100, 8192, 8193, 1_000_003]:
        a = random_keys(rng, dtype, n)
        if op == "multiplies" and dtype not in ("float", "double"):
            a = rng.integers(1, 6, size=n).astype(NP[dtype])
        if dtype in ("float", "double"):
            if op == "multiplies":
                a = (1.0 + rng.standard_normal(n) * 1e-3).astype(NP[dtype])
            got = float(to_np(bc.reduce(to_dev(cuda, a, dtype), op=op, dtype=dtype), dtype)[0])
            if op in ("min", "max"):
                assert got == float(oracle.fold(a, dtype, op=op))
            elif op == "plus":
                ref = oracle.sum_f64(a, dtype)
                # plain FP32/FP64 tree: |err| <= n * eps * sum|a| (worst-case bound)
                eps = np.finfo(NP[dtype]).eps
                assert abs(got - ref) <= n * eps * float(np.abs(a.astype(np.float64)).sum()) + 1e-30
            continue
        got = to_np(bc.reduce(to_dev(cuda, a, dtype), op=op, dtype=dtype), dtype)[0]
        assert got == oracle.fold(a, dtype, op=op), f"n={n}"


@pytest.mark.parametrize("dtype", ["float", "double"])
@pytest.mark.parametrize("compensated", [False, True])
def test_scan_float_types(bc, cuda, dtype, compensated):
    """float / double scans, plain and compensated, one tile and several
    (bulk-copy tiles: 16384 floats, 12288 doubles), against the FP64 oracle
    prefix.  Tolerance per prefix: the worst-case bound of an arbitrary-order
    sum in the element type, (i+1) * eps * sum|a[0..i]|; compensated sums
    within 4 eps * sum|a[0..i]|."""
    rng = np.random.default_rng(31)
    eps = float(np.finfo(NP[dtype]).eps)
    for n in [100, 3 * 16384 + 5]:
        a = (rng.standard_normal(n) * 1000.0).astype(NP[dtype])
        mag = np.cumsum(np.abs(a.astype(np.float64)))
        bound = (4.0 * eps * mag) if compensated else (np.arange(1, n + 1) * eps * mag)
        got = to_np(bc.inclusive_scan(to_dev(cuda, a, dtype), compensated=compensated, dtype=dtype),
                    dtype).astype(np.float64)
        ref = oracle.prefix_f64(a, dtype)
        assert (np.abs(got - ref) <= bound + 1e-30).all(), f"inclusive n={n}"
        got = to_np(bc.exclusive_scan(to_dev(cuda, a, dtype), init=2.5, compensated=compensated, dtype=dtype),
                    dtype).astype(np.float64)
        ref = oracle.prefix_f64(a, dtype, exclusive=True, init=2.5)
        mag_x = np.concatenate([[2.5], 2.5 + mag[:-1]])
        bound_x = (4.0 * eps * mag_x) if compensated else (np.arange(1, n + 1) * eps * mag_x)
        assert (np.abs(got - ref) <= bound_x + 1e-30).all(), f"exclusive n={n}"


def test_accumulate_float_compensated_accuracy(bc, cuda):
    """float accumulate of N(1000, 1): Neumaier in warps/blocks + FP64 combine
    lands within 1 ulp of the FP32 rounding of the FP64 sum; the reference's
    serial FP32 loop (oracle.fold) is far off."""
    rng = np.random.default_rng(2)
    n = 1 << 24
    a = rng.normal(1000.0, 1.0, size=n).astype(np.float32)
    ref = oracle.sum_f64(a, "float", init=0.0)
    got = bc.accumulate(to_dev(cuda, a, "float"), 0.0, compensated=True)
    ulp = np.spacing(np.float32(ref))
    assert abs(got - np.float32(ref)) <= ulp, (got, ref)
    serial = float(oracle.fold(a, "float", op="plus", init=0.0))
    assert abs(serial - ref) > 100 * ulp  # the plain serial FP32 loop drifts


def test_inclusive_scan_float_compensated(bc, cuda):
    rng = np.random.default_rng(4)
    n = (1 << 22) + 5
    a = rng.normal(1000.0, 1.0, size=n).astype(np.float32)
    ref = oracle.prefix_f64(a, "float")
    got = to_np(bc.inclusive_scan(to_dev(cuda, a, "float"), compensated=True), "float").astype(np.float64)
    rel = np.abs(got - ref) / np.abs(ref)
    # every prefix within 1 ulp (2^-23 relative) of the FP64 prefix
    assert rel.max() <= 2.0 ** -23, rel.max()
    ex = to_np(bc.exclusive_scan(to_dev(cuda, a, "float"), init=5.0, compensated=True), "float")
    refx = oracle.prefix_f64(a, "float", exclusive=True, init=5.0)
    assert (np.abs(ex.astype(np.float64) - refx) <= np.spacing(np.abs(refx).astype(np.float32))).all()


@pytest.mark.parametrize("n", [1, 7, 4096, 1_000_001])
def test_saxpy_bit_exact_fma(bc, cuda, n):
    rng = np.random.default_rng(n)
    x = rng.uniform(-1, 1, size=n).astype(np.float32)
    y = rng.uniform(-1, 1, size=n).astype(np.float32)
    r = bc.saxpy(2.5, to_dev(cuda, x, "float"), to_dev(cuda, y, "float"))
    np.testing.assert_array_equal(bits(to_np(r, "float")), bits(oracle.saxpy(2.5, x, y, fused=True)))


@pytest.mark.parametrize("dtype", ["int", "uint", "long", "char", "float", "double"])
@pytest.mark.parametrize("op", ["plus", "minus", "multiplies", "min", "max"])
def test_transform_binary_random(bc, cuda, dtype, op):
    rng = np.random.default_rng(1)
    for n, off in [(1, 0), (33, 1), (100_003, 3)]:
        a = random_keys(rng, dtype, n + 4)
        b = random_keys(rng, dtype, n + 4)
        da, db = to_dev(cuda, a, dtype), to_dev(cuda, b, dtype)
        r = bc.transform(da[off:off + n], op, other=db[off:off + n], dtype=dtype)
        ref = oracle.transform_binary(a[off:off + n], b[off:off + n], dtype, op)
        np.testing.assert_array_equal(bits(to_np(r, dtype)), bits(ref))


# ---- full-size properties ---------------------------------------------------
def test_sort_by_key_2p26_properties(bc, cuda):
    """Large uniform uint32 pairs (values = iota): output keys sorted, values a
    permutation, equal keys keep increasing values (stability), and the
    key multiset is unchanged (sum and xor checksums)."""
    torch = cuda
    n = 1 << 26
    g = torch.Generator(device="cuda").manual_seed(20261203)
    keys = torch.randint(-2**31, 2**31, (n,), dtype=torch.int32, device="cuda", generator=g)
    vals = torch.arange(n, dtype=torch.int32, device="cuda")
    ksum = keys.to(torch.int64).sum().item()
    bc.sort_by_key(keys, vals, dtype="uint")
    u = keys.to(torch.int64) & 0xFFFFFFFF
    assert bool((u[1:] >= u[:-1]).all())
    eq = u[1:] == u[:-1]
    assert bool((vals[1:][eq] > vals[:-1][eq]).all())
    assert keys.to(torch.int64).sum().item() == ksum
    assert int(vals.to(torch.int64).sum().item()) == n * (n - 1) // 2
    perm_keys = torch.randint(-2**31, 2**31, (n,), dtype=torch.int32, device="cuda",
                              generator=torch.Generator(device="cuda").manual_seed(20261203))
    assert bool((perm_keys[vals.long()] == keys).all())


def test_scan_reduce_2p28_consistency(bc, cuda):
    torch = cuda
    n = 1 << 28
    g = torch.Generator(device="cuda").manual_seed(1)
    a = torch.randint(0, 100, (n,), dtype=torch.int32, device="cuda", generator=g)
    ex = bc.exclusive_scan(a)
    inc = bc.inclusive_scan(a)
    total = int(bc.reduce(a).item())
    exact = int(a.to(torch.int64).sum().item()) & 0xFFFFFFFF
    assert total & 0xFFFFFFFF == exact  # int32 plus wraps modulo 2^32
    assert bool((inc - ex == a).all())
    assert int(inc[-1].item()) == total
    assert int(ex[0].item()) == 0


def test_device_error_word_clean(bc, cuda):
    bc.device_error_check()


# ---- reduce_by_key ----------------------------------------------------------
RBK_CASES = cases("reduce_by_key")


@pytest.mark.parametrize("case", RBK_CASES, ids=ids(RBK_CASES))
def test_reduce_by_key_golden(bc, cuda, case):
    kt, vt = case["dtype"], case["value_dtype"]
    ko, vo = bc.reduce_by_key(to_dev(cuda, arr(case["inputs"][0], kt), kt),
                              to_dev(cuda, arr(case["inputs"][1], vt), vt), op=case["op"])
    np.testing.assert_array_equal(to_np(ko, kt), arr(case["expected"][0], kt))
    np.testing.assert_array_equal(to_np(vo, vt), arr(case["expected"][1], vt))


def test_reduce_by_key_long_vector_golden(bc, cuda):
    # test/test_reduce_by_key.cpp:48-73
    keys = cuda.zeros(1024, dtype=cuda.int32, device="cuda")
    ko, vo = bc.reduce_by_key(keys, cuda.ones(1024, dtype=cuda.int32, device="cuda"))
    assert ko.tolist() == [0] and vo.tolist() == [1024]
    keys[[137, 677, 1001]] = 1
    keys = bc.inclusive_scan(keys)
    ko, vo = bc.reduce_by_key(keys, cuda.ones(1024, dtype=cuda.int32, device="cuda"))
    assert ko.tolist() == [0, 1, 2, 3] and vo.tolist() == [137, 540, 324, 23]


def test_reduce_by_key_empty(bc, cuda):
    ko, vo = bc.reduce_by_key(cuda.empty(0, dtype=cuda.int32, device="cuda"),
                              cuda.empty(0, dtype=cuda.int32, device="cuda"))
    assert ko.numel() == 0 and vo.numel() == 0


@pytest.mark.parametrize("kt,vt,op", [("int", "int", "plus"), ("uint", "long", "plus"), ("int", "int", "min"),
                                      ("long", "int", "max"), ("int", "uint", "multiplies"),
                                      ("float", "int", "plus"), ("ulong", "ulong", "plus")])
def test_reduce_by_key_random(bc, cuda, kt, vt, op):
    rng = np.random.default_rng(17)
    for n, mean_run in [(1, 1), (100, 3), (2049, 1), (70_001, 40), (1_000_003, 5000), (300_000, 1)]:
        runs = np.maximum(1, rng.geometric(1.0 / mean_run, size=n)).cumsum()
        keys = np.searchsorted(runs, np.arange(n), side="right")
        keys = (keys * 7 % 1000).astype(NP[kt])  # adjacent runs may share a key value
        vals = random_keys(rng, vt, n)
        if op == "multiplies":
            vals = rng.integers(1, 3, size=n).astype(NP[vt])
        ko, vo = bc.reduce_by_key(to_dev(cuda, keys, kt), to_dev(cuda, vals, vt), op=op,
                                  key_dtype=kt, value_dtype=vt)
        rk, rv = oracle.reduce_by_key(keys, vals, kt, vt, op=op)
        np.testing.assert_array_equal(to_np(ko, kt), rk, err_msg=f"n={n}")
        np.testing.assert_array_equal(to_np(vo, vt), rv, err_msg=f"n={n}")


def test_reduce_by_key_float_segments(bc, cuda):
    """reduce_by_key float32 N(0,1) with keys = segment ids: each segment sum
    within 2 ulp of its magnitude-scaled FP64 value (compensated pairs)."""
    rng = np.random.default_rng(23)
    sizes = np.exp(rng.uniform(np.log(16), np.log(1 << 14), size=400)).astype(np.int64)
    keys = np.repeat(np.arange(sizes.size, dtype=np.int32), sizes)
    vals = rng.standard_normal(keys.size).astype(np.float32)
    ko, vo = bc.reduce_by_key(to_dev(cuda, keys, "int"), to_dev(cuda, vals, "float"))
    rk, rv = oracle.reduce_by_key(keys, vals, "int", "float")
    np.testing.assert_array_equal(to_np(ko, "int"), rk)
    got = to_np(vo, "float").astype(np.float64)
    bound = np.array([np.abs(vals[keys == i]).sum() for i in range(sizes.size)]) * 2.0 ** -23 * 2
    assert (np.abs(got - rv.astype(np.float64)) <= bound + 1e-30).all()
