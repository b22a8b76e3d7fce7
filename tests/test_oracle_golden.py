"""Pins the CPU oracle to the reference's own known-answer tests (CPU only).

Every golden case extracted from the reference test suite must be reproduced
by the oracle restatement before the oracle is trusted as the checker of the
CUDA path.  Floats are compared as bit patterns where the reference's order
decides them (the radix order of -0.0/+0.0)."""
import numpy as np
import pytest

import oracle
from golden_cases import NP, arr, cases, ids, scalar

SORT_CASES = cases("radix_sort", "radix_sort_range", "sort", "insertion_sort")


@pytest.mark.parametrize("case", SORT_CASES, ids=ids(SORT_CASES))
def test_sort_golden(case):
    t = case["dtype"]
    data = arr(case["inputs"][0], t)
    expected = arr(case["expected"][0], t)
    desc = case["descending"]
    if case["kind"] == "radix_sort":
        got = oracle.radix_sort(data, t, descending=desc)
    elif case["kind"] == "radix_sort_range":
        a, b = case["range"]
        got = data.copy()
        got[a:b] = oracle.radix_sort(data[a:b], t, descending=desc)
    elif case["kind"] == "insertion_sort":
        got = oracle.insertion_sort(data, t, descending=desc)
    else:
        got = oracle.sort(data, t, descending=desc)
    np.testing.assert_array_equal(got, expected)


def test_float_zero_order_is_the_radix_order():
    # radix(): -0.0 sorts before +0.0 ascending AND descending
    # (algorithm/detail/radix_sort.hpp:100-127); bit patterns, not ==.
    data = np.array([0.0, -0.0, 1.0, -1.0], dtype=np.float32)
    asc = oracle.radix_sort(data, "float")
    assert np.signbit(asc[1]) and not np.signbit(asc[2])
    desc = oracle.radix_sort(data, "float", descending=True)
    assert desc.tolist() == [1.0, 0.0, 0.0, -1.0]
    assert np.signbit(desc[1]) and not np.signbit(desc[2])


PAIR_CASES = cases("radix_sort_by_key", "sort_by_key")


@pytest.mark.parametrize("case", PAIR_CASES, ids=ids(PAIR_CASES))
def test_sort_by_key_golden(case):
    kt, vt = case["dtype"], case["value_dtype"]
    keys = arr(case["inputs"][0], kt)
    vals = arr(case["inputs"][1], vt)
    if case["kind"] == "radix_sort_by_key":
        gk, gv = oracle.radix_sort(keys, kt, values=vals, descending=case["descending"])
    else:
        gk, gv = oracle.sort_by_key(keys, vals, kt, descending=case["descending"])
    np.testing.assert_array_equal(gk, arr(case["expected"][0], kt))
    np.testing.assert_array_equal(gv, arr(case["expected"][1], vt))


SCAN_CASES = cases("scan")


@pytest.mark.parametrize("case", SCAN_CASES, ids=ids(SCAN_CASES))
def test_scan_golden(case):
    t = case["dtype"]
    got = oracle.scan(arr(case["inputs"][0], t), t, op=case["op"], exclusive=case["exclusive"],
                      init=case.get("init", 0))
    np.testing.assert_array_equal(got, arr(case["expected"][0], t))


def test_scan_multiplies_long_vector():
    # test/test_scan.cpp:392-436: 1000 twos, multiplies (init 10 for exclusive),
    # compared with std::partial_sum in int arithmetic (wraps to 0).
    twos = np.full(1000, 2, dtype=np.int32)
    ref = np.ones(1000, dtype=np.int64)
    acc = 1
    for i in range(1000):
        acc = (acc * 2) & 0xFFFFFFFF
        ref[i] = acc
    np.testing.assert_array_equal(oracle.scan(twos, "int", op="multiplies"), ref.astype(np.uint32).view(np.int32))
    ex = oracle.scan(twos, "int", op="multiplies", exclusive=True, init=10)
    acc = 10
    exp = []
    for i in range(1000):
        exp.append(acc)
        acc = (acc * 2) & 0xFFFFFFFF
    np.testing.assert_array_equal(ex, np.array(exp, dtype=np.uint32).view(np.int32))


FOLD_CASES = cases("fold")


@pytest.mark.parametrize("case", FOLD_CASES, ids=ids(FOLD_CASES))
def test_fold_golden(case):
    t = case["dtype"]
    data = arr(case["inputs"][0], t)
    for chk in case["checks"]:
        init = None if chk["init"] is None else scalar(chk["init"], t)
        got = oracle.fold(data, t, op=chk["op"], init=init)
        assert got == NP[t](chk["expected"]), (chk, got)


def test_fold_iota_golden():
    (case,) = cases("fold_iota")
    for size, chk in zip(case["sizes"], case["checks"]):
        data = np.arange(size, dtype=np.int32)
        assert oracle.fold(data, "int", op=chk["op"], init=chk["init"]) == chk["expected"]


RBK_CASES = cases("reduce_by_key")


@pytest.mark.parametrize("case", RBK_CASES, ids=ids(RBK_CASES))
def test_reduce_by_key_golden(case):
    kt, vt = case["dtype"], case["value_dtype"]
    ko, vo = oracle.reduce_by_key(arr(case["inputs"][0], kt), arr(case["inputs"][1], vt), kt, vt, op=case["op"])
    np.testing.assert_array_equal(ko, arr(case["expected"][0], kt))
    np.testing.assert_array_equal(vo, arr(case["expected"][1], vt))


def test_reduce_by_key_long_vector():
    # test/test_reduce_by_key.cpp:48-73: keys 0..3 after an inclusive scan of
    # flags at 137/677/1001 -> sums (137, 540, 324, 23).
    flags = np.zeros(1024, dtype=np.int32)
    flags[[137, 677, 1001]] = 1
    keys = oracle.scan(flags, "int")
    ko, vo = oracle.reduce_by_key(keys, np.ones(1024, dtype=np.int32), "int", "int")
    assert ko.tolist() == [0, 1, 2, 3] and vo.tolist() == [137, 540, 324, 23]


TF_CASES = cases("transform_binary")


@pytest.mark.parametrize("case", TF_CASES, ids=ids(TF_CASES))
def test_transform_binary_golden(case):
    t = case["dtype"]
    got = oracle.transform_binary(arr(case["inputs"][0], t), arr(case["inputs"][1], t), t, case["op"])
    np.testing.assert_array_equal(got, arr(case["expected"][0], t))


def test_stable_sort_mid_golden():
    # test/test_stable_sort_by_key.cpp:165-204: three keys of -256 with values
    # 3, 1, 2 must come first and keep that order.
    keys = -np.arange(128, dtype=np.int32)
    vals = -np.arange(128, dtype=np.int32)
    keys[[64, 126, 127]] = -256
    vals[[64, 126, 127]] = [3, 1, 2]
    k, v = oracle.sort_by_key(keys, vals, "int")
    assert k[:3].tolist() == [-256] * 3 and v[:3].tolist() == [3, 1, 2]


def test_radix_key_matches_stated_total_order():
    # ascending float order = IEEE totalOrder on the bit patterns
    vals = np.array([np.nan, -np.inf, -1.0, -1e-45, -0.0, 0.0, 1e-45, 1.0, np.inf], dtype=np.float32)
    neg_nan = np.array([0xFFC00000], dtype=np.uint32).view(np.float32)
    data = np.concatenate([vals, neg_nan])
    k = oracle.radix_sort(data, "float")
    bits = k.view(np.uint32)
    assert bits[0] == 0xFFC00000  # -NaN first
    assert np.isnan(k[-1]) and not np.signbit(k[-1])  # +NaN last


def test_cpu_baseline_algorithms_agree_with_oracle():
    rng = np.random.default_rng(1)
    keys = rng.integers(0, 2**32, size=50_000, dtype=np.uint64).astype(np.uint32)
    vals = np.arange(keys.size, dtype=np.uint32)
    ek, ev = oracle.radix_sort(keys, "uint", values=vals)
    k2, v2 = keys.copy(), vals.copy()
    oracle.cpu_merge_sort_by_key_u32(k2, v2, threads=4)
    np.testing.assert_array_equal(k2, ek)
    np.testing.assert_array_equal(v2, ev)
    a = rng.integers(0, 100, size=100_001).astype(np.int32)
    out = np.empty_like(a)
    oracle.cpu_exclusive_scan_i32(a, out, threads=3)
    np.testing.assert_array_equal(out, oracle.scan(a, "int", exclusive=True))
    assert oracle.cpu_reduce_i32(a, threads=5) == oracle.fold(a, "int")
