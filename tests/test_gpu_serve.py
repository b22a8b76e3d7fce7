"""Continuous-batching server: every request's result is the same alone and in
the mix (integers bit-exact, float scan/sum within the FP64-oracle tolerance),
and small requests really are batched while larger ones overlap."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

NP = {"int": np.int32, "uint": np.uint32, "float": np.float32, "ulong": np.uint64}


def make_requests(rng, count):
    reqs = []
    for i in range(count):
        kind = rng.choice(["sort_by_key", "exclusive_scan", "reduce"], p=[0.5, 0.3, 0.2])
        dtype = rng.choice(["int", "uint", "float", "ulong"])
        n = int(np.exp(rng.uniform(np.log(1 << 6), np.log(1 << 20))))
        if dtype == "float":
            keys = rng.standard_normal(n).astype(np.float32)
        elif dtype == "ulong":
            keys = rng.integers(0, 2**63, size=n, dtype=np.int64).astype(np.uint64)
        else:
            keys = rng.integers(-2**31 if dtype == "int" else 0, 2**31, size=n).astype(NP[dtype])
        reqs.append((kind, dtype, keys))
    return reqs


def test_server_results_match_alone(cuda):
    from compute_gb300.serve import Server
    rng = np.random.default_rng(2026)
    reqs = make_requests(rng, 240)
    with Server(slots=8) as srv:
        tickets = []
        bufs = []
        for kind, dtype, keys in reqs:
            k = keys.copy()
            v = np.arange(k.size, dtype=np.uint32) if kind == "sort_by_key" else None
            out = None
            if kind == "exclusive_scan":
                out = np.empty_like(k)
            elif kind == "reduce":
                out = np.zeros(1, dtype=k.dtype)
            bufs.append((k, v, out))
            tickets.append(srv.submit(kind, dtype, k, values=v, out=out))
        lat = [srv.wait(t, timeout=120) for t in tickets]
        st = srv.stats()
    assert st["completed"] == len(reqs)
    assert st["batched_requests"] > 0, st  # small requests were packed into shared launches
    assert all(x >= 0 for x in lat)
    for (kind, dtype, keys), (k, v, out) in zip(reqs, bufs):
        if kind == "sort_by_key":
            rk, rv = oracle.radix_sort(keys, dtype, values=np.arange(keys.size, dtype=np.uint32))
            assert np.array_equal(k.view(np.uint8), rk.view(np.uint8))
            assert np.array_equal(v, rv)
        elif kind == "exclusive_scan":
            if dtype == "float":
                ref = oracle.prefix_f64(keys, "float", exclusive=True)
                bound = np.concatenate([[0.0], np.cumsum(np.abs(keys.astype(np.float64)))[:-1]]) * 2.0 ** -22 + 1e-30
                assert (np.abs(out.astype(np.float64) - ref) <= bound).all()
            else:
                assert np.array_equal(out, oracle.scan(keys, dtype, exclusive=True))
        else:
            if dtype == "float":
                ref = oracle.sum_f64(keys, "float")
                assert abs(float(out[0]) - ref) <= float(np.abs(keys.astype(np.float64)).sum()) * 2.0 ** -22 + 1e-30
            else:
                assert out[0] == oracle.fold(keys, dtype)


@pytest.mark.parametrize("small_limit", [None, 0], ids=["batched", "direct"])
def test_server_device_resident_out_of_place(cuda, small_limit):
    """Device buffers, sorts written out of place: inputs are left untouched and
    several requests may read the same input buffer.  Batched requests move
    through one gather and one scatter launch; with small_limit=0 every
    request computes directly on its own buffers."""
    import torch
    from compute_gb300.serve import Server
    rng = np.random.default_rng(7)
    shared = rng.integers(0, 2**32, size=1 << 16, dtype=np.uint64).astype(np.uint32)
    dk = torch.from_numpy(shared.view(np.int32)).to("cuda")
    dv = torch.arange(shared.size, dtype=torch.int32, device="cuda")
    outs = []
    red = torch.zeros(1, dtype=torch.int64, device="cuda")
    with Server(slots=4, small_limit=small_limit) as srv:
        tickets = []
        for i in range(24):
            n = int(rng.integers(1, shared.size + 1))
            ok = torch.empty(n, dtype=torch.int32, device="cuda")
            ov = torch.empty(n, dtype=torch.int32, device="cuda")
            tickets.append(srv.submit("sort_by_key", "uint", dk, values=dv, out=ok, out_values=ov, n=n,
                                      device=True))
            outs.append((n, ok, ov))
        os_ = torch.empty(shared.size, dtype=torch.int32, device="cuda")
        tickets.append(srv.submit("exclusive_scan", "uint", dk, out=os_, device=True))
        tickets.append(srv.submit("reduce", "ulong", dk, out=red, n=shared.size // 2, device=True))
        for t in tickets:
            srv.wait(t, timeout=120)
    assert np.array_equal(dk.cpu().numpy().view(np.uint32), shared)
    for n, ok, ov in outs:
        rk, rv = oracle.radix_sort(shared[:n], "uint", values=np.arange(n, dtype=np.uint32))
        assert np.array_equal(ok.cpu().numpy().view(np.uint32), rk)
        assert np.array_equal(ov.cpu().numpy().view(np.uint32), rv)
    assert np.array_equal(os_.cpu().numpy().view(np.uint32), oracle.scan(shared, "uint", exclusive=True))
    as_u64 = shared.view(np.uint64)  # the same bytes read as n/2 uint64 values
    assert int(red.cpu().numpy().view(np.uint64)[0]) == int(oracle.fold(as_u64, "ulong"))


def _sort_request(srv, rng, n):
    keys = rng.integers(0, 2**32, size=n, dtype=np.uint64).astype(np.uint32)
    k = keys.copy()
    v = np.arange(n, dtype=np.uint32)
    return keys, k, v, srv.submit("sort_by_key", "uint", k, values=v)


def test_server_admission_by_free_memory(cuda):
    """Admission follows the device's free memory: with free memory faked below
    what a request needs and nothing else running, the request fails with
    BCX_MEM_ALLOCATION_FAILURE instead of waiting forever; a request that fits
    is served; with the real figure back, the large request is served too."""
    from compute_gb300 import BcxError
    from compute_gb300._lib import MEM_ALLOCATION_FAILURE
    from compute_gb300.serve import Server
    rng = np.random.default_rng(11)
    with Server(slots=2) as srv:
        srv.inject_faults(fake_free_bytes=64 << 10)  # 64 KiB "free"
        _, _, _, t_big = _sort_request(srv, rng, 1 << 20)  # needs about 8 MiB
        with pytest.raises(BcxError) as e:
            srv.wait(t_big, timeout=60)
        assert e.value.status == MEM_ALLOCATION_FAILURE
        keys, k, v, t_small = _sort_request(srv, rng, 1000)  # about 8 KB: fits
        srv.wait(t_small, timeout=60)
        rk, rv = oracle.radix_sort(keys, "uint", values=np.arange(1000, dtype=np.uint32))
        assert np.array_equal(k, rk) and np.array_equal(v, rv)
        srv.inject_faults(fake_free_bytes=0)
        keys, k, v, t = _sort_request(srv, rng, 1 << 20)
        srv.wait(t, timeout=60)
        rk, rv = oracle.radix_sort(keys, "uint", values=np.arange(1 << 20, dtype=np.uint32))
        assert np.array_equal(k, rk) and np.array_equal(v, rv)


def test_server_survives_allocation_failure(cuda):
    """A batch whose device allocation fails ends its requests with
    BCX_MEM_ALLOCATION_FAILURE; the server goes on serving later requests
    correctly and keeps its memory accounting balanced."""
    from compute_gb300 import BcxError
    from compute_gb300._lib import MEM_ALLOCATION_FAILURE
    from compute_gb300.serve import Server
    rng = np.random.default_rng(12)
    with Server(slots=2) as srv:
        srv.inject_faults(fail_allocations=1)
        _, _, _, t1 = _sort_request(srv, rng, 5000)
        with pytest.raises(BcxError) as e:
            srv.wait(t1, timeout=60)
        assert e.value.status == MEM_ALLOCATION_FAILURE
        outs = [_sort_request(srv, rng, n) for n in (5000, 70_000, 300_001)]
        for keys, k, v, t in outs:
            srv.wait(t, timeout=60)
            rk, rv = oracle.radix_sort(keys, "uint", values=np.arange(keys.size, dtype=np.uint32))
            assert np.array_equal(k, rk) and np.array_equal(v, rv)
        srv.drain()
        assert srv.stats()["used_bytes"] == 0
