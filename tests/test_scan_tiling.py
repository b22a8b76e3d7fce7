"""The staged scan's tile arithmetic, restated in Python and checked on the CPU.

scan_staged_kernel (compute_gb300/csrc/bcx_scan.cuh) gives thread t the
contiguous run of VPT 16-byte vectors starting at vector t*VPT and visits them
starting at vector t mod VPT, wrapping around, so that the eight threads of a
shared-memory phase touch eight different bank groups.  The fold keeps the
vectors [r, VPT) and [0, r) apart and combines them in element order.  These
tests model that index logic for the shapes the kernel uses (64 KB tiles of
256 threads: 16 vectors per thread; 96 KB tiles for 8-byte elements: 24) and
check that (1) every output equals the serial scan for full and ragged tiles,
inclusive and exclusive, and (2) no phase of a 16-byte shared-memory access
has two threads on one bank group.
"""
import numpy as np
import pytest

THREADS = 256


def staged_tile_scan(x, cnt, vpt, n_per_vec, exclusive, prefix):
    """Outputs of one tile (int64 plus) the way the kernel forms them."""
    items = vpt * n_per_vec
    tile = THREADS * items
    te = np.zeros(tile, dtype=np.int64)
    te[:cnt] = x[:cnt]
    full = cnt == tile
    totals, parts = [], []
    for t in range(THREADS):
        r = t % vpt
        a = part_a = 0
        for k in range(vpt):
            v = k + r - (vpt if k + r >= vpt else 0)
            if k > 0 and v == 0:
                part_a, a = a, 0
            for m in range(n_per_vec):
                i = t * items + v * n_per_vec + m
                if full or i < cnt:
                    a += int(te[i])
        part_b = 0
        if r == 0:
            part_a = a
        else:
            part_b = a
        totals.append(part_b + part_a)
        parts.append(part_b)
    excl = np.concatenate([[0], np.cumsum(totals)[:-1]])
    out = np.zeros(tile, dtype=np.int64)
    for t in range(THREADS):
        r = t % vpt
        pre = prefix + int(excl[t])
        run = pre + parts[t]
        for k in range(vpt):
            v = k + r - (vpt if k + r >= vpt else 0)
            if k > 0 and v == 0:
                run = pre
            for m in range(n_per_vec):
                i = t * items + v * n_per_vec + m
                ok = full or i < cnt
                if exclusive:
                    out[i] = run
                    if ok:
                        run += int(te[i])
                else:
                    if ok:
                        run += int(te[i])
                    out[i] = run
    return out[:cnt], sum(totals)


@pytest.mark.parametrize("vpt,n_per_vec", [(16, 4), (16, 16), (24, 2)])
@pytest.mark.parametrize("exclusive", [False, True])
def test_rotated_runs_scan_in_element_order(vpt, n_per_vec, exclusive):
    rng = np.random.default_rng(vpt * 100 + n_per_vec)
    tile = THREADS * vpt * n_per_vec
    for cnt in (tile, tile - 1, 1, n_per_vec + 3, tile // 3 + 7):
        x = rng.integers(0, 100, tile)
        got, agg = staged_tile_scan(x, cnt, vpt, n_per_vec, exclusive, prefix=7)
        ref = np.cumsum(x[:cnt]) + 7
        if exclusive:
            ref = np.concatenate([[7], ref[:-1]])
        np.testing.assert_array_equal(got, ref, err_msg=f"cnt={cnt}")
        assert agg == int(x[:cnt].sum())


@pytest.mark.parametrize("vpt", [16, 24])
def test_rotated_vector_order_has_no_bank_conflicts(vpt):
    """A 16-byte shared-memory access is served in phases of 8 threads; thread t
    at step k reads vector t*vpt + ((k + t) mod vpt), i.e. bank group
    (that index) mod 8.  Every phase must use 8 distinct groups."""
    for k in range(vpt):
        for p in range(0, THREADS, 8):
            groups = [(t * vpt + (k + t % vpt) % vpt) % 8 for t in range(p, p + 8)]
            assert len(set(groups)) == 8, (vpt, k, p, groups)
