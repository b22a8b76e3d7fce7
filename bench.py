"""Benchmark of the bcx hot path on GB300.

One step = one compute::sort_by_key of 2^28 uint32 keys (uniform 32-bit) with
uint32 values (iota) -- the large plain-primitive configuration, the one the
headline "sort Gkeys/s" is quoted on.  Every step sorts its own freshly
generated buffer (2 GiB per step, far larger than the 129 MB L2, so no flush
is needed).  The same run also times the other primitives of that
configuration (exclusive_scan and reduce of 2^30 int32 in [0,100), transform
saxpy a=2.5 over 2^28 float32 U[-1,1]) and reports them under "primitives".

Prints ONE JSON line (rank 0).  `value` is device throughput with inputs
resident in HBM; `e2e` is the same metric through the C ABI host-buffer entry
point (bcx_sort_pairs_host: host->device copy, sort, device->host copy inside
the timed region); `roofline` is the onesweep pass kernel's algorithmic bytes
per launch over its average CUDA-event duration inside the timed region;
`cpu_baseline` is the reference's CPU-device sort (the oracle port of
merge_sort_by_key_on_cpu) timed on a bounded sample on the host cores.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "sort Gkeys/s, scan/reduce GB/s vs HBM peak; batched p50/p99 vs plain, 1 GB300"
N_SORT = DEFAULT_N_SORT = 1 << 28
N_SCAN = DEFAULT_N_SCAN = 1 << 30
N_SAXPY = 1 << 28
WORKLOAD = ("sort_by_key uint32 keys (uniform 32-bit) with uint32 values (iota), n=2^28; "
            "also exclusive_scan/reduce int32 n=2^30 and saxpy float32 n=2^28")
# Algorithmic bytes (fixed model): sort_by_key 4 B histogram read + 4 passes x
# (8 B read + 8 B write) = 68 B/pair; one onesweep pass = 16 B/pair.
SORT_BYTES_PER_PAIR = 68
ONESWEEP_BYTES_PER_PAIR = 16
# DRAM traffic of one onesweep launch per pair, from the ncu capture summarised
# in profiles/radix_onesweep_u32_pairs.md (None until captured).
ONESWEEP_DRAM_BYTES_PER_PAIR = None


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """Samples nvidia-smi clocks/throttle reasons every 200 ms in a thread."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                     timeout=5).stdout.strip()
                if out:
                    self.samples.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def dist_init(n_gpus):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_sort_baseline(sample=1 << 24, trials=3):
    """The reference's CPU-device sort_by_key (merge_sort_by_key_on_cpu, as
    restated in the oracle) on `sample` uint32 pairs with every host thread."""
    import numpy as np

    import oracle
    threads = oracle.hardware_threads()
    rng = np.random.default_rng(20261203)
    keys0 = rng.integers(0, 2**32, size=sample, dtype=np.uint64).astype(np.uint32)
    vals0 = np.arange(sample, dtype=np.uint32)
    times = []
    for _ in range(trials):
        k, v = keys0.copy(), vals0.copy()
        t0 = time.perf_counter()
        oracle.cpu_merge_sort_by_key_u32(k, v, threads=threads)
        times.append(time.perf_counter() - t0)
    best = min(times)
    return {"value": sample / best / 1e9, "unit": "Gkeys/s", "cores": threads, "kind": "port",
            "sample": f"{sample} uint32 pairs (uniform keys, iota values), best of {trials}, "
                      f"merge_sort_by_key_on_cpu restated in oracle/oracle.cpp",
            "median_s": statistics.median(times)}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import numpy as np

    import oracle
    threads = oracle.hardware_threads()
    sample = 1 << 23
    rng = np.random.default_rng(20261203)
    keys0 = rng.integers(0, 2**32, size=sample, dtype=np.uint64).astype(np.uint32)
    vals0 = np.arange(sample, dtype=np.uint32)
    for _ in range(args.warmup):
        k, v = keys0.copy(), vals0.copy()
        oracle.cpu_merge_sort_by_key_u32(k, v, threads=threads)
    total = 0.0
    for _ in range(args.steps):
        k, v = keys0.copy(), vals0.copy()
        t0 = time.perf_counter()
        oracle.cpu_merge_sort_by_key_u32(k, v, threads=threads)
        total += time.perf_counter() - t0
    value = sample * args.steps / total / 1e9
    line = {"metric": METRIC, "impl": "reference", "value": value, "unit": "Gkeys/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": total / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "uint32", "data": "synthetic (seeded uniform uint32 keys, iota values)",
            "config": {"workload": WORKLOAD, "reference_sample": f"{sample} pairs per step"},
            "cpu_baseline": {"value": value, "unit": "Gkeys/s", "cores": threads, "kind": "port",
                             "sample": f"{sample} uint32 pairs per step; the reference's CPU-device "
                                       "sort_by_key (merge_sort_by_key_on_cpu) restated in oracle/; the "
                                       "reference itself needs OpenCL+Boost, absent on this box"},
            "e2e": {"value": value, "unit": "Gkeys/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def time_primitive(torch, fn, steps, warmup):
    s = torch.cuda.current_stream()
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(s)
    for _ in range(steps):
        fn()
    b.record(s)
    b.synchronize()
    return a.elapsed_time(b) / steps


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="bcx", choices=["bcx", "reference"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--only", default="all", choices=["all", "sort", "prims"],
                    help="'sort' skips the other primitives, 'prims' skips the sort (profiling runs)")
    ap.add_argument("--n-sort", type=int, default=DEFAULT_N_SORT, help="pairs per sort (default 2^28)")
    ap.add_argument("--n-scan", type=int, default=DEFAULT_N_SCAN, help="scan/reduce elements (default 2^30)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
        return

    import torch

    import compute_gb300 as bc
    global N_SORT, N_SCAN
    N_SORT = args.n_sort
    N_SCAN = args.n_scan
    if args.only == "prims":
        N_SORT = 1 << 20
    rank, world, local = dist_init(args.gpus)
    torch.cuda.set_device(local)
    hbm, peak_kind = peaks()
    dev = torch.device("cuda", local)

    # ---- headline: sort_by_key 2^28 uint32 pairs --------------------------
    total_steps = args.warmup + args.steps
    g = torch.Generator(device=dev).manual_seed(20261203 + rank)
    keys0 = torch.randint(-2**31, 2**31, (N_SORT,), dtype=torch.int32, device=dev, generator=g)
    vals0 = torch.arange(N_SORT, dtype=torch.int32, device=dev)
    bufs = [(keys0.clone(), vals0.clone()) for _ in range(total_steps)]
    del keys0, vals0
    torch.cuda.synchronize()
    for i in range(args.warmup):
        bc.sort_by_key(bufs[i][0], bufs[i][1], dtype="uint")
    torch.cuda.synchronize()
    barrier(world)
    s = torch.cuda.current_stream()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clocks:
        time.sleep(0.3)
        with bc.profile() as prof:
            torch.cuda.synchronize()
            ev0.record(s)
            for i in range(args.warmup, total_steps):
                bc.sort_by_key(bufs[i][0], bufs[i][1], dtype="uint")
            ev1.record(s)
            ev1.synchronize()
        ms_total = ev0.elapsed_time(ev1)
    torch.cuda.synchronize()
    ms_total = max_over_ranks(ms_total, world)
    barrier(world)
    ms_step = ms_total / args.steps
    value = N_SORT * args.steps * world / (ms_total / 1e3) / 1e9
    # correctness of the last timed step (cheap property check)
    k_last = bufs[-1][0].to(torch.int64) & 0xFFFFFFFF
    sorted_ok = bool((k_last[1:] >= k_last[:-1]).all())
    del k_last
    bufs = None
    torch.cuda.empty_cache()

    ks = prof.kernels
    onesweep = ks.get("radix_onesweep", {"launches": 0, "ms": 0.0})
    launches = sum(k["launches"] for k in ks.values())
    avg_ms = onesweep["ms"] / max(onesweep["launches"], 1)
    achieved = ONESWEEP_BYTES_PER_PAIR * N_SORT / (avg_ms / 1e3) / 1e9 if avg_ms > 0 else None
    roofline = {"bound": "hbm", "kernel": "radix_onesweep (one 8-bit pass, uint32 pairs)",
                "achieved": achieved, "peak": hbm, "peak_kind": peak_kind, "unit": "GB/s",
                "frac": achieved / hbm if achieved else None,
                "traffic": (ONESWEEP_DRAM_BYTES_PER_PAIR * N_SORT) if ONESWEEP_DRAM_BYTES_PER_PAIR else None,
                "algorithmic_bytes_per_launch": ONESWEEP_BYTES_PER_PAIR * N_SORT,
                "avg_launch_ms": avg_ms,
                "whole_sort_frac": (SORT_BYTES_PER_PAIR * N_SORT / (ms_step / 1e3) / 1e9) / hbm}
    kernel_share = {k: round(v["ms"] / max(sum(x["ms"] for x in ks.values()), 1e-9), 4) for k, v in ks.items()}

    # ---- other primitives of the configuration ----------------------------
    prims = {}
    psteps = max(3, min(args.steps, 10))
    if args.only == "sort":
        psteps = 0
    if psteps:
        prims = run_primitives(torch, bc, dev, g, psteps, hbm)

    # ---- e2e through the C ABI host-buffer entry point ---------------------
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(torch, bc, rank, world)

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_sort_baseline()

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "Gkeys/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "uint32",
                "data": "synthetic (seeded uniform 32-bit keys, iota values; BASELINE configs' shapes)",
                "config": {"workload": WORKLOAD if N_SORT == 1 << 28 else f"sort_by_key uint32 pairs n={N_SORT}",
                           "l2": "inputs larger than L2: every step sorts its own buffer",
                           "parallelism": "replicas" if world > 1 else "single GPU"},
                "sorted_check": sorted_ok, "roofline": roofline, "kernel_share": kernel_share,
                "gpu_launches": launches, "primitives": prims, "e2e": e2e, "cpu_baseline": cpu,
                "clocks": clocks.summary()}
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def run_primitives(torch, bc, dev, g, psteps, hbm):
    prims = {}
    a = torch.randint(0, 100, (N_SCAN,), dtype=torch.int32, device=dev, generator=g)
    out = torch.empty_like(a)
    red = torch.zeros(1, dtype=torch.int32, device=dev)
    ms = time_primitive(torch, lambda: bc.exclusive_scan(a, out=out), psteps, 3)
    gbs = 8 * N_SCAN / (ms / 1e3) / 1e9
    prims["exclusive_scan_i32_2p30"] = {"ms": ms, "GB/s": gbs, "frac": gbs / hbm, "bytes_per_elem": 8}
    ms = time_primitive(torch, lambda: bc.reduce(a, out=red), psteps, 3)
    gbs = 4 * N_SCAN / (ms / 1e3) / 1e9
    prims["reduce_i32_2p30"] = {"ms": ms, "GB/s": gbs, "frac": gbs / hbm, "bytes_per_elem": 4}
    del a, out
    x = torch.rand(N_SAXPY, dtype=torch.float32, device=dev, generator=g) * 2 - 1
    y = torch.rand(N_SAXPY, dtype=torch.float32, device=dev, generator=g) * 2 - 1
    r = torch.empty_like(x)
    ms = time_primitive(torch, lambda: bc.saxpy(2.5, x, y, out=r), psteps, 3)
    gbs = 12 * N_SAXPY / (ms / 1e3) / 1e9
    prims["saxpy_f32_2p28"] = {"ms": ms, "GB/s": gbs, "frac": gbs / hbm, "bytes_per_elem": 12}
    del x, y, r
    torch.cuda.empty_cache()
    return prims


def run_e2e(torch, bc, rank, world):
    import numpy as np
    rng = np.random.default_rng(20261203 + rank)
    hk0 = rng.integers(0, 2**32, size=N_SORT, dtype=np.uint64).astype(np.uint32)
    hk = torch.from_numpy(hk0.view(np.int32)).pin_memory()
    hv = torch.arange(N_SORT, dtype=torch.int32).pin_memory()
    src_k = torch.from_numpy(hk0.view(np.int32))
    src_v = torch.arange(N_SORT, dtype=torch.int32)
    e2e_steps = 3
    bc.sort_by_key_host(hk, hv, dtype="uint")  # warm-up
    tot = 0.0
    for _ in range(e2e_steps):
        hk.copy_(src_k)
        hv.copy_(src_v)
        barrier(world)
        t0 = time.perf_counter()
        bc.sort_by_key_host(hk, hv, dtype="uint")
        tot += time.perf_counter() - t0
    tot = max_over_ranks(tot, world)
    return {"value": N_SORT * e2e_steps * world / tot / 1e9, "unit": "Gkeys/s",
            "h2d_bytes_per_step": 8 * N_SORT, "d2h_bytes_per_step": 8 * N_SORT,
            "ms_per_step": tot / e2e_steps * 1e3, "steps": e2e_steps,
            "path": "bcx_sort_pairs_host (pinned host buffers)"}


if __name__ == "__main__":
    main()
