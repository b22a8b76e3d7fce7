"""Benchmark of the bcx hot path on GB300.

One step = one compute::sort_by_key of 2^28 uint32 keys (uniform 32-bit) with
uint32 values (iota) -- the large plain-primitive configuration, the one the
headline "sort Gkeys/s" is quoted on.  Every step sorts its own freshly
generated buffer (2 GiB per step, far larger than the 129 MB L2, so no flush
is needed).  The same run reports, in sections of the JSON line:

  primitives  README float sort of 2^20; exclusive_scan and reduce of 2^30
              int32 in [0,100); transform saxpy a=2.5 over 2^28 float32 U[-1,1]
  precision   accumulate / inclusive_scan of 2^30 float32 N(1000,1):
              compensated vs plain FP32 vs a serial FP32 fold, errors against an
              FP64 reference; float32 sort of 2^27 with NaN/+-0/denormals/+-inf;
              uint64 sorts of 2^27 keys (Zipf 1.1, equal, presorted, 8 bits)
  segmented   10,000 log-uniform segments in [16, 2^20] (and the first 2^28
              elements of them): segmented sort_by_key, exclusive_scan,
              reduce_by_key -- autotuned, replayed from a CUDA graph, against one
              plain call per segment
  serving     open-loop Poisson arrivals of mixed requests through the
              continuous-batching server: p50/p99 latency and throughput
              against serial plain calls

`value` is device throughput with inputs resident in HBM; `e2e` is the same
metric through the C ABI host-buffer entry point (bcx_sort_pairs_host:
host->device copy, sort, device->host copy inside the timed region);
`roofline` is the onesweep pass kernel's algorithmic bytes per launch over its
average CUDA-event duration inside the timed region; `cpu_baseline` is the
reference's CPU-device sort (the oracle port of merge_sort_by_key_on_cpu)
timed on a bounded sample on the host cores.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                    [--only all|sort|prims|precision|serve|segmented]
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
# DRAM traffic of one onesweep launch per pair: dram__bytes_read.sum +
# dram__bytes_write.sum of one captured launch at 2^25 pairs, per pair, scaled
# to the 2^28-pair launch by the pairs it moves.
ONESWEEP_DRAM_BYTES_PER_PAIR = (278.886656e6 + 239.637504e6) / (1 << 25)


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


def dist_init(n_gpus, backend="nccl"):
    """Rank, world size and local rank from the torchrun environment; joins
    the process group when there is more than one rank (replicas: the group
    only carries the barrier and the max-over-ranks of the step time)."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        if not dist.is_initialized():
            dist.init_process_group(backend)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    """The largest x over all ranks (the job's time is its slowest rank's)."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank, seconds_max, world, scale=1e-9):
    """Whole-job throughput: the units all ranks processed over the slowest
    rank's time (weak scaling: every rank processes units_per_rank)."""
    return units_per_rank * world / seconds_max * scale


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


def cpu_prims_baseline(sample=1 << 27, trials=3):
    """The reference's CPU-device scan (scan_on_cpu), reduce (reduce_on_cpu)
    and the saxpy transform, as restated in the oracle, on `sample` elements
    with every host thread: GB/s over the same algorithmic bytes as the GPU
    lines (scan 8 B, reduce 4 B, saxpy 12 B per element)."""
    import numpy as np

    import oracle
    threads = oracle.hardware_threads()
    rng = np.random.default_rng(20261203)
    a = rng.integers(0, 100, size=sample).astype(np.int32)
    out = np.empty_like(a)
    x = rng.uniform(-1, 1, size=sample).astype(np.float32)
    y = rng.uniform(-1, 1, size=sample).astype(np.float32)
    r = np.empty_like(x)

    def best(fn):
        ts = []
        for _ in range(trials):
            t0 = time.perf_counter()
            fn()
            ts.append(time.perf_counter() - t0)
        return min(ts)

    out_lines = {}
    for name, fn, bpe, ref in [
            ("exclusive_scan_i32", lambda: oracle.cpu_exclusive_scan_i32(a, out, 0, threads=threads), 8,
             "scan_on_cpu"),
            ("reduce_i32", lambda: oracle.cpu_reduce_i32(a, threads=threads), 4, "reduce_on_cpu"),
            ("saxpy_f32", lambda: oracle.cpu_saxpy_f32(2.5, x, y, r, threads=threads), 12,
             "transform (2.5f * x + y)")]:
        t = best(fn)
        out_lines[name] = {"value": bpe * sample / t / 1e9, "unit": "GB/s", "cores": threads, "kind": "port",
                           "sample": f"{sample} elements, best of {trials}, {ref} restated in oracle/oracle.cpp"}
    return out_lines


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
    ap.add_argument("--only", default="all", choices=["all", "sort", "prims", "precision", "serve", "segmented"],
                    help="'sort' skips the other sections; 'prims', 'precision', 'serve', 'segmented' run a "
                         "2^20 sort and that section only (profiling runs)")
    ap.add_argument("--serve-count", type=int, default=1000, help="requests per arrival rate")
    ap.add_argument("--seg-count", type=int, default=10_000, help="segments of the segmented workloads")
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
    if args.only in ("prims", "precision", "serve", "segmented"):
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
    value = job_throughput(N_SORT * args.steps, ms_total / 1e3, world)
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

    # ---- e2e through the C ABI host-buffer entry point (measured before the
    # other sections, on the same fresh process state as the headline) -------
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(torch, bc, rank, world)

    # ---- other primitives of the configuration ----------------------------
    prims = {}
    psteps = max(3, min(args.steps, 10))
    if args.only != "all" and args.only != "prims":
        psteps = 0
    if psteps:
        prims = run_primitives(torch, bc, dev, g, psteps, hbm)
        if rank == 0:
            torch.cuda.synchronize()
            prims["drop_in_generated"] = run_drop_in(psteps)
            for v in prims["drop_in_generated"].values():
                if isinstance(v, dict) and "GB/s" in v:
                    v["frac"] = v["GB/s"] / hbm
    precision = None
    if args.only in ("all", "precision"):
        precision = run_precision(torch, bc, dev, hbm)
    segmented = None
    if args.only in ("all", "segmented"):
        segmented = run_segmented(torch, bc, dev, hbm, nseg=args.seg_count)
    serving = None
    if args.only in ("all", "serve") and world == 1:
        serving = run_serving(torch, bc, dev, count=args.serve_count)


    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_sort_baseline()
        if prims:
            for name, line in cpu_prims_baseline().items():
                for key in prims:
                    if key.startswith(name):
                        prims[key]["cpu_baseline"] = line

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "Gkeys/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "uint32",
                "data": "synthetic (seeded uniform 32-bit keys, iota values; the configuration's shapes)",
                "config": {"workload": WORKLOAD if N_SORT == 1 << 28 else f"sort_by_key uint32 pairs n={N_SORT}",
                           "l2": "inputs larger than L2: every step sorts its own buffer",
                           "parallelism": "replicas" if world > 1 else "single GPU"},
                "sorted_check": sorted_ok, "roofline": roofline, "kernel_share": kernel_share,
                "gpu_launches": launches, "primitives": prims, "precision": precision, "segmented": segmented, "serving": serving, "e2e": e2e,
                "cpu_baseline": cpu,
                "clocks": clocks.summary()}
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def run_primitives(torch, bc, dev, g, psteps, hbm):
    prims = {}
    # README example: compute::sort of 2^20 float32 integers in [0, 2^31-1]
    # (launch-bound at this size: reported, not a roofline target)
    n_small = 1 << 20
    base = torch.randint(0, 2**31 - 1, (n_small,), dtype=torch.int64, device=dev, generator=g).to(torch.float32)
    bufs = [base.clone() for _ in range(psteps + 3)]
    for i in range(3):
        bc.sort(bufs[i])
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for i in range(3, psteps + 3):
        bc.sort(bufs[i])
    b.record()
    b.synchronize()
    ms = a.elapsed_time(b) / psteps
    prims["sort_f32_readme_2p20"] = {"us": ms * 1e3, "Gkeys/s": n_small / ms / 1e6,
                                     "sorted": bool((bufs[-1][1:] >= bufs[-1][:-1]).all())}
    del bufs, base
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


def run_drop_in(steps):
    """The drop-in calls whose kernels are generated at run time (saxpy as the
    lambda alpha * _1 + _2, user-function scans and accumulate), timed by
    tests/cpp/drop_in_bench.cpp through the boost::compute headers."""
    import shutil
    import tempfile
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        return {"unavailable": "no C++ compiler"}
    src = os.path.join(ROOT, "tests", "cpp", "drop_in_bench.cpp")
    libdir = os.path.join(ROOT, "compute_gb300")
    with tempfile.TemporaryDirectory() as tmp:
        exe = os.path.join(tmp, "drop_in_bench")
        r = subprocess.run([cxx, "-std=c++17", "-O2", f"-I{os.path.join(ROOT, 'include')}", src, "-o", exe,
                            f"-L{libdir}", "-lbcx", f"-Wl,-rpath,{libdir}"], capture_output=True, text=True)
        if r.returncode != 0:
            return {"unavailable": "build failed: " + r.stderr[-300:]}
        run = subprocess.run([exe, str(steps)], capture_output=True, text=True, timeout=600)
        if run.returncode != 0:
            return {"failed": (run.stdout + run.stderr)[-500:]}
        return json.loads(run.stdout.strip().splitlines()[-1])


def run_e2e(torch, bc, rank, world):
    import numpy as np
    rng = np.random.default_rng(20261203 + rank)
    hk0 = rng.integers(0, 2**32, size=N_SORT, dtype=np.uint64).astype(np.uint32)
    hk = torch.from_numpy(hk0.view(np.int32)).pin_memory()
    hv = torch.arange(N_SORT, dtype=torch.int32).pin_memory()
    src_k = torch.from_numpy(hk0.view(np.int32))
    src_v = torch.arange(N_SORT, dtype=torch.int32)
    e2e_steps = 16
    for _ in range(3):  # warm-up (pool, page-locked pages, copy engines)
        bc.sort_by_key_host(hk, hv, dtype="uint")
    tot = 0.0
    per = []
    for _ in range(e2e_steps):
        hk.copy_(src_k)
        hv.copy_(src_v)
        barrier(world)
        t0 = time.perf_counter()
        bc.sort_by_key_host(hk, hv, dtype="uint")
        per.append(time.perf_counter() - t0)
        tot += per[-1]
    tot = max_over_ranks(tot, world)
    # The link bound of one step: the same 2 x 4 B x n bytes copied to the
    # device and back as plain pinned copies, no sort in between.
    dk = torch.empty(N_SORT, dtype=torch.int32, device="cuda")
    dv = torch.empty_like(dk)
    copies = []
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        dk.copy_(hk, non_blocking=True)
        dv.copy_(hv, non_blocking=True)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        hk.copy_(dk, non_blocking=True)
        hv.copy_(dv, non_blocking=True)
        torch.cuda.synchronize()
        copies.append((t1 - t0, time.perf_counter() - t1))
    # The same plain copies over as many steps as the timed loop, with the
    # same host refill between steps: the steps that take far longer than
    # the median occur here too, without any library code in them.
    plain = []
    for _ in range(e2e_steps):
        hk.copy_(src_k)
        hv.copy_(src_v)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        dk.copy_(hk, non_blocking=True)
        dv.copy_(hv, non_blocking=True)
        hk.copy_(dk, non_blocking=True)
        hv.copy_(dv, non_blocking=True)
        torch.cuda.synchronize()
        plain.append(time.perf_counter() - t0)
    del dk, dv
    h2d = min(c[0] for c in copies)
    d2h = min(c[1] for c in copies)

    def slow(xs):
        med = statistics.median(xs)
        return sum(1 for x in xs if x > 1.5 * med)

    link = {"h2d_ms": h2d * 1e3, "d2h_ms": d2h * 1e3, "h2d_GBps": 8 * N_SORT / h2d / 1e9,
            "d2h_GBps": 8 * N_SORT / d2h / 1e9, "copies_ms": (h2d + d2h) * 1e3,
            "how": "the step's 2 x 4 B x n bytes each way as plain pinned torch copies, best of 3",
            "plain_copy_steps_ms": [round(x * 1e3, 2) for x in plain],
            "slow_steps": {"e2e": slow(per), "plain_copies": slow(plain),
                           "note": "steps over 1.5x their loop's median"}}
    return {"value": job_throughput(N_SORT * e2e_steps, tot, world), "unit": "Gkeys/s", "link_bound": link,
            "h2d_bytes_per_step": 8 * N_SORT, "d2h_bytes_per_step": 8 * N_SORT,
            "ms_per_step": tot / e2e_steps * 1e3, "ms_median_step": statistics.median(per) * 1e3,
            "ms_steps": [round(x * 1e3, 2) for x in per],
            "steps": e2e_steps, "path": "bcx_sort_pairs_host (pinned host buffers)"}


# ---- precision and key-distribution stress ---------------------------------
def run_precision(torch, bc, dev, hbm, seed=20261206, n_acc=1 << 30, n_sort=1 << 27, steps=3):
    """accumulate / inclusive_scan of 2^30 float32 N(1000, 1): compensated
    (Neumaier in FP32, FP64 combine) against plain FP32, errors against an
    FP64 reference computed on the device (torch float64), plus the error of a
    strictly serial FP32 left fold (what the reference's float accumulate
    computes).  Then float32 sorts of 2^27 keys with 1% NaN, +-0.0, denormals
    and +-inf, and uint64 sorts of 2^27 keys: Zipf(1.1), all equal, presorted
    and 8 significant bits (throughput; order checked by a sortedness scan)."""
    import numpy as np
    g = torch.Generator(device=dev).manual_seed(seed)
    out = {}
    x = torch.randn(n_acc, dtype=torch.float32, device=dev, generator=g) + 1000.0
    ref = float(x.double().sum().item())
    comp = bc.accumulate(x, 0.0, compensated=True)
    plain = float(bc.reduce(x, compensated=False).item())
    ms_comp = time_primitive(torch, lambda: bc.reduce(x, compensated=True), steps, 3)
    ms_plain = time_primitive(torch, lambda: bc.reduce(x, compensated=False), steps, 3)
    xs = x.cpu().numpy()
    serial = float(np.cumsum(xs, dtype=np.float32)[-1])  # strict left-to-right FP32 fold
    del xs
    out["accumulate_f32_N1000_2p30"] = {
        "fp64_sum": ref, "compensated": comp, "plain_fp32": plain, "serial_fp32": serial,
        "rel_err_compensated": abs(comp - ref) / abs(ref), "rel_err_plain_fp32": abs(plain - ref) / abs(ref),
        "rel_err_serial_fp32": abs(serial - ref) / abs(ref),
        "ulp_of_fp32_result": float(np.spacing(np.float32(ref))),
        "abs_err_compensated_in_ulps": abs(comp - ref) / float(np.spacing(np.float32(ref))),
        "ms_compensated": ms_comp, "ms_plain": ms_plain,
        "GB_per_s_compensated": 4 * n_acc / ms_comp / 1e6, "frac_compensated": 4 * n_acc / ms_comp / 1e6 / hbm}
    y = torch.empty_like(x)
    bc.inclusive_scan(x, out=y, compensated=True)
    ref_scan = torch.cumsum(x.double(), 0)
    rel = ((y.double() - ref_scan).abs() / ref_scan.abs())
    err_c = float(rel.max().item())
    bc.inclusive_scan(x, out=y, compensated=False)
    rel = ((y.double() - ref_scan).abs() / ref_scan.abs())
    err_p = float(rel.max().item())
    del rel, ref_scan
    ms_c = time_primitive(torch, lambda: bc.inclusive_scan(x, out=y, compensated=True), steps, 3)
    ms_p = time_primitive(torch, lambda: bc.inclusive_scan(x, out=y, compensated=False), steps, 3)
    out["inclusive_scan_f32_N1000_2p30"] = {
        "max_rel_err_compensated": err_c, "max_rel_err_plain_fp32": err_p, "ms_compensated": ms_c,
        "ms_plain": ms_p, "GB_per_s_compensated": 8 * n_acc / ms_c / 1e6,
        "frac_compensated": 8 * n_acc / ms_c / 1e6 / hbm}
    del x, y
    torch.cuda.empty_cache()

    def time_sort(make, dtype, label, check_key):
        base = make()
        bufs = [base.clone() for _ in range(steps + 1)]
        bc.sort(bufs[0], dtype=dtype)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for i in range(1, steps + 1):
            bc.sort(bufs[i], dtype=dtype)
        b.record()
        b.synchronize()
        ms = a.elapsed_time(b) / steps
        k = check_key(bufs[-1])
        ok = bool((k[1:] >= k[:-1]).all())
        del bufs, base, k
        torch.cuda.empty_cache()
        out[label] = {"ms": ms, "Gkeys_per_s": n_sort / ms / 1e6, "sorted": ok}

    def f32_stress():
        v = torch.randn(n_sort, dtype=torch.float32, device=dev, generator=g) * 1e3
        r = torch.rand(n_sort, device=dev, generator=g)
        v[r < 0.01] = float("nan")
        v[(r >= 0.01) & (r < 0.02)] = 0.0
        v[(r >= 0.02) & (r < 0.03)] = -0.0
        v[(r >= 0.03) & (r < 0.04)] = 1e-40
        v[(r >= 0.04) & (r < 0.05)] = -1e-40
        v[(r >= 0.05) & (r < 0.055)] = float("inf")
        v[(r >= 0.055) & (r < 0.06)] = -float("inf")
        return v

    def f32_order_key(t):
        # the total order of the sort: sign-flipped bits compared as unsigned
        u = t.view(torch.int32).to(torch.int64) & 0xFFFFFFFF
        neg = u >= 0x80000000
        return torch.where(neg, 0xFFFFFFFF - u, u + 0x80000000)

    time_sort(f32_stress, "float", "sort_f32_specials_2p27", f32_order_key)

    def u64(kind):
        def make():
            if kind == "zipf":
                z = np.random.default_rng(seed).zipf(1.1, size=n_sort).astype(np.int64)  # >= 1
                return torch.from_numpy(z).to(dev)
            if kind == "equal":
                return torch.full((n_sort,), 0x123456789, dtype=torch.int64, device=dev)
            if kind == "sorted":
                return torch.arange(n_sort, dtype=torch.int64, device=dev) * 3
            return torch.randint(0, 256, (n_sort,), dtype=torch.int64, device=dev, generator=g)
        return make

    def u64_key(t):  # values here are non-negative, so signed order is unsigned order
        return t

    for kind in ("zipf", "equal", "sorted", "8bit"):
        time_sort(u64(kind), "ulong", f"sort_u64_{kind}_2p27", u64_key)
    return out


# ---- segmented work --------------------------------------------------------
def segment_offsets(nseg=10_000, lo=16, hi=1 << 20, seed=20261205, total_cap=None):
    """10,000 segment sizes log-uniform in [16, 2^20] (seeded); with total_cap,
    the first segments whose sizes reach that total."""
    import numpy as np
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(lo), np.log(hi), size=nseg)).astype(np.int64)
    if total_cap is not None:
        csum = np.cumsum(sizes)
        k = int(np.searchsorted(csum, total_cap)) + 1
        sizes = sizes[:k]
    return np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)


def _events(torch):
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def _graph_of(torch, fn):
    """fn() captured once in a CUDA graph (after one eager warm-up call)."""
    fn()
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        fn()
    torch.cuda.synchronize()
    return g


def run_segmented(torch, bc, dev, hbm, steps=3, seed=20261205, nseg=10_000):
    """Segmented sort_by_key (uint32/uint32), segmented exclusive_scan (int32)
    and reduce_by_key (float32 N(0,1), keys = segment ids) over 10,000
    log-uniform segments: one launch sequence each, tuned by the autotuner and
    replayed from a captured CUDA graph, against one plain call per segment on
    the same stream."""
    import ctypes as C

    import numpy as np

    from compute_gb300._lib import DTYPES, lib
    L = lib()
    results = {}
    configs = ((f"{nseg}_segments", None), ("2^28_total", 1 << 28)) if nseg == 10_000 else ((f"{nseg}_segments", None),)
    for label, cap in configs:
        offsets = segment_offsets(nseg=nseg, total_cap=cap, seed=seed)
        nseg = offsets.size - 1
        n = int(offsets[-1])
        sizes = np.diff(offsets).astype(np.int64)
        offs = torch.from_numpy(offsets.view(np.int64).copy()).to(dev)
        st = torch.cuda.current_stream().cuda_stream
        g = torch.Generator(device=dev).manual_seed(seed)
        entry = {"segments": int(nseg), "elements": n, "min_segment": int(sizes.min()),
                 "max_segment": int(sizes.max())}
        rep = C.create_string_buffer(1 << 14)

        # -- segmented sort_by_key uint32 / uint32
        keys0 = torch.randint(-2**31, 2**31 - 1, (n,), dtype=torch.int32, device=dev, generator=g)
        vals0 = torch.arange(n, dtype=torch.int32, device=dev)
        keys, vals = keys0.clone(), vals0.clone()
        t0 = time.perf_counter()
        rc = L.bcx_tune_segmented_sort_pairs(st, DTYPES["uint"], 4, keys0.data_ptr(), vals0.data_ptr(), n,
                                             offs.data_ptr(), nseg, rep, len(rep))
        assert rc == 0, L.bcx_last_error_string()
        tune_s = time.perf_counter() - t0
        tuned = [ln for ln in rep.value.decode().splitlines() if "->" in ln]
        tb = C.c_size_t(0)
        rc = L.bcx_segmented_sort_pairs(st, DTYPES["uint"], 4, keys.data_ptr(), vals.data_ptr(), n, offs.data_ptr(),
                                        nseg, 0, None, C.byref(tb))
        assert rc == 0, L.bcx_last_error_string()
        temp = torch.empty(tb.value, dtype=torch.uint8, device=dev)

        def seg_sort():
            t = C.c_size_t(temp.numel())
            r = L.bcx_segmented_sort_pairs(torch.cuda.current_stream().cuda_stream, DTYPES["uint"], 4,
                                           keys.data_ptr(), vals.data_ptr(), n, offs.data_ptr(), nseg, 0,
                                           temp.data_ptr(), C.byref(t))
            assert r == 0, L.bcx_last_error_string()

        graph = _graph_of(torch, seg_sort)
        ms = []
        for _ in range(steps):
            keys.copy_(keys0)
            vals.copy_(vals0)
            a, b = _events(torch)
            a.record()
            graph.replay()
            b.record()
            b.synchronize()
            ms.append(a.elapsed_time(b))
        graph_ms = statistics.median(ms)
        # correctness: every segment non-decreasing (as uint32)
        k64 = keys.to(torch.int64) & 0xFFFFFFFF
        inner = torch.ones(n, dtype=torch.bool, device=dev)
        inner[offs[:-1].clamp(max=n - 1)] = False
        ok = bool(((k64[1:] >= k64[:-1]) | ~inner[1:]).all())
        del k64, inner
        # one plain sort_by_key per segment
        keys.copy_(keys0)
        vals.copy_(vals0)
        torch.cuda.synchronize()
        kp, vp = keys.data_ptr(), vals.data_ptr()
        a, b = _events(torch)
        a.record()
        for s_, m in zip(offsets[:-1].tolist(), sizes.tolist()):
            L.bcx_sort_pairs(st, DTYPES["uint"], 4, kp + 4 * s_, vp + 4 * s_, m, 0, None, None)
        b.record()
        b.synchronize()
        plain_ms = a.elapsed_time(b)
        small_tile = 4096
        for ln in tuned:
            if "small_tile" in ln:
                small_tile = int(ln.split("->")[1])
        large = int(sizes[sizes > small_tile].sum())
        alg_bytes = 68 * large + 16 * (n - large)
        entry["sort_by_key_u32"] = {
            "graph_ms": graph_ms, "per_segment_plain_ms": plain_ms, "speedup_vs_plain": plain_ms / graph_ms,
            "Gkeys_per_s": n / graph_ms / 1e6, "algorithmic_bytes": alg_bytes,
            "GB_per_s": alg_bytes / graph_ms / 1e6, "frac": alg_bytes / graph_ms / 1e6 / hbm,
            "segments_sorted": ok, "tuned": tuned, "tune_s": tune_s}
        del keys0, vals0, keys, vals, temp, graph
        torch.cuda.empty_cache()

        # -- segmented exclusive_scan int32
        x = torch.randint(0, 100, (n,), dtype=torch.int32, device=dev, generator=g)
        out = torch.empty_like(x)
        rc = L.bcx_tune_segmented_scan(st, DTYPES["int"], x.data_ptr(), n, offs.data_ptr(), nseg, rep, len(rep))
        assert rc == 0, L.bcx_last_error_string()
        tuned = [ln for ln in rep.value.decode().splitlines() if "->" in ln]
        zero = (C.c_ubyte * 8)()
        rc = L.bcx_segmented_scan(st, DTYPES["int"], 0, 1, zero, x.data_ptr(), out.data_ptr(), n, offs.data_ptr(),
                                  nseg, 0, None, C.byref(tb))
        assert rc == 0, L.bcx_last_error_string()
        temp = torch.empty(max(tb.value, 1), dtype=torch.uint8, device=dev)

        def seg_scan():
            t = C.c_size_t(temp.numel())
            r = L.bcx_segmented_scan(torch.cuda.current_stream().cuda_stream, DTYPES["int"], 0, 1, zero,
                                     x.data_ptr(), out.data_ptr(), n, offs.data_ptr(), nseg, 0, temp.data_ptr(),
                                     C.byref(t))
            assert r == 0, L.bcx_last_error_string()

        graph = _graph_of(torch, seg_scan)
        ms = []
        for _ in range(steps):
            a, b = _events(torch)
            a.record()
            graph.replay()
            b.record()
            b.synchronize()
            ms.append(a.elapsed_time(b))
        graph_ms = statistics.median(ms)
        xp, op_ = x.data_ptr(), out.data_ptr()
        a, b = _events(torch)
        a.record()
        for s_, m in zip(offsets[:-1].tolist(), sizes.tolist()):
            L.bcx_scan(st, DTYPES["int"], 0, 1, zero, xp + 4 * s_, op_ + 4 * s_, m, 0, None, None)
        b.record()
        b.synchronize()
        plain_ms = a.elapsed_time(b)
        entry["exclusive_scan_i32"] = {
            "graph_ms": graph_ms, "per_segment_plain_ms": plain_ms, "speedup_vs_plain": plain_ms / graph_ms,
            "GB_per_s": 8 * n / graph_ms / 1e6, "frac": 8 * n / graph_ms / 1e6 / hbm, "tuned": tuned}
        del x, out, temp, graph
        torch.cuda.empty_cache()

        # -- reduce_by_key float32 N(0,1), keys = segment ids
        seg_id = torch.repeat_interleave(torch.arange(nseg, dtype=torch.int32, device=dev),
                                         torch.from_numpy(sizes).to(dev))
        v = torch.randn(n, dtype=torch.float32, device=dev, generator=g)
        ko = torch.empty(nseg, dtype=torch.int32, device=dev)
        vo = torch.empty(nseg, dtype=torch.float32, device=dev)
        runs = torch.zeros(1, dtype=torch.int64, device=dev)
        rc = L.bcx_reduce_by_key(st, DTYPES["int"], DTYPES["float"], 0, seg_id.data_ptr(), v.data_ptr(), n,
                                 ko.data_ptr(), vo.data_ptr(), runs.data_ptr(), 1, None, C.byref(tb))
        assert rc == 0, L.bcx_last_error_string()
        temp = torch.empty(max(tb.value, 1), dtype=torch.uint8, device=dev)

        def rbk():
            t = C.c_size_t(temp.numel())
            r = L.bcx_reduce_by_key(torch.cuda.current_stream().cuda_stream, DTYPES["int"], DTYPES["float"], 0,
                                    seg_id.data_ptr(), v.data_ptr(), n, ko.data_ptr(), vo.data_ptr(),
                                    runs.data_ptr(), 1, temp.data_ptr(), C.byref(t))
            assert r == 0, L.bcx_last_error_string()

        graph = _graph_of(torch, rbk)
        ms = []
        for _ in range(steps):
            a, b = _events(torch)
            a.record()
            graph.replay()
            b.record()
            b.synchronize()
            ms.append(a.elapsed_time(b))
        graph_ms = statistics.median(ms)
        runs_ok = int(runs.item()) == nseg
        # the offset-based segmented reduce (autotuned grid), same sums
        rc = L.bcx_tune_segmented_reduce(st, DTYPES["float"], v.data_ptr(), offs.data_ptr(), nseg, rep, len(rep))
        assert rc == 0, L.bcx_last_error_string()
        tuned = [ln for ln in rep.value.decode().splitlines() if "->" in ln]
        so = torch.empty(nseg, dtype=torch.float32, device=dev)
        zf = (C.c_ubyte * 8)()
        rc = L.bcx_segmented_reduce(st, DTYPES["float"], 0, v.data_ptr(), offs.data_ptr(), nseg, zf, so.data_ptr(),
                                    1, None, C.byref(tb))
        assert rc == 0, L.bcx_last_error_string()
        temp2 = torch.empty(max(tb.value, 1), dtype=torch.uint8, device=dev)

        def segred():
            t = C.c_size_t(temp2.numel())
            r = L.bcx_segmented_reduce(torch.cuda.current_stream().cuda_stream, DTYPES["float"], 0, v.data_ptr(),
                                       offs.data_ptr(), nseg, zf, so.data_ptr(), 1, temp2.data_ptr(), C.byref(t))
            assert r == 0, L.bcx_last_error_string()

        graph2 = _graph_of(torch, segred)
        ms = []
        for _ in range(steps):
            a, b = _events(torch)
            a.record()
            graph2.replay()
            b.record()
            b.synchronize()
            ms.append(a.elapsed_time(b))
        segred_ms = statistics.median(ms)
        # one plain (compensated) reduce per segment
        vp_ = v.data_ptr()
        po = so.data_ptr()
        a, b = _events(torch)
        a.record()
        for i, (s_, m) in enumerate(zip(offsets[:-1].tolist(), sizes.tolist())):
            L.bcx_reduce(st, DTYPES["float"], 0, vp_ + 4 * s_, m, po + 4 * i, 1, None, None)
        b.record()
        b.synchronize()
        plain_ms = a.elapsed_time(b)
        entry["reduce_by_key_f32"] = {
            "graph_ms": graph_ms, "per_segment_plain_ms": plain_ms, "speedup_vs_plain": plain_ms / graph_ms,
            "GB_per_s": 8 * n / graph_ms / 1e6, "frac": 8 * n / graph_ms / 1e6 / hbm, "runs_ok": runs_ok,
            "segmented_reduce_by_offsets_ms": segred_ms,
            "segmented_reduce_GB_per_s": 4 * n / segred_ms / 1e6, "tuned": tuned}
        del seg_id, v, ko, vo, runs, temp, temp2, so, graph, graph2
        torch.cuda.empty_cache()
        results[label] = entry
    return results


# ---- serving loop ----------------------------------------------------------
SERVE_KINDS = ("sort_by_key", "exclusive_scan", "reduce")
SERVE_DTYPES = ("int", "uint", "float", "ulong")
SERVE_RATES = (1000, 3000, 10000, 30000, 100000)


def make_serving_requests(count, seed, lo=10, hi=26):
    """Seeded request stream: 50% sort_by_key, 30% exclusive_scan, 20% reduce;
    n log-uniform in [2^lo, 2^hi]; dtype uniform over int/uint/float/ulong."""
    import numpy as np
    rng = np.random.default_rng(seed)
    kinds = rng.choice(3, size=count, p=[0.5, 0.3, 0.2])
    dtypes = rng.integers(0, 4, size=count)
    ns = np.exp(rng.uniform(np.log(2.0 ** lo), np.log(2.0 ** hi), size=count)).astype(np.int64)
    offs = rng.integers(0, 1 << 20, size=count) * 64  # element offset into the input pool (64-aligned)
    return kinds, dtypes, ns, offs


def run_serving(torch, bc, dev, count=1000, rates=SERVE_RATES, seed=20261204, lo=10, hi=26, slots=16,
                small_limit=None, batch_elems=0, batch_count=0, baselines=True):
    """Open-loop Poisson arrivals of device-resident requests through the
    continuous-batching server, against the same requests issued as serial
    plain C-ABI calls (each waited for before the next, as a caller that needs
    its result does) and as plain calls queued back to back on one stream."""
    import ctypes as C

    import numpy as np

    from compute_gb300._lib import DTYPES, DTYPE_SIZE, Request, lib
    from compute_gb300.serve import Server
    L = lib()
    kinds, dtypes, ns, offs = make_serving_requests(count, seed, lo, hi)
    pool_n = (1 << hi) + (1 << 20) * 64
    gen = torch.Generator(device=dev).manual_seed(seed)
    pools = {}
    for name in SERVE_DTYPES:
        if name == "float":
            pools[name] = torch.rand(pool_n, dtype=torch.float32, device=dev, generator=gen)
        elif name == "ulong":
            pools[name] = torch.randint(-2**63, 2**63 - 1, (pool_n,), dtype=torch.int64, device=dev, generator=gen)
        else:
            pools[name] = torch.randint(-2**31, 2**31 - 1, (pool_n,), dtype=torch.int32, device=dev, generator=gen)
    vals = torch.arange(pool_n, dtype=torch.int32, device=dev)
    # Output arena: every request gets its own output slices.
    sizes = []
    for k, d, n in zip(kinds, dtypes, ns):
        es = DTYPE_SIZE[SERVE_DTYPES[d]]
        if k == 0:
            sizes.append((n * es + 255) // 256 * 256 + (n * 4 + 255) // 256 * 256)
        elif k == 1:
            sizes.append((n * es + 255) // 256 * 256)
        else:
            sizes.append(256)
    arena = torch.empty(int(sum(sizes)), dtype=torch.uint8, device=dev)
    base = arena.data_ptr()
    reqs, elems, bytes_moved = [], 0, 0
    cur = base
    for k, d, n, o, sz in zip(kinds, dtypes, ns, offs, sizes):
        name = SERVE_DTYPES[d]
        es = DTYPE_SIZE[name]
        n = int(n)
        src = pools[name].data_ptr() + int(o) * es
        if k == 0:
            ov = cur + (n * es + 255) // 256 * 256
            r = Request(0, DTYPES[name], 4, n, 1, src, vals.data_ptr() + int(o) * 4, cur, ov)
            bytes_moved += n * (es + 4) * 2
        elif k == 1:
            r = Request(1, DTYPES[name], 0, n, 1, src, None, cur, None)
            bytes_moved += n * es * 2
        else:
            r = Request(2, DTYPES[name], 0, n, 1, src, None, cur, None)
            bytes_moved += n * es
        reqs.append(r)
        elems += n
        cur += int(sz)
    torch.cuda.synchronize()

    # -- serial plain calls through the C ABI on one stream
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    zero = (C.c_ubyte * 8)()
    DTYPE_SIZE_BY_CODE = {DTYPES[k]: DTYPE_SIZE[k] for k in SERVE_DTYPES}

    def plain(r):
        if r.kind == 0:
            es = DTYPE_SIZE_BY_CODE[r.dtype]
            L.bcx_memcpy_async(r.out, r.keys, r.n * es, stream)
            L.bcx_memcpy_async(r.out_values, r.values, r.n * 4, stream)
            return L.bcx_sort_pairs(stream, r.dtype, 4, r.out, r.out_values, r.n, 0, None, None)
        comp = 1 if r.dtype == DTYPES["float"] else 0
        if r.kind == 1:
            return L.bcx_scan(stream, r.dtype, 0, 1, zero, r.keys, r.out, r.n, comp, None, None)
        return L.bcx_reduce(stream, r.dtype, 0, r.keys, r.n, r.out, comp, None, None)

    for r in reqs[:20]:
        assert plain(r) == 0
    L.bcx_stream_synchronize(stream)
    if not baselines:  # server only (configuration sweeps)
        reqs_for_baseline = []
    else:
        reqs_for_baseline = reqs
    per_call = []
    dev_ms = 0.0  # device time of each plain call alone (CUDA events around it)
    ea, eb = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    for r in reqs_for_baseline:
        a = time.perf_counter()
        ea.record()
        rc = plain(r)
        eb.record()
        L.bcx_stream_synchronize(stream)
        per_call.append(time.perf_counter() - a)
        dev_ms += ea.elapsed_time(eb)
        assert rc == 0
    serial_s = max(time.perf_counter() - t0, 1e-9)
    t0 = time.perf_counter()
    for r in reqs_for_baseline:
        plain(r)
    L.bcx_stream_synchronize(stream)
    queued_s = max(time.perf_counter() - t0, 1e-9)
    per_call_ms = np.array(per_call if per_call else [0.0]) * 1e3
    out = {"requests_per_rate": count, "elements": int(elems), "bytes_per_pass": int(bytes_moved),
           "mix": "50% sort_by_key (values uint32) / 30% exclusive_scan / 20% reduce; "
                  f"n log-uniform [2^{lo}, 2^{hi}]; dtype uniform int32/uint32/float32/uint64; "
                  "device-resident inputs, per-request outputs",
           "server": {"slots": slots, "small_limit": small_limit if small_limit is not None else 1 << 18,
                      "batch_elems": batch_elems or 1 << 24, "batch_count": batch_count or 4096},
           "serial_plain": {"req_per_s": count / serial_s, "GB_per_s": bytes_moved / serial_s / 1e9,
                            "p50_ms": float(np.percentile(per_call_ms, 50)),
                            "p99_ms": float(np.percentile(per_call_ms, 99)),
                            "note": "one plain C-ABI call per request, each waited for"},
           "queued_plain": {"req_per_s": count / queued_s, "GB_per_s": bytes_moved / queued_s / 1e9,
                            "note": "the same plain calls back to back on one stream, one wait at the end"},
           "kernel_time_bound": {"req_per_s": count / max(dev_ms / 1e3, 1e-9), "device_ms_total": dev_ms,
                                 "note": "requests over the summed device time of each plain call alone: "
                                         "the rate of plain kernels with every per-call gap removed"},
           "rates": []}

    # -- the server, open-loop Poisson arrivals
    rng = np.random.default_rng(seed + 1)
    with Server(slots=slots, small_limit=small_limit, batch_elems=batch_elems, batch_count=batch_count) as srv:
        for r in reqs[:20]:
            srv.wait(srv.submit_request(r))
        for rate in rates:
            srv.reset_stats()
            gaps = rng.exponential(1.0 / rate, size=count)
            arrivals = np.cumsum(gaps)
            tickets = [0] * count
            t0 = time.perf_counter()
            for i, r in enumerate(reqs):
                target = t0 + arrivals[i]
                while time.perf_counter() < target:
                    pass
                tickets[i] = srv.submit_request(r)
            lat = np.array([srv.wait(t) for t in tickets])
            t_end = max(t0 + arrivals[i] + lat[i] / 1e3 for i in range(count))
            span = t_end - t0
            st = srv.stats()
            out["rates"].append({
                "offered_req_per_s": rate, "achieved_req_per_s": count / span,
                "GB_per_s": bytes_moved / span / 1e9,
                "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                "max_ms": float(lat.max()), "batches": int(st["batches"]),
                "batched_requests": int(st["batched_requests"])})
    best = max(x["achieved_req_per_s"] for x in out["rates"])
    out["server_best_req_per_s"] = best
    out["speedup_vs_serial_plain"] = best / out["serial_plain"]["req_per_s"]
    out["speedup_vs_queued_plain"] = best / out["queued_plain"]["req_per_s"]
    out["server_vs_kernel_time_bound"] = best / out["kernel_time_bound"]["req_per_s"]
    del arena, pools, vals
    torch.cuda.empty_cache()
    return out


if __name__ == "__main__":
    main()
