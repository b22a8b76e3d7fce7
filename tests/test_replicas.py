"""The N>1 path of bench.py on CPU: two gloo ranks run the barrier and the
max-over-ranks of the step time, and the job throughput is the units all
ranks processed over the slowest rank's time (replicas, weak scaling).  The
reference arm prints from rank 0 only; other ranks exit without work."""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    sys.path.insert(0, ROOT)
    import bench
    r, w, local = bench.dist_init(world, backend="gloo")
    assert (r, w, local) == (rank, world, rank)
    bench.barrier(w)
    slowest = bench.max_over_ranks(0.010 * (rank + 1), w)
    value = bench.job_throughput(1_000_000, slowest, w)
    with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as f:
        f.write(f"{slowest} {value}")
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_gloo_ranks_max_time_and_job_throughput(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    for rank in range(2):
        slowest, value = map(float, (tmp_path / f"rank{rank}.txt").read_text().split())
        assert slowest == pytest.approx(0.020)
        assert value == pytest.approx(1_000_000 * 2 / 0.020 * 1e-9)


def test_reference_arm_only_rank0_prints():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1", MASTER_ADDR="127.0.0.1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3"], capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
