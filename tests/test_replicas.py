"""Multi-GPU is replicas only: each rank runs its own walkers with no data
exchange, and the job's throughput is all ranks' units over the slowest
rank's time.  The aggregation runs here as two gloo ranks on the CPU."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r processed (r + 1) * 1000 units in (r + 1) * 10 ms
        rate, ms = bench.replica_rate((rank + 1) * 1000, (rank + 1) * 10.0, dist, torch.device("cpu"))
        out[rank] = (rate, ms)
    finally:
        dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_replica_rate_two_gloo_ranks():
    world = 2
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.start_processes(_rank, args=(world, _free_port(), out), nprocs=world, start_method="spawn")
        res = dict(out)
    for r in range(world):
        rate, ms = res[r]
        assert ms == 20.0                       # the slowest rank's time
        assert rate == pytest.approx(3000 / 0.020)  # all ranks' units over it


def test_replica_rate_single_process():
    import bench
    rate, ms = bench.replica_rate(500, 5.0)
    assert ms == 5.0 and rate == pytest.approx(1e5)


@pytest.mark.timeout(600)
def test_bench_gpus_2_spawns_two_ranks():
    """``bench.py --gpus 2`` outside a launcher starts two ranks itself (one
    per GPU); on the reference arm, which runs on the host CPU, rank 0 alone
    prints the line and reports both ranks."""
    import json
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ)
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK", "MASTER_ADDR", "MASTER_PORT"):
        env.pop(k, None)
    r = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "3"], capture_output=True, text=True, env=env, timeout=580)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
