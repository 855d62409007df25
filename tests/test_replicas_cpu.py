"""The N > 1 path of bench.py on CPU: ranks as gloo processes (world size 2). The path is
replicas (independent simulations, no data-path collective): the job's value is the sum of
the ranks' bond-updates over the slowest rank's time, and the reference arm runs on rank 0
only."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import bench
    dist = bench.dist_setup(world, "gloo")
    bench.barrier(dist)
    total = bench.sum_over_ranks(dist, 1.0e9 * (rank + 1))
    slowest = bench.max_over_ranks(dist, 10.0 * (rank + 1))
    q.put((rank, total, slowest))
    dist.destroy_process_group()


def test_replica_aggregation_over_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == [(0, 3.0e9, 20.0), (1, 3.0e9, 20.0)]


def test_reference_arm_prints_once_under_torchrun(tmp_path):
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), str(ROOT / "bench.py"), "--impl", "reference",
           "--gpus", "2", "--steps", "2", "--warmup", "1", "--cpu-budget", "1", "--workload", "two_sphere"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=tmp_path)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["n_gpus"] == 2
