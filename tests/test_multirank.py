"""The N > 1 path of bench.py on the host: replicas only (no data-path
collective), one process per rank, the job timed by its slowest rank.  Runs
as world-size-2 gloo process groups on the CPU."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
torch = pytest.importorskip("torch")


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    # rank r took (r + 1) seconds: the job takes the slowest rank's time
    t = bench.max_over_ranks(dist, float(rank + 1))
    rate = bench.job_rate(world, 1000, 2, 5, t)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, t, rate))


def test_slowest_rank_times_the_job():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    for rank, t, rate in res:
        assert t == 2.0
        assert rate == 2 * 1000 * 2 * 5 / 2.0


def test_without_process_group_nothing_is_reduced():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(None, 3.5) == 3.5


def test_reference_arm_under_torchrun_prints_once():
    """`bench.py --impl reference` launched on two ranks: rank 0 times the
    reference's CPU path and prints one JSON line; rank 1 exits 0 without work."""
    port = free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "3", "--cpu-size", "12"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    out = json.loads(lines[0])
    assert out["impl"] == "reference" and out["n_gpus"] == 2 and out["value"] > 0
    assert out["config"]["parallelism"] == "replicas"
