"""The benchmark's multi-process path on the CPU (gloo, world size 2): the replicas' barrier and
max over ranks, the whole-job rate from the slowest rank, and the reference arm under torchrun
(rank 0 alone runs and prints; the other rank exits 0 without work).  The GPU arm uses the same
rank_ops with NCCL, one replica per GPU and no collective on the data path."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist
    barrier, max_over_ranks = bench.rank_ops(world, rank, backend="gloo")
    barrier()
    ms = 100.0 + 50.0 * rank  # rank 1 is the slow replica
    ms_max = max_over_ranks(ms)
    value = bench.replica_rate(1000, 4, world, ms_max)
    barrier()
    out.put((rank, ms_max, value))
    dist.destroy_process_group()


def test_replicas_take_the_slowest_rank():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # every rank sees the slowest time; the rate counts both replicas' cells
    assert [g[1] for g in got] == [150.0, 150.0]
    assert all(abs(g[2] - 1000 * 4 * 2 / 0.150) < 1e-6 for g in got)


def test_reference_arm_under_torchrun_prints_once():
    pytest.importorskip("torch")
    port = free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl",
           "reference", "--gpus", "2", "--config", "c0", "--ref-window", "6", "--steps", "1",
           "--warmup", "1"]
    env = dict(os.environ, OMP_NUM_THREADS="2")
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port"
