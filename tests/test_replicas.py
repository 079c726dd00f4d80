"""More than one GPU runs as independent replicas (the index replicated, no data-path exchange):
bench.py's rank helpers -- barrier, maximum over ranks, whole-job throughput -- under a gloo
world of 2 on the CPU, and the reference arm under torchrun, where rank 0 alone measures and
prints."""
import json
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench.rank_barrier()
        slowest = bench.rank_max(10.0 + 5.0 * rank)          # per-step ms of each replica
        q.put((rank, slowest, bench.replica_throughput(1000, world, slowest)))
        bench.rank_barrier()
    finally:
        dist.destroy_process_group()


def test_replica_helpers_gloo_world2():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=5) for _ in range(world))
    # every rank sees the slowest replica's time; the job throughput counts all ranks' reads
    assert [g[1] for g in got] == [15.0, 15.0]
    assert all(g[2] == pytest.approx(2 * 1000 / 15e-3) for g in got)


def test_rank_helpers_single_process():
    sys.path.insert(0, ROOT)
    import bench
    bench.rank_barrier()
    assert bench.rank_max(3.5) == 3.5
    assert bench.replica_throughput(500, 1, 2.0) == pytest.approx(250000.0)


def test_reference_arm_under_torchrun_world2():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--gpus", "2", "--impl", "reference", "--steps", "1", "--warmup", "1", "--cpu-scale",
           "0.005", "--cpu-seconds", "1"]
    r = subprocess.run(cmd, capture_output=True, text=True, cwd=ROOT, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip().startswith("{")]
    assert len(lines) == 1, r.stdout
    out = json.loads(lines[0])
    assert out["impl"] == "reference" and out["n_gpus"] == 2 and out["value"] > 0
