"""bench.py's multi-rank logic on CPU: the max over ranks with 2 gloo ranks,
the replica arithmetic, and the reference arm under a 2-process torchrun
(rank 0 prints the one JSON line, rank 1 exits without work)."""
import json
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT

sys.path.insert(0, ROOT)
import bench  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        q.put((rank, bench.world_max(10.0 + 5.0 * rank, dist, "cpu")))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_world_max_over_two_gloo_ranks():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
        assert p.exitcode == 0
    got = dict(q.get(timeout=10) for _ in range(2))
    assert got == {0: 15.0, 1: 15.0}


def test_world_max_without_group_and_replica_value():
    assert bench.world_max(3.5, None, "cpu") == 3.5
    # two replicas of 1 GB each in 1 ms: 2000 GB/s for the job
    assert bench.replica_value(1e9, 2, 1.0) == pytest.approx(2000.0)
    assert bench.replica_value(1e9, 1, 1.0) == pytest.approx(1000.0)


def test_reference_arm_under_two_rank_torchrun():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--gpus", "2", "--impl", "reference", "--steps", "2", "--warmup", "1", "--cols", "4096"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    lines = [json.loads(ln) for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = lines[0]
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["steps"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0
