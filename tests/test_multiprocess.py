"""The N > 1 path of bench.py on the CPU: independent replicas joined by a gloo process group
(world size 2, 127.0.0.1): a barrier, the maximum of the per-rank times, and the reference arm
running on rank 0 only."""

import multiprocessing as mp
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _replica(rank: int, world: int, port: int, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench
    try:
        w, r, local = bench.dist_setup()
        t = bench.dist_max(1.5 * (rank + 1), w)
        bench.barrier(w)
        # the reference arm returns at once on every rank but 0 (rank 0 alone times the host path)
        class A:
            steps, warmup, gpus = 1, 3, world
        ran = None
        if rank != 0:
            ran = bench.bench_reference(A, w, r)
        q.put((rank, w, r, local, t, ran))
    finally:
        if dist.is_initialized():
            dist.destroy_process_group()


def test_replicas_join_with_max_over_ranks():
    pytest.importorskip("torch")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_replica, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1]
    assert all(o[1] == 2 for o in out)
    # every rank sees the slowest rank's time
    assert all(o[4] == 3.0 for o in out)
    assert out[1][5] is None
