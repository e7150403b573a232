"""The replica timing of bench.py --gpus N over a real process group, on CPU.

Under torchrun each rank runs its own batch of segments on its own GPU and
the ranks exchange nothing inside a sweep; the job's time is the slowest
rank's (barrier, then an all-reduce MAX) and the job's rate counts every
rank's segments.  Two gloo ranks on 127.0.0.1 exercise exactly those calls.
"""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = bench.max_over_replicas(100.0 + 50.0 * rank, dist)
        q.put((rank, ms, bench.replica_value(world, 64, 10, ms)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_replicas_take_the_slowest_rank():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as tmp
    ctx = tmp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[1] for g in got] == [150.0, 150.0]
    # 2 ranks x 64 segments x 10 steps in 0.150 s
    assert all(abs(g[2] - 2 * 64 * 10 / 0.150) < 1e-9 for g in got)


def test_single_process_keeps_its_own_time():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.max_over_replicas(42.0, None) == 42.0
    assert bench.replica_value(1, 64, 20, 1000.0) == 64 * 20
