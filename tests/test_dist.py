"""bench.py's multi-process helpers with two gloo ranks on the CPU: replicas
take the maximum time over ranks and sum the pixels of all ranks."""
import os
import socket
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench.barrier(world)
        mx = bench.reduce_max(1.5 + rank, world, "gloo")
        sm = bench.reduce_sum(10.0 * (rank + 1), world, "gloo")
        q.put((rank, mx, sm))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_reduce_max_and_sum():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == [(0, 2.5, 30.0), (1, 2.5, 30.0)]
