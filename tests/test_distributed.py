"""bench.py's multi-rank reduction (replicas: barrier, max of times, sum of pairs) on two
gloo ranks over 127.0.0.1, without a GPU."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import bench

    D = bench.Dist(world)
    D.barrier()
    q.put((rank, D.max(1.0 + rank), D.sum(10 * (rank + 1))))
    D.close()


def test_two_rank_reduction():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert got == [(0, 2.0, 30.0), (1, 2.0, 30.0)]


def test_rank_device_selection():
    """Under torchrun every rank keeps one GPU visible: its entry of CUDA_VISIBLE_DEVICES."""
    sys.path.insert(0, ROOT)
    import bench

    assert bench.rank_visible_device(1, "0,1,2,3") == "1"
    assert bench.rank_visible_device(2, "4, 5,6") == "6"
    assert bench.rank_visible_device(3, None) == "3"
    assert bench.rank_visible_device(0, "") == "0"
    assert bench.rank_visible_device(3, "7,6") == "6"
