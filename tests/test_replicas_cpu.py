"""The replica path of bench.py (one independent sweep per rank, the step
time taken as the slowest rank's) on two gloo ranks, CPU only."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        # rank r: (r + 1, 10 - r, 5): the maximum over ranks is (ws, 10, 5)
        out = bench.max_over_ranks([rank + 1.0, 10.0 - rank, 5.0], ws, "cpu")
        q.put((rank, out))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks():
    ws = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, ws, port, q)) for r in range(ws)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in range(ws))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in range(ws):
        assert res[r] == [2.0, 10.0, 5.0]


def test_max_over_ranks_one_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks([3, 1.5], 1, "cpu") == [3.0, 1.5]
