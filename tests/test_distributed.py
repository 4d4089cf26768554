"""Multi-GPU host logic on CPU: two gloo ranks shard a view list and reduce
their rates (sum of pixels, slowest rank's time), as bench.py does under
torchrun. Nothing here touches a GPU."""
import os
import socket

import pytest

from futspace_gb300 import replicas


def test_shard_covers_exactly_once():
    items = list(range(513))
    for world in (1, 2, 3, 4, 8):
        parts = [replicas.shard(items, r, world) for r in range(world)]
        assert sum(parts, []) == items
        assert max(map(len, parts)) - min(map(len, parts)) <= 1
    with pytest.raises(ValueError):
        replicas.shard(items, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        views = [(w, h) for w, h in [(320, 240), (640, 480), (1920, 1080)] * 7]
        mine = replicas.shard(views, rank, world)
        pixels = sum(w * h for w, h in mine)
        ms = 10.0 + 5.0 * rank  # the slowest rank sets the job time
        out = replicas.aggregate(pixels, ms, dist=dist)
        gathered = [None] * world
        dist.all_gather_object(gathered, mine)
        q.put((rank, out, sum(gathered, []) == views))
    finally:
        dist.destroy_process_group()


def test_two_rank_aggregate_gloo():
    import torch.multiprocessing as mp

    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    total = sum(w * h for w, h in [(320, 240), (640, 480), (1920, 1080)] * 7)
    for rank, out, complete in res:
        assert complete
        assert out["world"] == 2 and out["pixels"] == total and out["ms"] == 15.0
        assert abs(out["gpix_s"] - total / 15.0 / 1e6) < 1e-9
