"""Multi-process logic of bench.py on CPU (two gloo ranks): the job time is the
maximum over ranks, counts add up, and ensemble models are sharded over
ranks without overlap (no data-path collective)."""
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


def _worker(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t = bench.max_over_ranks(1.5 + rank, world, "cpu")
        mine = bench.shard(list(range(11)), rank, world)
        n = bench.sum_over_ranks(len(mine), world, "cpu")
        gathered = [None] * world
        dist.all_gather_object(gathered, mine)
        out.put((rank, t, n, gathered))
    finally:
        dist.destroy_process_group()


def test_two_rank_reductions_and_sharding():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, n, gathered in results:
        assert t == 2.5                      # max over ranks
        assert n == 11                       # every model counted once
        flat = sorted(x for part in gathered for x in part)
        assert flat == list(range(11))       # disjoint shards covering all models
        assert gathered[0] == list(range(0, 11, 2)) and gathered[1] == list(range(1, 11, 2))


def test_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(3.0, 1) == 3.0
    assert bench.sum_over_ranks(4, 1) == 4
    assert bench.shard([1, 2, 3], 0, 1) == [1, 2, 3]
