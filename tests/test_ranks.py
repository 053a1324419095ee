"""Multi-rank host logic on CPU (gloo, world size 2): the body sharding of the
batched workload and the max-over-ranks timing that the benchmark uses under
torchrun.  No GPU: ranks are CPU processes, the collectives run on gloo."""
import os
import socket

import pytest

from andromeda_gb300 import ranks


def test_shard_partitions_every_body_once():
    for n in (0, 1, 7, 512):
        for world in (1, 2, 3, 8):
            got = sorted(i for r in range(world) for i in ranks.shard(n, world, r))
            assert got == list(range(n))
    with pytest.raises(ValueError):
        ranks.shard(10, 2, 2)


def test_single_process_identity():
    assert ranks.max_over_ranks([1.5, 2.0]) == [1.5, 2.0]
    ranks.barrier()  # no process group: a no-op


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, local = ranks.dist_env()
        mine = ranks.shard(11, w, r)
        ranks.barrier()
        # rank r "took" (r + 1) x 1.5 s of device time and 10 - r s of wall time
        dev, wall = ranks.max_over_ranks([(r + 1) * 1.5, 10.0 - r])
        everyone = [None] * w
        dist.all_gather_object(everyone, mine)
        q.put((r, w, local, mine, dev, wall, everyone))
    finally:
        dist.destroy_process_group()


def test_gloo_world_size_2():
    import multiprocessing as mp
    pytest.importorskip("torch.distributed")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = [q.get(timeout=120) for _ in ps]
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    for r, (rank, world, local, mine, dev, wall, everyone) in enumerate(out):
        assert (rank, world, local) == (r, 2, r)
        assert mine == list(range(r, 11, 2))
        assert dev == 3.0 and wall == 10.0  # the slowest rank's device time, the longest wall time
        assert sorted(i for part in everyone for i in part) == list(range(11))
