"""Host logic of the multi-GPU bench path, run as world-size-2 gloo ranks on
CPU: instances shard across ranks with no overlap and no data exchange, and
the job time is the slowest rank's."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, B, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        seeds = bench.instance_seeds(rank, B)
        allseeds = [None] * world
        dist.all_gather_object(allseeds, seeds)
        t = 1.0 + rank * 0.5
        tmax = bench.max_over_ranks(t, dist, None)
        q.put((rank, allseeds, tmax))
    finally:
        dist.destroy_process_group()


def test_two_ranks_shard_instances_and_take_max_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    B = 4
    procs = [ctx.Process(target=_rank, args=(r, 2, port, B, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, allseeds, tmax in out:
        flat = [s for ss in allseeds for s in ss]
        assert len(flat) == 2 * B and len(set(flat)) == 2 * B  # disjoint instance sets
        assert tmax == pytest.approx(1.5)                        # slowest rank
