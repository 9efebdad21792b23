"""Host logic of the multi-GPU bench path, run as world-size-2 gloo ranks on
CPU: instances shard across ranks with no overlap and no data exchange, the
job time is the slowest rank's, and the per-instance results gathered from
the ranks in seed order are bitwise those of one rank running every instance
(each instance's problem, window objective included, does not depend on the
rank that runs it). The gradients come from the CPU oracle on a small mesh of
the benchmark's workload family; the GPU sharding itself is not measured on
hardware (one GPU per run)."""
import os
import socket
import sys

import numpy as np
import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NE, NSTEPS = 6, 3


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _gradients(first, B):
    """J and dJ/dq0 of instances first .. first + B - 1 (oracle, 6^2 P3, Chebyshev 5)."""
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import bench
    import igr_sensitivities_gb300 as igr
    import oracle_lib as O
    from igr_sensitivities_gb300 import workloads as W
    basis, mesh, q0, gam, alp, dts, prm = bench.make_batch(igr, W, B, first=first, ne=NE)
    G = O.Grid2D(bench.P, NE, NE)
    J, dq = np.zeros(B), np.zeros_like(q0)
    for b in range(B):
        J[b], g, _, _ = O.adjoint_2d(G, gam[b], alp[b], NSTEPS, float(dts[b]), bench.N_ITER, bench.SOLVER, bench.OBJ,
                                     list(q0[b]), prm)
        dq[b] = np.stack(g)
    return J, dq


def _rank(rank, world, port, B, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        seeds = bench.instance_seeds(rank, B)
        J, dq = _gradients(seeds[0], B)
        allseeds, (Jall, dqall) = bench.gather_by_seed(dist, seeds, J, dq)
        tmax = bench.max_over_ranks(1.0 + rank * 0.5, dist, None)
        q.put((rank, allseeds, tmax, Jall, dqall))
    finally:
        dist.destroy_process_group()


def test_two_ranks_shard_instances_gather_results_and_take_max_time():
    sys.path.insert(0, ROOT)
    import bench
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    B = 3
    procs = [ctx.Process(target=_rank, args=(r, 2, port, B, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=300) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    J1, dq1 = _gradients(0, 2 * B)  # one rank, every instance
    for rank, allseeds, tmax, Jall, dqall in out:
        assert allseeds == bench.instance_seeds(0, 2 * B)  # disjoint shards that cover the job, in seed order
        assert tmax == pytest.approx(1.5)                   # slowest rank
        assert np.array_equal(Jall, J1) and np.array_equal(dqall, dq1)
