"""The replicas path on CPU: two gloo ranks run the bench's rendezvous and max-over-ranks
timing, and shard a batch of meshes between them with no data-path collective."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, costs, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    from lmtpp_gb300.batch import shard
    r, w, local, barrier, allmax = bench.dist_setup(world)
    assert (r, w, local) == (rank, world, rank)
    barrier()
    a, b = shard(costs, r, w)
    t = allmax(10.0 * (r + 1))  # each rank's "time"; the bench reports the max
    shares = [None] * w
    dist.all_gather_object(shares, (a, b))
    out[rank] = (t, shares)
    dist.destroy_process_group()


def test_two_gloo_ranks_rendezvous_time_and_shard():
    world = 2
    rng = np.random.default_rng(20251203)
    sides = rng.integers(8, 33, 256)
    costs = ((sides + 1) ** 3).tolist()
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_rank_main, args=(world, _free_port(), costs, out), nprocs=world, join=True,
                       start_method="spawn")
    for rank in range(world):
        t, shares = out[rank]
        assert t == 20.0  # max over ranks
        assert shares == out[0][1]
    shares = out[0][1]
    assert shares[0][0] == 0 and shares[-1][1] == 256
    assert all(shares[k][1] == shares[k + 1][0] for k in range(world - 1))
    loads = [sum(costs[a:b]) for a, b in shares]
    assert max(loads) <= 1.05 * sum(costs) / world


def test_shard_covers_every_mesh_once():
    from lmtpp_gb300.batch import shard
    costs = [5, 1, 1, 1, 9, 2, 2, 3]
    for world in (1, 2, 3, 8, 12):
        parts = [shard(costs, r, world) for r in range(world)]
        covered = [i for a, b in parts for i in range(a, b)]
        assert covered == list(range(len(costs)))
