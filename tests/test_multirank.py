"""Multi-process host logic of the N-GPU bench path, on CPU with gloo.

Energies shard across ranks with no data-path collective (each (energy, k)
image is independent, src/cudaMain.cu:499-503); the only collective is the
max-over-ranks of the timed region.
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, energies, per_rank, q):
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = bench.shard_energies(energies, rank, world, per_rank)
    gathered = [None] * world
    dist.all_gather_object(gathered, mine)
    t = torch.tensor([10.0 * (rank + 1)])
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    if rank == 0:
        q.put((gathered, float(t.item())))
    dist.destroy_process_group()


@pytest.mark.parametrize("world,per_rank", [(2, 3), (2, 8)])
def test_energy_shards_are_disjoint_and_timing_is_max(world, per_rank):
    energies = [270.0 + i for i in range(5)]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    mp.spawn(_worker, args=(world, port, energies, per_rank, q), nprocs=world, join=True)
    gathered, tmax = q.get(timeout=60)
    flat = [e for part in gathered for e in part]
    assert len(flat) == world * per_rank
    assert len(set(flat)) == len(flat)  # disjoint shards
    assert all(len(p) == per_rank for p in gathered)  # weak scaling: fixed work per rank
    assert tmax == 10.0 * world
