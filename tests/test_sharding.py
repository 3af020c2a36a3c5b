"""Multi-rank host logic on CPU: the terrain split, and a world_size-2 gloo
run in which each rank erodes its own terrains of a batch (oracle on the
CPU) and the gathered results equal one process eroding the whole batch."""
import os
import socket

import numpy as np
import pytest

from simplehydrology_gb300 import sharding as sh


def test_batch_workload_shape():
    specs = sh.batch_workload(64)
    assert len(specs) == 64
    sides = [t.nx for t in specs]
    assert min(sides) >= 128 and max(sides) <= 1024
    assert any(s & (s - 1) for s in sides)  # non-powers of two occur
    assert [t.seed for t in specs] == [1000 + i for i in range(64)]
    assert all(t.drops == round(0.25 * t.cells) for t in specs)
    assert sh.batch_workload(64) == specs  # seeded


@pytest.mark.parametrize("world_size", [1, 2, 3, 4, 8])
def test_shard_is_a_balanced_partition(world_size):
    specs = sh.batch_workload(64)
    costs = [sh.terrain_cost(t) for t in specs]
    parts = sh.shard(costs, world_size)
    flat = sorted(i for p in parts for i in p)
    assert flat == list(range(64))
    loads = [sum(costs[i] for i in p) for p in parts]
    # longest-processing-time: the spread is at most the largest item
    assert max(loads) - min(loads) <= max(costs) + 1e-6
    assert sh.shard(costs, world_size) == parts  # deterministic


def test_shard_edge_cases():
    assert sh.shard([], 3) == [[], [], []]
    assert sh.shard([5.0], 4) == [[0], [], [], []]
    with pytest.raises(ValueError):
        sh.shard([1.0], 0)
    with pytest.raises(ValueError):
        sh.shard([float("nan")], 2)
    with pytest.raises(ValueError):
        sh.rank_terrains(sh.batch_workload(2), 2, 2)


def test_aggregate_single_process():
    assert sh.aggregate(10, 2.5) == (10.0, 2.5)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world_size, port, specs, out_dir):
    import torch.distributed as dist

    from oracle import pyoracle as po
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world_size)
    mine = sh.rank_terrains(specs, world_size, rank)
    results = {}
    steps = 0
    for t in mine:
        m = po.Maps(t.nx, t.ny, height=po.value_noise(t.nx, t.ny, t.seed))
        acc = po.erode_batched(m, t.seed, 0, t.drops, 2)
        steps += acc.steps
        results[t.index] = np.asarray(m.height).copy()
    gathered = [None] * world_size
    dist.all_gather_object(gathered, results)
    units, secs = sh.aggregate(steps, 1.0 + rank, dist)
    if rank == 0:
        allres = {}
        for g in gathered:
            assert not set(g) & set(allres)  # no terrain on two ranks
            allres.update(g)
        np.savez(os.path.join(out_dir, "ranks.npz"), units=units, secs=secs,
                 **{f"t{i}": h for i, h in allres.items()})
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_gloo_batch_equals_single_process(po, tmp_path):
    import torch.multiprocessing as mp
    specs = [sh.TerrainSpec(i, n, n, 1000 + i, max(1, n * n // 4)) for i, n in enumerate([24, 40, 33, 17, 48])]
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, specs, str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    got = np.load(tmp_path / "ranks.npz")
    assert float(got["secs"]) == 2.0  # the slowest rank
    steps = 0
    for t in specs:
        m = po.Maps(t.nx, t.ny, height=po.value_noise(t.nx, t.ny, t.seed))
        steps += po.erode_batched(m, t.seed, 0, t.drops, 2).steps
        assert np.array_equal(got[f"t{t.index}"].view(np.uint32), np.asarray(m.height).view(np.uint32))
    assert float(got["units"]) == steps
