"""The N > 1 path on CPU: two gloo ranks shard a batch of scenes, check the
shards are disjoint and complete, step their scenes with the oracle, and
reduce the timing frame (max time, summed body-steps) exactly as bench.py
does over NCCL."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from diomedes_gb300 import dist as dio_dist
from diomedes_gb300 import scenes


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_shard_scenes_is_balanced_disjoint_and_complete():
    costs = [int(np.exp(x)) for x in np.random.default_rng(1).uniform(np.log(16), np.log(2048), 64)]
    for ws in (1, 2, 3, 4):
        owned = dio_dist.shard_scenes(costs, ws)
        flat = sorted(s for o in owned for s in o)
        assert flat == list(range(len(costs)))
        loads = [sum(costs[s] for s in o) for o in owned]
        assert max(loads) - min(loads) <= max(costs)
    assert dio_dist.shard_scenes(costs, 2) == dio_dist.shard_scenes(costs, 2)


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import oracle_lib as O

        parts = [scenes.pyramid(levels=3), scenes.constraints_demo(), scenes.box_demo(count=16),
                 scenes.pyramid(levels=4)]
        for p in parts:
            p.options = parts[0].options
        batch = scenes.pack(parts)
        costs = dio_dist.scene_costs(batch.scene_offsets, batch.constraints)
        mine = dio_dist.shard_scenes(costs, world)[rank]
        bodies = 0
        for s in mine:
            w = O.World(parts[s] if parts[s].containers else scenes.Scene(
                parts[s].name, parts[s].bodies, parts[s].state, constraints=parts[s].constraints,
                containers=[batch.containers[s]], options=parts[s].options))
            w.step(batch.options, 2)
            bodies += parts[s].n
        t, units = dio_dist.frame(dist, 10.0 + rank, bodies * 2)
        q.put((rank, sorted(mine), t, units))
    finally:
        dist.destroy_process_group()


def test_scene_split_is_contiguous_complete_and_rebased():
    """Scene.split (the batch held as several worlds): contiguous runs of whole
    scenes covering every body once, joints rebased into their run."""
    from diomedes_gb300 import scenes

    sc = scenes.batched(n_scenes=40, lo=16, hi=256, seed=7)
    for groups in (1, 3, 7, 40, 99):
        parts, starts = sc.split(groups)
        assert len(parts) == min(groups, sc.n_scenes)
        assert starts[0] == 0 and all(p.n > 0 for p in parts)
        assert [s + p.n for s, p in zip(starts, parts)][:-1] == starts[1:]
        assert starts[-1] + parts[-1].n == sc.n
        assert sum(p.n_scenes for p in parts) == sc.n_scenes
        assert sum(len(p.constraints) for p in parts) == len(sc.constraints)
        for p, lo in zip(parts, starts):
            assert np.array_equal(p.bodies.view(np.uint8), sc.bodies[lo:lo + p.n].view(np.uint8))
            assert p.scene_offsets[0] == 0 and p.scene_offsets[-1] == p.n
            assert len(p.containers) == p.n_scenes
            if len(p.constraints):
                assert p.constraints["a"].max() < p.n and p.constraints["b"].max() < p.n
    parts, _ = sc.split(4)
    assert max(p.n for p in parts) < 0.5 * sc.n  # balanced by bodies, not by scenes
    one = scenes.pyramid(levels=3)  # a single scene (no offsets) stays whole
    parts, starts = one.split(3)
    assert len(parts) == 1 and starts == [0] and parts[0].n == one.n


def test_two_gloo_ranks_shard_and_reduce():
    pytest.importorskip("torch")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    out = sorted(q.get(timeout=10) for _ in range(2))
    owned = [o[1] for o in out]
    assert sorted(owned[0] + owned[1]) == [0, 1, 2, 3] and not set(owned[0]) & set(owned[1])
    total_bodies = sum(p.n for p in [scenes.pyramid(levels=3), scenes.constraints_demo(), scenes.box_demo(count=16),
                                     scenes.pyramid(levels=4)])
    for rank, mine, t, units in out:
        assert t == 11.0  # max over ranks
        assert units == 2 * total_bodies  # every scene stepped twice, once, by one rank
