"""Scene sharding across ranks (opendeformer_gb300.sharding), on CPU.

The partition is a function of the scenes' work alone, so every rank
computes the same one without communicating; shards are disjoint and cover
the batch; and two gloo ranks that each step only their shard produce, for
every scene, bit for bit what one process stepping all scenes produces (the
stepping engine here is the oracle's restatement, which runs on CPU; on the
GPU each rank steps its shard as one od_batch)."""
import os
import socket

import numpy as np
import pytest

from opendeformer_gb300 import meshgen, sharding


def test_shards_cover_the_batch_once_and_balance_work():
    insts = meshgen.batch_instances(512)
    work = [6 * int(np.prod(i["dims"])) for i in insts]
    for world in (1, 2, 3, 4, 8):
        shards = sharding.shard_scenes(work, world)
        flat = sorted(i for s in shards for i in s)
        assert flat == list(range(len(work)))
        assert shards == sharding.shard_scenes(work, world)   # deterministic
        assert all(sharding.my_shard(work, r, world) == shards[r] for r in range(world))
        assert sharding.imbalance(work, world) <= 1.02
    with pytest.raises(ValueError):
        sharding.my_shard(work, 2, 2)


SMALL = [dict(dims=(4, 2, 2), kind="corotational", E=2e5, nu=0.4, seed=1),
         dict(dims=(3, 3, 2), kind="neohookean", E=5e4, nu=0.45, seed=2),
         dict(dims=(5, 2, 2), kind="corotational", E=1e6, nu=0.3, seed=3),
         dict(dims=(2, 2, 4), kind="neohookean", E=2e4, nu=0.35, seed=4),
         dict(dims=(3, 2, 3), kind="neohookean", E=3e5, nu=0.48, seed=5)]


def step_scene(k, steps=3):
    """Newmark steps of SMALL[k] under gravity with the oracle restatement."""
    from oracle import restated as O
    inst = SMALL[k]
    g = meshgen.tet_grid(*inst["dims"], h=0.05, jitter=0.1, seed=inst["seed"])
    cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
    o = O.OracleScene(g.X, g.tets, g.facets, cd, inst["kind"], 1000.0, inst["E"], inst["nu"], 0.1)
    o.integrator_setup(1 / 60, 0.01, 0.001, newton=1, tol=1e-8, maxit=2000, precond="block_jacobi")
    o.set_fext(o.loads(body=[0.0, 0.0, -9800.0]))
    o.nm_step(steps)
    u = o.displacements()
    o.close()
    return u


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    work = [6 * int(np.prod(i["dims"])) for i in SMALL]
    mine = sharding.my_shard(work, rank, world)
    res = {k: step_scene(k) for k in mine}       # no exchange while stepping
    gathered = [None] * world
    dist.all_gather_object(gathered, res)        # only to check the results
    if rank == 0:
        merged = {}
        for part in gathered:
            assert not set(part) & set(merged)
            merged.update(part)
        np.savez(os.path.join(out_dir, "sharded.npz"), **{str(k): v for k, v in merged.items()})
    dist.barrier()
    dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_step_their_shards_like_one_process(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as tmp
    world = 2
    tmp.spawn(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    sharded = np.load(tmp_path / "sharded.npz")
    assert sorted(int(k) for k in sharded.files) == list(range(len(SMALL)))
    for k in range(len(SMALL)):
        alone = step_scene(k)
        assert np.abs(alone).max() > 0
        assert np.array_equal(sharded[str(k)], alone), k
    del torch
