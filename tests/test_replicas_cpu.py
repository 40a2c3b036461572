"""Several replicas as gloo ranks on the CPU: each rank takes its own share
of a batch of scenes, steps it with the CPU oracle (no collective on the
data path), and the ranks agree on the job's time as the maximum of theirs.
The union of the shards' results equals one process stepping every scene."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _scenes():
    from collision_gb300 import scenes
    return [scenes.cloth_on_obstacle(8 + 2 * i, "sphere" if i % 2 else "box", 0.2, 1.5 + i, seed=i)
            for i in range(5)]


def _step_all(scs, nsteps):
    from oracle.ccopy import OracleSolver
    out = []
    for sc in scs:
        o = OracleSolver(sc, record=0)
        x, v, hc = sc.x.copy(), sc.v.copy(), np.zeros(sc.nv, np.uint8)
        for _ in range(nsteps):
            r = o.step(x, x + sc.params["dt"] * v, v, hc)
            assert r["rc"] == 0
            x, v, hc = r["x"], r["v"], r["has_collsn"]
        out.append(x)
    return out


def _rank_main(rank, world, port, outdir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist
    from collision_gb300.replicas import dist_env, max_over_ranks, shard, sum_over_ranks
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ws, rk, _ = dist_env()
    mine = shard(_scenes(), rk, ws)
    res = _step_all(mine, 3)
    t = max_over_ranks(1.0 + rk)
    n = sum_over_ranks(len(mine))
    np.savez(os.path.join(outdir, f"r{rk}.npz"), t=t, n=n, *res)
    dist.barrier()
    dist.destroy_process_group()


def test_shards_cover_and_partition():
    from collision_gb300.replicas import shard
    items = list(range(11))
    parts = [shard(items, r, 4) for r in range(4)]
    assert sum(parts, []) == items
    assert max(map(len, parts)) - min(map(len, parts)) <= 1


def test_two_gloo_ranks_step_their_shards(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn", join=True)
    ref = _step_all(_scenes(), 3)
    got = []
    for rk in range(2):
        z = np.load(tmp_path / f"r{rk}.npz")
        assert float(z["t"]) == 2.0          # max over ranks of 1 + rank
        assert int(z["n"]) == len(ref)       # every scene stepped by exactly one rank
        got += [z[k] for k in sorted(z.files, key=lambda s: (len(s), s)) if k.startswith("arr_")]
    assert len(got) == len(ref)
    for a, b in zip(got, ref):
        assert np.array_equal(a, b)
