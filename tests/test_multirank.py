"""Multi-rank path on CPU (gloo, world size 2): worlds are sharded across
ranks with no data exchange, each rank steps its shard (here with the CPU
oracle, as a stand-in for its GPU), and rank 0 gathers the results, which
must equal a single-process run bit for bit."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def test_shard_covers_every_world_once_and_balances():
    from bendy2d_gb300.sharding import shard
    rng = np.random.default_rng(0)
    costs = np.exp(rng.uniform(np.log(64), np.log(4096), size=500))
    for n in (1, 2, 3, 8):
        parts = shard(costs, n)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(costs)))
        loads = [costs[p].sum() for p in parts]
        assert max(loads) <= min(loads) + costs.max()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world_size, port, q):
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world_size)
    from bendy2d_gb300 import scenes
    from bendy2d_gb300.sharding import shard, world_cost
    from oracle import load_scene
    worlds = scenes.config3(seed=2, n_worlds=12, lo=64, hi=400)
    mine = shard([world_cost(w) for w in worlds], world_size)[rank]
    results = {}
    for i in mine:
        o = load_scene(worlds[i])
        o.update(worlds[i].dt)
        results[i] = o.particles()[0].tobytes()
    gathered = [None] * world_size if rank == 0 else None
    dist.gather_object(results, gathered, dst=0)
    if rank == 0:
        merged = {}
        for part in gathered:
            assert not (set(part) & set(merged))
            merged.update(part)
        q.put(merged)
    dist.destroy_process_group()


def test_two_rank_shards_match_single_process():
    from bendy2d_gb300 import scenes
    from oracle import load_scene
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    merged = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    worlds = scenes.config3(seed=2, n_worlds=12, lo=64, hi=400)
    assert sorted(merged) == list(range(len(worlds)))
    for i, w in enumerate(worlds):
        o = load_scene(w)
        o.update(w.dt)
        assert merged[i] == o.particles()[0].tobytes()
