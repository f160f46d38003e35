"""Serving: continuous batching of world-solve requests (configuration 4).

Each request's result must be the same alone and in a mix (bit-exact: every
world is computed independently and particle contacts are summed in fixed
point), equal to running the same updates on a plain Solver, and admission
must respect the device-memory budget."""
import numpy as np
import pytest

from helpers import assert_same_state, solver_state

pytestmark = pytest.mark.gpu


def _pool(n, seed, lo=64, hi=2000):
    from bendy2d_gb300.serving import request_pool
    return request_pool(n, seed, lo, hi)


def _run(server, items):
    """submit (world, steps) items, wait, return final solvers by index"""
    import time
    ids = {server.submit(w.to_solver(), k, w.dt): i for i, (w, k) in enumerate(items)}
    out = {}
    t_end = time.time() + 120
    while len(out) < len(ids) and time.time() < t_end:
        for rid in server.finished():
            s, lat, q = server.take(rid)
            assert lat >= q >= 0.0
            out[ids[rid]] = s
        time.sleep(0.002)
    assert len(out) == len(ids)
    return out


def test_alone_equals_mix_equals_solver(gpu):
    from bendy2d_gb300.serving import Server
    pool = _pool(12, seed=3)
    target = pool[0]
    sv = Server(1 << 32)
    sv.start()
    alone = _run(sv, [(target, 9)])[0]
    mix_items = [(pool[i % len(pool)], 3 + (i * 7) % 11) for i in range(1, 24)]
    mix_items.insert(5, (target, 9))
    mixed = _run(sv, mix_items)[5]
    sv.stop()
    sv.close()
    direct = target.to_solver()
    for _ in range(9):
        direct.update(target.dt)
    assert_same_state(solver_state(alone), solver_state(mixed), "alone vs mix")
    assert_same_state(solver_state(alone), solver_state(direct), "served vs solver")


def test_budget_limits_residency(gpu):
    from bendy2d_gb300.serving import Server
    pool = _pool(6, seed=5, lo=1500, hi=2000)
    sv = Server(1 << 20)  # room for only a few worlds at a time
    sv.start()
    res = _run(sv, [(pool[i % 6], 4) for i in range(10)])
    st = sv.stats()
    sv.stop()
    sv.close()
    assert st["completed"] == 10 and st["failed"] == 0
    assert st["resident_bytes"] == 0
    assert len(res) == 10


def test_world_over_budget_is_rejected(gpu):
    from bendy2d_gb300 import B2DError
    from bendy2d_gb300.serving import Server
    pool = _pool(1, seed=7, lo=2000, hi=2001)
    sv = Server(1024)
    with pytest.raises(B2DError) as e:
        sv.submit(pool[0].to_solver(), 3, pool[0].dt)
    assert e.value.code == 9
    sv.close()


def test_poisson_smoke(gpu):
    from bendy2d_gb300.serving import run_poisson
    pool = _pool(8, seed=9, lo=64, hi=1000)
    r = run_poisson(lam=200.0, duration=0.5, seed=1, pool=8, steps_lo=5, steps_hi=20,
                    drain_s=60.0, scenes_pool=pool)
    assert r["completed"] == r["submitted"] > 0
    assert 0.0 < r["p50_latency_ms"] <= r["p99_latency_ms"]
