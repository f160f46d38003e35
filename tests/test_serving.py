"""Serving: continuous batching of world-solve requests (configuration 4).

Each request's result must be the same alone and in a mix (bit-exact: every
world is computed independently and particle contacts are summed in fixed
point), equal to the oracle running the same updates (a request is that
many Solver::update calls, src/solver.rs:106-116), and admission must
respect the device-memory budget and the residency limit.  Cancellation and
an injected allocation failure drop only the request concerned."""
import numpy as np
import pytest

from helpers import assert_same_state, oracle_state, solver_state

pytestmark = pytest.mark.gpu


def _pool(n, seed, lo=64, hi=2000):
    from bendy2d_gb300.serving import request_pool
    return request_pool(n, seed, lo, hi)


def _run(server, items, expect_missing=()):
    """submit (world, steps) items, wait, return final solvers by index
    (items listed in expect_missing must finish without a result)"""
    import time
    from bendy2d_gb300 import B2DError
    ids = {server.submit(w.to_solver(), k, w.dt): i for i, (w, k) in enumerate(items)}
    out, gone = {}, set()
    t_end = time.time() + 120
    while len(out) + len(gone) < len(ids) and time.time() < t_end:
        for rid in server.finished():
            try:
                s, lat, q = server.take(rid)
            except B2DError as e:
                assert e.code == 11  # failed or cancelled: B2D_ERR_STATE
                gone.add(ids[rid])
                continue
            assert lat >= q >= 0.0
            out[ids[rid]] = s
        time.sleep(0.002)
    assert len(out) + len(gone) == len(ids)
    assert gone == set(expect_missing), (gone, expect_missing)
    return out


def _oracle_after(world, steps):
    from oracle import load_scene
    o = load_scene(world)
    for _ in range(steps):
        assert o.update(world.dt) == 0
    return o


def _big_world():
    """A configuration-4-style request whose 100x100 cloth (10,000 particles,
    39,402 links) does not fit one CTA's shared memory with its links and
    schedule (large-body executor), with particle collisions."""
    from bendy2d_gb300 import scenes
    from bendy2d_gb300.scenes import COLLIDE_PP
    rng = np.random.default_rng(21)
    body = scenes.grid_body(100, 100, (300.0, 400.0), 1.0, 0.01, rng)
    sc = scenes._assemble("big_request", [body], bounds=(0.0, 0.0, 2000.0, 2000.0), sub_steps=8,
                          link_iters=4, collide=COLLIDE_PP)
    sc.prev = scenes._velocity_prev(sc.pos, rng, 0.5, (1.0 / 60.0) / 8.0)
    return sc


def test_served_results_match_oracle_alone_and_in_mix(gpu):
    """Configuration-4 request worlds (grids of log-uniform size with
    particle collisions, one over a CTA's shared memory) served alone and in
    a mix of 25 requests: every result equals the oracle's bit for bit."""
    from bendy2d_gb300.serving import Server
    pool = _pool(24, seed=31, lo=64, hi=3000)
    big = _big_world()
    assert big.to_solver().plan_stats()["large_bodies"] == 1
    items = [(w, 2 + (i * 5) % 7) for i, w in enumerate(pool)] + [(big, 3)]
    sv = Server(1 << 33)
    sv.start()
    alone = {i: _run(sv, [items[i]])[0] for i in (0, 7, len(items) - 1)}
    mixed = _run(sv, items)
    sv.stop()
    sv.close()
    for i, (w, k) in enumerate(items):
        assert_same_state(solver_state(mixed[i]), oracle_state(_oracle_after(w, k)),
                          f"request {i} ({w.n_particles} particles, {k} steps) in the mix")
    for i, s in alone.items():
        assert_same_state(solver_state(s), solver_state(mixed[i]), f"request {i} alone vs mix")


def test_residency_limit_bounds_resident_particles(gpu):
    """With a residency limit the worker never holds more solver particles
    than the limit (beyond the one request always admitted onto an idle
    device), and every request still completes with the oracle's result."""
    import threading
    import time
    from bendy2d_gb300.serving import Server
    pool = _pool(10, seed=41, lo=500, hi=1500)
    limit = 2500
    sv = Server(1 << 33)
    sv.set_max_resident_particles(limit)
    sv.start()
    peak = [0]
    stop = threading.Event()

    def watch():
        while not stop.is_set():
            peak[0] = max(peak[0], sv.stats()["resident_particles"])
            time.sleep(0.0005)

    th = threading.Thread(target=watch, daemon=True)
    th.start()
    items = [(w, 3) for w in pool]
    res = _run(sv, items)
    stop.set()
    th.join()
    st = sv.stats()
    sv.stop()
    sv.close()
    assert peak[0] <= max(limit, max(w.n_particles for w in pool))
    assert st["resident_particles"] == 0 and st["completed"] == len(items)
    for i in (0, 5, 9):
        assert_same_state(solver_state(res[i]), oracle_state(_oracle_after(*items[i])),
                          f"request {i} under the residency limit")


def test_cancelled_requests_leave_the_others_exact(gpu):
    """Cancel one request while queued and one while running: both finish as
    cancelled (take reports B2D_ERR_STATE), the rest equal the oracle."""
    import time
    from bendy2d_gb300 import B2DError
    from bendy2d_gb300.serving import CANCELLED, Server
    pool = _pool(6, seed=51, lo=200, hi=800)
    sv = Server(1 << 33)
    long_id = sv.submit(pool[0].to_solver(), 5000, pool[0].dt)  # runs for a while
    ids = [sv.submit(w.to_solver(), 3, w.dt) for w in pool[1:]]
    sv.cancel(ids[2])  # still queued: the worker has not started
    assert sv.poll(ids[2]) == CANCELLED
    sv.start()
    t_end = time.time() + 60
    while sv.poll(long_id) != 1 and time.time() < t_end:  # wait until it is RUNNING
        time.sleep(0.001)
    sv.cancel(long_id)
    got, gone = {}, set()
    while len(got) + len(gone) < 6 and time.time() < t_end:
        for rid in sv.finished():
            if sv.poll(rid) == CANCELLED:
                gone.add(rid)
                with pytest.raises(B2DError) as e:
                    sv.take(rid)
                assert e.value.code == 11
            else:
                got[rid] = sv.take(rid)[0]
        time.sleep(0.002)
    st = sv.stats()
    sv.stop()
    sv.close()
    assert gone == {long_id, ids[2]}
    assert st["cancelled"] == 2 and st["completed"] == 4 and st["resident_particles"] == 0
    for k, rid in enumerate(ids):
        if rid != ids[2]:
            assert_same_state(solver_state(got[rid]), oracle_state(_oracle_after(pool[k + 1], 3)),
                              f"request {k + 1} beside cancelled ones")
    with pytest.raises(B2DError):
        sv2 = Server(1 << 20)
        try:
            sv2.cancel(12345)  # unknown id
        finally:
            sv2.close()


def test_injected_allocation_failure_fails_only_that_request(gpu):
    """A device allocation that fails at admission (injected on the host)
    fails that request alone; the server keeps serving the others exactly."""
    from bendy2d_gb300._native import FAULT_ALLOC
    from bendy2d_gb300.serving import Server
    pool = _pool(5, seed=61, lo=200, hi=900)
    sv = Server(1 << 33)
    sv.set_fault(FAULT_ALLOC, 1)  # the first request installed fails
    items = [(w, 2) for w in pool]
    import time
    ids = [sv.submit(w.to_solver(), k, w.dt) for w, k in items]
    sv.start()
    out, failed = {}, []
    t_end = time.time() + 60
    from bendy2d_gb300 import B2DError
    while len(out) + len(failed) < len(ids) and time.time() < t_end:
        for rid in sv.finished():
            try:
                out[rid] = sv.take(rid)[0]
            except B2DError as e:
                assert e.code == 11 and "injected" in str(e)
                failed.append(rid)
        time.sleep(0.002)
    st = sv.stats()
    sv.stop()
    sv.close()
    assert failed == [ids[0]]
    assert st["failed"] == 1 and st["completed"] == 4 and st["resident_bytes"] == 0
    for k in range(1, 5):
        assert_same_state(solver_state(out[ids[k]]), oracle_state(_oracle_after(*items[k])),
                          f"request {k} after a failed admission")


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
