"""GPU parity: the CUDA path through the C ABI against the CPU oracle.

Bar: bit-exact float32 (NaN-aware) in reference-order mode and in every
other mode against the oracle fed the same link order, which is stronger
than the 1e-5 (1 step) / 1e-3 (10 steps) relative tolerance the path is
specified with; the tolerance check is kept as a second assertion."""
import numpy as np
import pytest

from helpers import (assert_same_state, kat_cases, kat_to_solver, oracle_state, rel_err,
                     same_bits, solver_state)

pytestmark = pytest.mark.gpu
TOL_1 = 1e-5
TOL_10 = 1e-3
CASES = kat_cases()


def run_both(scene, steps, link_order=None, solver=None):
    from oracle import load_scene
    s = solver or scene.to_solver()
    o = load_scene(scene, link_order=link_order)
    for _ in range(steps):
        s.update(scene.dt)
        assert o.update(scene.dt) == 0
    return s, o


def check(scene, steps, what, link_order=None):
    s, o = run_both(scene, steps, link_order)
    g, r = solver_state(s), oracle_state(o)
    tol = TOL_1 if steps <= 1 else TOL_10
    assert rel_err(g[0], r[0]) <= tol, what
    assert_same_state(g, r, what)
    return s, o


@pytest.mark.parametrize("name", sorted(CASES))
def test_kat_on_gpu(gpu, name):
    from bendy2d_gb300 import B2DError
    case = CASES[name]
    s = kat_to_solver(case["scene"])
    if "expect_status" in case:
        with pytest.raises(B2DError) as e:
            s.update(case["scene"]["dt"])
        assert e.value.code == case["expect_status"]
        return
    for _ in range(case["steps"]):
        s.update(case["scene"]["dt"])
    if "expect_pos" in case:
        pos, prev = s.read_state()
        assert same_bits(pos, case["expect_pos"]), (pos, case["expect_pos"])
        assert same_bits(prev, case["expect_prev"])
    if "expect_circles_pos" in case:
        cs = s.get_circles()
        assert same_bits([c.point.pos for c in cs], case["expect_circles_pos"])
        assert same_bits([c.point.prev_pos for c in cs], case["expect_circles_prev"])
    if "expect_polygons" in case:
        for g, e in zip(s.get_polygons(), case["expect_polygons"]):
            assert same_bits([p.pos for p in g.particles], e["pos"])
            assert same_bits([p.prev_pos for p in g.particles], e["prev"])
            assert same_bits(g.center, e["center"])


@pytest.mark.parametrize("steps", [1, 10])
def test_config1_cloth(gpu, steps):
    from bendy2d_gb300 import scenes
    check(scenes.config1(seed=steps), steps, f"config1 x{steps}")


def test_config1_long_run_stays_exact(gpu):
    from bendy2d_gb300 import scenes
    check(scenes.config1(seed=7), 60, "config1 x60")


@pytest.mark.parametrize("steps", [1, 10])
def test_config2_small_with_collisions(gpu, steps):
    from bendy2d_gb300 import scenes
    sc = scenes.config2(seed=steps, n_bodies=6, box=120.0, n_circles=4, n_polys=3)
    check(sc, steps, f"config2-small x{steps}")


@pytest.mark.parametrize("steps", [1, 10])
def test_config2_full(gpu, steps):
    """Full configuration (65,536 particles, 249,984 links, collisions on)."""
    from bendy2d_gb300 import scenes
    check(scenes.config2(seed=0), steps, f"config2 x{steps}")


def test_config2_reference_semantics_no_collisions(gpu):
    from bendy2d_gb300 import scenes
    sc = scenes.config2(seed=4, n_bodies=8, box=300.0, collide=0)
    check(sc, 5, "config2 no-ext x5")


@pytest.mark.parametrize("collide", [1, 2, 4, 3, 5, 6, 7])
def test_collision_flag_combinations(gpu, collide):
    from bendy2d_gb300 import scenes
    sc = scenes.config2(seed=collide, n_bodies=4, box=90.0, n_circles=5, n_polys=3,
                        collide=collide)
    check(sc, 6, f"collide={collide}")


@pytest.mark.parametrize("collide", [1, 3, 7])
def test_per_particle_collide_matches_oracle(gpu, collide):
    """The collide pass with one thread per particle (taken by large
    launches; forced here with collide_thread_min = 0) against the oracle,
    with particle-particle contacts alone and with circles and polygons."""
    from bendy2d_gb300 import scenes
    sc = scenes.config2(seed=20 + collide, n_bodies=5, box=100.0, n_circles=5, n_polys=3,
                        collide=collide)
    s = sc.to_solver()
    s.set_tuning(collide_thread_min=0)
    from oracle import load_scene
    o = load_scene(sc)
    for _ in range(6):
        s.update(sc.dt)
        assert o.update(sc.dt) == 0
    assert_same_state(solver_state(s), oracle_state(o), f"per-particle collide, collide={collide}")


def test_fast_mode_matches_oracle_in_colour_order(gpu):
    from bendy2d_gb300 import MODE_FAST, scenes
    sc = scenes.config1(seed=3)
    sc.mode = MODE_FAST
    s = sc.to_solver()
    order = s.link_order()
    from oracle import load_scene
    o = load_scene(sc, link_order=order)
    for _ in range(10):
        s.update(sc.dt)
        assert o.update(sc.dt) == 0
    assert_same_state(solver_state(s), oracle_state(o), "fast mode")


def test_fast_mode_residual_close_to_reference(gpu):
    """Fast mode reorders Gauss-Seidel, so it is compared by residual."""
    from bendy2d_gb300 import MODE_FAST, scenes
    from oracle import load_scene
    sc = scenes.config1(seed=5)
    ref = load_scene(sc)
    sc.mode = MODE_FAST
    s = sc.to_solver()
    fast = load_scene(sc, link_order=s.link_order())
    for _ in range(30):
        ref.update(sc.dt)
        fast.update(sc.dt)
        s.update(sc.dt)
    r_ref, r_fast = ref.link_residual(), fast.link_residual()
    assert r_fast < max(5 * r_ref, 1e-2), (r_ref, r_fast)


@pytest.mark.parametrize("iters,sub", [(1, 1), (2, 3), (4, 8), (8, 20)])
def test_iterations_and_substeps(gpu, iters, sub):
    from bendy2d_gb300 import scenes
    sc = scenes.config1(seed=iters)
    sc.link_iters, sc.sub_steps = iters, sub
    check(sc, 3, f"I={iters} S={sub}")


def test_rings_serial_executor_with_stiffness(gpu):
    from bendy2d_gb300 import scenes
    rng = np.random.default_rng(11)
    sc = scenes.config3_world(rng, 1500, link_iters=2)
    assert sc.to_solver().plan_stats()["serial_bodies"] >= 1
    check(sc, 5, "rings")


def _big_cloth(side, collide, sub_steps, link_iters, seed=2, box=100.0):
    from bendy2d_gb300 import scenes
    rng = np.random.default_rng(seed)
    body = scenes.grid_body(side, side, (10.0, 20.0), 1.0, 0.01, rng)
    sc = scenes._assemble("big", [body], bounds=(0.0, 0.0, box, box), sub_steps=sub_steps,
                          link_iters=link_iters, collide=collide)
    sc.prev = scenes._velocity_prev(sc.pos, rng, 0.5, sc.dt / sub_steps)
    return sc


@pytest.mark.parametrize("side,collide,clusters", [(72, 0, 1), (100, 0, 2), (100, 1, 1)])
def test_large_body_executor_matches_oracle_and_global_executor(gpu, side, collide, clusters):
    """A body whose state, links and schedule do not fit one CTA's shared
    memory: the large-body executor (positions in the shared memory of a
    cluster of `clusters` CTAs) and, with large_max = 0, the global-memory
    group executor both match the oracle bit for bit."""
    from oracle import load_scene
    sc = _big_cloth(side, collide, 2, 2)
    s = sc.to_solver()
    st = s.plan_stats()
    assert st["large_bodies"] == 1 and st["global_bodies"] == 0
    g = sc.to_solver()
    g.set_tuning(large_max=0)
    assert g.plan_stats()["global_bodies"] == 1
    o = load_scene(sc)
    for _ in range(3):
        s.update(sc.dt)
        g.update(sc.dt)
        assert o.update(sc.dt) == 0
    assert_same_state(solver_state(s), oracle_state(o), f"large-body executor {side}x{side}")
    assert_same_state(solver_state(g), oracle_state(o), f"global executor {side}x{side}")


def test_large_body_cluster_with_wide_ops(gpu):
    """A 260x260 cloth (67,600 particles) with particle collisions: its link
    passes run on a cluster of five CTAs, with link endpoints read from the
    body-local link table (more than 65,535 particles)."""
    sc = _big_cloth(260, 1, 2, 1, seed=5, box=300.0)
    s = sc.to_solver()
    assert s.plan_stats()["large_bodies"] == 1
    check(sc, 2, "cluster of five CTAs")


def test_free_particles_and_mixed_components(gpu):
    """Link-free particles, tiny components packed into one body, a chain."""
    from bendy2d_gb300 import scenes
    rng = np.random.default_rng(5)
    bodies = [scenes.grid_body(3, 2, rng.uniform(10, 80, 2), 1.0, 0.01, rng) for _ in range(20)]
    free = (rng.uniform(5, 95, size=(37, 2)).astype(np.float32), np.zeros(0, np.uint64),
            np.zeros(0, np.uint64))
    chain_pos = np.stack([np.linspace(20, 60, 41), np.full(41, 70.0)], 1).astype(np.float32)
    chain = (chain_pos, np.arange(40, dtype=np.uint64), np.arange(1, 41, dtype=np.uint64))
    sc = scenes._assemble("mixed", bodies + [free, chain], bounds=(0.0, 0.0, 100.0, 100.0),
                          sub_steps=4, link_iters=3)
    sc.prev = (sc.pos + rng.normal(0, 0.05, sc.pos.shape)).astype(np.float32)
    check(sc, 8, "mixed")


def test_heavy_polygon_and_circle_contacts(gpu):
    """Overlapping dynamic polygons and piled circles: many speculative
    rounds in the pair loops."""
    from bendy2d_gb300 import scenes
    rng = np.random.default_rng(9)
    polys = [{"points": scenes.convex_polygon(rng, rng.uniform(40, 60, 2), rng.uniform(5, 15),
                                              int(rng.integers(3, 9))), "static": False}
             for _ in range(9)]
    circles = [scenes._circle(rng.uniform(30, 70, 2), rng.uniform(2, 8), False)
               for _ in range(24)]
    sc = scenes._assemble("pile", [], circles=circles, polygons=polys,
                          bounds=(0.0, 0.0, 100.0, 100.0), sub_steps=4, link_iters=2)
    check(sc, 12, "pile")


def test_contact_sums_past_2_pow_53(gpu):
    """Particles millions of units wide, all overlapping: a particle's
    fixed-point contact sum passes 2^53, where it converts back through the
    double path; smaller sums take the float path."""
    from bendy2d_gb300 import scenes
    from bendy2d_gb300.scenes import COLLIDE_PP
    rng = np.random.default_rng(13)
    pos = (rng.uniform(4.0e8, 4.02e8, size=(24, 2))).astype(np.float32)
    free = (pos, np.zeros(0, np.uint64), np.zeros(0, np.uint64))
    sc = scenes._assemble("wide", [free], bounds=(0.0, 0.0, 1.0e9, 1.0e9), sub_steps=2,
                          link_iters=1, collide=COLLIDE_PP, radius=3.0e6, cell=8388608.0)
    check(sc, 3, "wide contacts")


def test_circle_links_and_static_circles(gpu):
    from bendy2d_gb300 import scenes
    rng = np.random.default_rng(4)
    circles = [scenes._circle(rng.uniform(20, 80, 2), rng.uniform(1, 4), i % 3 == 0)
               for i in range(10)]
    sc = scenes._assemble("clinks", [], circles=circles, bounds=(0.0, 0.0, 100.0, 100.0),
                          sub_steps=3, link_iters=2)
    sc.circle_links = [(0, 1, 6.0), (1, 2, 5.0), (2, 5, 8.0), (3, 9, 4.0)]
    check(sc, 10, "circle links")


@pytest.mark.parametrize("collide", [2, 7])
def test_collision_flags_without_solver_particles(gpu, collide):
    """A world with collision flags but only circles and a polygon (no
    solver particles) runs the sub-step pipeline with no particle work:
    no particle kernel is launched, the circles and the polygon move as in
    the oracle."""
    from bendy2d_gb300 import scenes
    rng = np.random.default_rng(8)
    circles = [scenes._circle(rng.uniform(20, 80, 2), rng.uniform(1, 4), False) for _ in range(6)]
    polys = [{"points": scenes.convex_polygon(rng, (50.0, 50.0), 10.0, 5), "static": False}]
    sc = scenes._assemble("no_particles", [], circles=circles, polygons=polys,
                          bounds=(0.0, 0.0, 100.0, 100.0), sub_steps=3, link_iters=1,
                          collide=collide)
    check(sc, 5, f"collision flags {collide}, no solver particles")


def test_empty_and_degenerate_worlds(gpu):
    from bendy2d_gb300 import Solver
    s = Solver()
    s.update(0.016)            # empty world
    s.add_particle((5.0, 5.0))
    s.update(0.016)
    assert s.get_particle_len() == 1
    s.set_sub_steps(0)         # zero sub-steps: nothing moves
    before = s.read_state()
    s.update(0.016)
    after = s.read_state()
    assert same_bits(before[0], after[0])


def test_add_after_update_keeps_state(gpu):
    """Adding bodies between updates keeps the device state (host mirror sync)."""
    from bendy2d_gb300 import scenes
    from oracle import load_scene
    sc = scenes.config1(seed=8)
    s = sc.to_solver()
    o = load_scene(sc)
    for _ in range(3):
        s.update(sc.dt)
        o.update(sc.dt)
    s.add_particle((10.0, 90.0))
    o.add_particles(np.array([[10.0, 90.0]], np.float32))
    for _ in range(3):
        s.update(sc.dt)
        o.update(sc.dt)
    assert_same_state(solver_state(s), oracle_state(o), "add after update")


def test_batch_equals_alone(gpu):
    """Worlds stepped together in one batch give the same bits as alone."""
    from bendy2d_gb300 import Batch, scenes
    rng = np.random.default_rng(21)
    worlds = [scenes.config3_world(rng, int(n)) for n in rng.integers(64, 1500, size=12)]
    worlds.append(scenes.config1(seed=2))
    worlds.append(scenes.config2(seed=3, n_bodies=3, box=100.0, n_circles=3, n_polys=2))
    alone = [w.to_solver() for w in worlds]
    together = [w.to_solver() for w in worlds]
    b = Batch(together)
    for _ in range(4):
        for s, w in zip(alone, worlds):
            s.update(w.dt)
        b.update(worlds[0].dt)
    for a, t in zip(alone, together):
        assert_same_state(solver_state(a), solver_state(t), "batch")
    b.close()


def test_mixed_batch_matches_oracle(gpu):
    """A batch mixing one world of 160 cloth bodies (more than there are SMs:
    its launch class streams schedules) with serving-style worlds of mixed
    sizes (small classes hold schedules resident and run on branch streams),
    all with particle collisions: every world matches the oracle."""
    from bendy2d_gb300 import Batch, scenes
    from oracle import load_scene
    rng = np.random.default_rng(41)
    worlds = [scenes.config2(seed=9, n_bodies=160, collide=1)]
    worlds += [scenes.config4_request(rng, int(n))
               for n in np.exp(rng.uniform(np.log(64), np.log(6000), 20)).astype(int)]
    sols = [w.to_solver() for w in worlds]
    b = Batch(sols)
    for _ in range(2):
        b.update(worlds[0].dt)
    for w, s in zip(worlds, sols):
        o = load_scene(w)
        for _ in range(2):
            assert o.update(w.dt) == 0
        assert_same_state(solver_state(s), oracle_state(o), f"mixed batch {w.name}")
    b.close()


def test_plain_mode_equals_batched(gpu):
    """The one-world-per-launch baseline computes the same bits."""
    from bendy2d_gb300 import Batch, scenes
    rng = np.random.default_rng(31)
    worlds = [scenes.config3_world(rng, int(n)) for n in rng.integers(64, 900, size=8)]
    worlds.append(scenes.config1(seed=4))
    a = [w.to_solver() for w in worlds]
    b = [w.to_solver() for w in worlds]
    ba, bb = Batch(a), Batch(b)
    bb.set_plain(True)
    for _ in range(3):
        ba.update(worlds[0].dt)
        bb.update(worlds[0].dt)
    assert bb.launch_count() > ba.launch_count()
    for x, y in zip(a, b):
        assert_same_state(solver_state(x), solver_state(y), "plain vs batched")
    ba.close()
    bb.close()


def test_write_state_roundtrip_and_clone(gpu):
    from bendy2d_gb300 import scenes
    sc = scenes.config1(seed=1)
    s = sc.to_solver()
    s.update(sc.dt)
    pos, prev = s.read_state()
    c = s.clone()
    s.update(sc.dt)
    c.update(sc.dt)
    assert same_bits(s.read_state()[0], c.read_state()[0])
    s.write_state(pos, prev)
    s.update(sc.dt)
    assert same_bits(s.read_state()[0], c.read_state()[0])


def test_graph_and_eager_launches_agree(gpu):
    from bendy2d_gb300 import scenes
    sc = scenes.config2(seed=6, n_bodies=4, box=100.0, n_circles=3, n_polys=2)
    a, b = sc.to_solver(), sc.to_solver()
    b.set_graphs(False)
    for _ in range(3):
        a.update(sc.dt)
        b.update(sc.dt)
    assert_same_state(solver_state(a), solver_state(b), "graph vs eager")


@pytest.mark.parametrize("full", [False, True])
def test_resident_and_streamed_schedules_agree(gpu, full):
    """A body's schedule is either held whole in shared memory (one bulk
    copy) or streamed through two chunk buffers; both run the same ops."""
    from bendy2d_gb300 import scenes
    collide = 7 if not full else 0
    sc = scenes.config2(seed=8, n_bodies=3, box=120.0, n_circles=2, n_polys=1, collide=collide)
    b = sc.to_solver()
    b.set_tuning(resident=0)
    a, o = run_both(sc, 3)
    for _ in range(3):
        b.update(sc.dt)
    assert_same_state(solver_state(a), solver_state(b), "resident vs streamed")
    assert_same_state(solver_state(a), oracle_state(o), "resident vs oracle")


def test_config5_full_size_isolated_bodies_match_oracle(gpu):
    """Full configuration 5 (1,048,576 particles, fast mode, collisions) for
    one step on the GPU.  Size-independent check: bodies are 90 units apart,
    so in one step each body interacts only with itself and with the circles
    and polygons (which particles never push back); a sub-world holding a
    few of the bodies plus every circle and polygon must therefore give the
    same bits on the oracle."""
    from bendy2d_gb300 import MODE_FAST, scenes
    from oracle import load_scene
    full = scenes.config5(seed=0, mode=MODE_FAST)
    s = full.to_solver()
    s.update(full.dt)
    pos, prev = s.read_state()
    pick = [0, 517, 1023]
    sub = scenes.config5(seed=0, mode=MODE_FAST)
    keep = np.concatenate([np.arange(k * 1024, (k + 1) * 1024) for k in pick])
    remap = -np.ones(len(full.pos), np.int64)
    remap[keep] = np.arange(len(keep))
    lk = np.isin(full.la.astype(np.int64), keep) & np.isin(full.lb.astype(np.int64), keep)
    sub.pos, sub.prev = full.pos[keep], full.prev[keep]
    sub.la = remap[full.la[lk].astype(np.int64)].astype(np.uint64)
    sub.lb = remap[full.lb[lk].astype(np.int64)].astype(np.uint64)
    sub.rest, sub.stiff = full.rest[lk], full.stiff[lk]
    probe = sub.to_solver()
    o = load_scene(sub, link_order=probe.link_order())
    assert o.update(sub.dt) == 0
    opos, oprev = o.particles()
    assert same_bits(pos[keep], opos)
    assert same_bits(prev[keep], oprev)
    gc = s.get_circles()
    oc, _ = o.circles()
    assert same_bits([c.point.pos for c in gc], oc)


@pytest.mark.parametrize("tuning", [
    {"t_max": 64}, {"t_min": 256, "t_max": 256}, {"width_per_thread": 2.0},
    {"resident": 0}, {"serial_width": 1000.0}, {"serial_width": 0.0},
    {"max_groups": 1, "warp_groups": 1}, {"stage_frac": 0.0}, {"stage_frac": 2.0},
    {"smem_max": 16384}, {"collide_thread_min": 0}, {"grid_slot_max": 0},
    {"grid_slot_max": 0, "collide_thread_min": 0},
])
def test_tunables_never_change_results(gpu, tuning):
    """Executor tunables move work between executors, group sizes, launch
    classes and pack kinds; the bits must stay those of the defaults."""
    from bendy2d_gb300 import Batch, scenes
    rng = np.random.default_rng(51)
    worlds = [scenes.config2(seed=11, n_bodies=4, box=110.0, n_circles=3, n_polys=2),
              scenes.config3_world(rng, 900, link_iters=2), scenes.config1(seed=6)]
    ref = [w.to_solver() for w in worlds]
    tuned = [w.to_solver() for w in worlds]
    bref, btun = Batch(ref), Batch(tuned)
    btun.set_tuning(**tuning)
    for _ in range(3):
        bref.update(worlds[0].dt)
        btun.update(worlds[0].dt)
    for a, b in zip(ref, tuned):
        assert_same_state(solver_state(a), solver_state(b), f"tuning {tuning}")
    bref.close()
    btun.close()


def test_autotune_returns_a_valid_tuning(gpu):
    from bendy2d_gb300 import autotune, scenes
    sc = scenes.config2(seed=12, n_bodies=2, box=80.0, n_circles=2, n_polys=1)
    best = autotune.autotune(sc, steps=1, warmup=1, space={"t_max": [128, 256], "resident": [0, 1]})
    knobs = {k: v for k, v in best.items() if not k.startswith("_")}
    assert set(knobs) <= {"t_max", "resident"}
    assert best.get("_ms_per_step", 1.0) > 0.0
    s = sc.to_solver()
    if knobs:
        s.set_tuning(**knobs)
    s.update(sc.dt)


def test_batch_updates_from_two_threads(gpu):
    """Batch calls hold the batch's lock: two threads updating one batch
    concurrently give exactly two steps."""
    import threading
    from bendy2d_gb300 import Batch, scenes
    rng = np.random.default_rng(61)
    worlds = [scenes.config3_world(rng, int(n)) for n in (200, 700, 1300)]
    worlds.append(scenes.config2(seed=13, n_bodies=2, box=90.0, n_circles=2, n_polys=1))
    alone = [w.to_solver() for w in worlds]
    shared = [w.to_solver() for w in worlds]
    b = Batch(shared)
    errs = []

    def one():
        try:
            b.update(worlds[0].dt)
        except Exception as e:  # surfaced below
            errs.append(e)

    th = [threading.Thread(target=one) for _ in range(2)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert not errs, errs
    for s, w in zip(alone, worlds):
        s.update(w.dt)
        s.update(w.dt)
    for a, t in zip(alone, shared):
        assert_same_state(solver_state(a), solver_state(t), "two threads")
    b.close()


def test_body_over_65535_particles_uses_wide_ops(gpu):
    """A 260x260 cloth (67,600 particles) is one body too large for 16-bit
    local endpoints: the global executor runs wide ops (link ids resolved
    through the link table)."""
    from bendy2d_gb300 import scenes
    rng = np.random.default_rng(71)
    body = scenes.grid_body(260, 260, (10.0, 10.0), 1.0, 0.01, rng)
    sc = scenes._assemble("huge", [body], bounds=(0.0, 0.0, 300.0, 300.0), sub_steps=2,
                          link_iters=1)
    st = sc.to_solver().plan_stats()
    assert st["global_bodies"] == 1 and st["group_bodies"] == 1
    check(sc, 2, "wide ops")


def test_ring_too_large_for_shared_memory_runs_serially_from_global(gpu):
    """A hub-and-spoke ring of 9,000 rim particles: its positions alone
    exceed a serial pack and with its links it exceeds a CTA's shared
    memory, so the global-memory serial executor replays it."""
    from bendy2d_gb300 import scenes
    p, a, b = scenes.ring_body(9000, (500.0, 500.0), 300.0)
    sc = scenes._assemble("ring", [(p, a, b)], bounds=(0.0, 0.0, 1000.0, 1000.0), sub_steps=4,
                          link_iters=1)
    st = sc.to_solver().plan_stats()
    assert st["serial_bodies"] == 1
    check(sc, 2, "large ring")


def test_programmatic_launches_do_not_change_results(gpu):
    """The sub-step pipeline's kernels start early under programmatic
    dependent launch; profiling mode launches them one after another
    without it.  Both give the same bits."""
    from bendy2d_gb300 import scenes
    sc = scenes.config2(seed=14, n_bodies=5, box=120.0, n_circles=3, n_polys=2)
    a, b = sc.to_solver(), sc.to_solver()
    b.set_profiling(True)
    for _ in range(4):
        a.update(sc.dt)
        b.update(sc.dt)
    assert_same_state(solver_state(a), solver_state(b), "programmatic vs serial launches")


def _clumped_cloths(seed, sub_steps, n_bodies=4):
    """Cloth grids plus a 3 x 3 grid packed into one collision cell (nine
    entries in one bucket: five in its overflow chain), particle collisions."""
    from bendy2d_gb300 import scenes
    rng = np.random.default_rng(seed)
    bodies = [scenes.grid_body(16, 16, rng.uniform(0.0, 80.0, 2), 1.0, 0.01, rng)
              for _ in range(n_bodies)]
    bodies.append(scenes.grid_body(3, 3, (95.3, 95.3), 0.05, 0.0, rng))
    sc = scenes._assemble(f"clumped_s{sub_steps}", bodies, bounds=(0.0, 0.0, 100.0, 100.0),
                          sub_steps=sub_steps, link_iters=2, collide=1)
    sc.prev = scenes._velocity_prev(sc.pos, rng, 0.5, sc.dt / sc.sub_steps)
    return sc


@pytest.mark.parametrize("slot_max", [1 << 30, 0])
def test_collision_grid_odd_and_mixed_sub_steps(gpu, slot_max):
    """The slotted grid double-buffers its cell words by sub-step parity and
    clears parity 0 in the copy-back when an update has an odd number of
    sub-steps; overflow chains hold a bucket's entries past its slots.
    Several updates of worlds with 1, 3 and 4 sub-steps, alone and in one
    batch (odd and even sub-step counts together), with a dense clump, in
    both grid forms (slot_max 0: the sorted grid): every world matches the
    oracle."""
    from bendy2d_gb300 import Batch
    from oracle import load_scene
    worlds = [_clumped_cloths(61, 3), _clumped_cloths(62, 4), _clumped_cloths(63, 1)]
    alone = [w.to_solver() for w in worlds]
    for s in alone:
        s.set_tuning(grid_slot_max=slot_max)
    together = [w.to_solver() for w in worlds]
    b = Batch(together)
    b.set_tuning(grid_slot_max=slot_max)
    oracles = [load_scene(w) for w in worlds]
    for step in range(4):
        for s, w, o in zip(alone, worlds, oracles):
            s.update(w.dt)
            assert o.update(w.dt) == 0
        b.update(worlds[0].dt)
        for s, t, o, w in zip(alone, together, oracles, worlds):
            assert_same_state(solver_state(s), oracle_state(o), f"{w.name} alone, update {step}")
            assert_same_state(solver_state(t), oracle_state(o), f"{w.name} batched, update {step}")
    b.close()
    for s in alone:
        s.close()
