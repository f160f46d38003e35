"""C ABI and host logic on the CPU: the library loads, exports every entry
point include/bendy2d.h declares, plans worlds on the host, reports the
reference's panic conditions as status codes, and refuses to run without a
GPU (there is no CPU fallback)."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    text = (ROOT / "include" / "bendy2d.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(b2d_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(native_lib):
    syms = declared_symbols()
    assert len(syms) > 60
    missing = [s for s in syms if not hasattr(native_lib, s)]
    assert not missing, missing


def test_python_binding_covers_header(native_lib):
    from bendy2d_gb300 import _native
    bound = set(_native.SIGNATURES) | {"b2d_last_error", "b2d_version"}
    assert set(declared_symbols()) <= bound


def test_version(native_lib):
    assert b"bendy2d" in native_lib.b2d_version()


def test_solver_defaults_match_reference(native_lib):
    """Solver::new, src/solver.rs:34-50."""
    from bendy2d_gb300 import Solver
    s = Solver()
    assert s.gravity == pytest.approx((0.0, 98.2))
    b = s.bounds
    assert b.pos == (0.0, 0.0) and b.size == (100.0, 100.0)
    assert s.bounds_active is True
    assert s.sub_steps == 1
    assert s.get_particle_len() == 0 and s.get_circles_len() == 0 and s.get_polygons_len() == 0


def test_getters_return_none_out_of_range(native_lib):
    """get_particle / get_circle / get_polygon return None (src/solver.rs:96-104)."""
    from bendy2d_gb300 import Solver
    s = Solver()
    s.add_particle((1.0, 2.0))
    assert s.get_particle(0).pos == (1.0, 2.0)
    assert s.get_particle(1) is None
    assert s.get_circle(0) is None
    assert s.get_polygon(0) is None


def test_polygon_builders_match_oracle(native_lib):
    """Polygon::circle / Polygon::new built by the product's host code equal
    the oracle's restatement bit for bit."""
    from oracle import Oracle
    from bendy2d_gb300 import Polygon
    from helpers import same_bits
    for n in (3, 5, 8, 13):
        g = Polygon.circle(7.5, (40.0, 60.0), n, False)
        o = Oracle()
        o.add_polygon_circle(7.5, 40.0, 60.0, n, False)
        pos, _, ctr = o.polygons()[0]
        assert same_bits(np.asarray([p.pos for p in g.particles]), pos)
        assert same_bits(np.asarray(g.center), ctr)
        a, b, t = o.polygon_links(0)
        assert [l.link.particle_a for l in g.particle_links] == a.tolist()
        assert [l.link.particle_b for l in g.particle_links] == b.tolist()
        assert same_bits([l.link.target_distance for l in g.particle_links], t)
    pts = [(1.0, 1.0), (5.0, 1.5), (6.0, 7.0), (0.5, 4.0)]
    g = Polygon.new(pts, True)
    o = Oracle()
    o.add_polygon_points(np.asarray(pts, np.float32), True)
    pos, _, ctr = o.polygons()[0]
    assert same_bits(np.asarray([p.pos for p in g.particles]), pos)
    assert same_bits(np.asarray(g.center), ctr)
    assert g.is_static


@pytest.mark.parametrize("bad,code", [((1, 0), 2), ((0, 0), 2), ((0, 2), 2)])
def test_bad_particle_links_are_status_codes(native_lib, bad, code):
    """The reference panics in ParticleLink::solve (src/link.rs:19-21)."""
    from bendy2d_gb300 import B2DError, Link, Solver
    s = Solver()
    s.add_particle((1.0, 1.0))
    s.add_particle((2.0, 2.0))
    s.add_particle_link(Link(bad[0], bad[1], 1.0))
    with pytest.raises(B2DError) as e:
        s.plan_stats()
    assert e.value.code == code


def test_bad_polygon_circle_is_status_code(native_lib):
    from bendy2d_gb300 import B2DError, Solver
    s = Solver()
    s.add_polygon_circle(5.0, (50.0, 50.0), 2, False)
    with pytest.raises(B2DError) as e:
        s.plan_stats()
    assert e.value.code == 4


def test_update_without_gpu_fails_loudly(native_lib):
    from conftest import HAS_GPU
    if HAS_GPU:
        pytest.skip("a GPU is present")
    from bendy2d_gb300 import B2DError, Solver
    s = Solver()
    s.add_particle((1.0, 1.0))
    with pytest.raises(B2DError) as e:
        s.update(0.016)
    assert e.value.code == 7 and "no CPU path" in str(e.value)


def test_plan_cloth_grid(native_lib):
    """One 32x32 cloth: one group body whose full-step schedule merges all
    8 sub-steps x 4 link passes (+ integrate) into 413 levels."""
    from bendy2d_gb300 import scenes
    s = scenes.config1(steps=1).to_solver()
    st = s.plan_stats()
    assert st["bodies"] == 1 and st["group_bodies"] == 1 and st["serial_bodies"] == 0
    assert st["ops"] == 8 * (4 * 3906 + 1024)
    assert st["levels"] == 413


def test_plan_rings_run_serially(native_lib):
    """Rings with a hub are chains in the reference's order (every spoke shares
    the centre), so they go to the serial executor."""
    from bendy2d_gb300 import scenes
    rng = np.random.default_rng(3)
    sc = scenes.config3_world(rng, 900)
    st = sc.to_solver().plan_stats()
    assert st["serial_bodies"] >= 1 and st["group_bodies"] == 0


def test_fast_mode_colouring_is_proper(native_lib):
    """Fast mode: no two links of one colour class share a particle, and the
    order is a permutation of the links."""
    from bendy2d_gb300 import MODE_FAST, scenes
    sc = scenes.config1(steps=1)
    sc.mode = MODE_FAST
    s = sc.to_solver()
    order = s.link_order()
    assert sorted(order.tolist()) == list(range(len(sc.la)))
    st = s.plan_stats()
    assert 4 <= st["colours"] <= 16
    # replay the greedy colouring: consecutive runs with disjoint particles
    la, lb = sc.la[order.astype(np.int64)], sc.lb[order.astype(np.int64)]
    seen, classes = set(), 0
    for a, b in zip(la.tolist(), lb.tolist()):
        if a in seen or b in seen:
            seen = set()
            classes += 1
        seen.update((a, b))
    assert classes + 1 <= st["colours"]
    # fast mode needs far fewer levels than reference order
    ref = scenes.config1(steps=1).to_solver().plan_stats()
    assert st["levels"] < ref["levels"]


def test_plan_config2_links_only_levels(native_lib):
    """With particle collisions on, each sub-step's 4 link passes form their
    own schedule: 153 levels for every 32x32 cloth (64 bodies)."""
    from bendy2d_gb300 import scenes
    st = scenes.config2(seed=0).to_solver().plan_stats()
    assert st["group_bodies"] == 64 and st["serial_bodies"] == 0
    assert st["levels"] == 64 * 153
    assert st["ops"] == 64 * 4 * 3906


def test_tunables_move_bodies_between_executors(native_lib):
    """serial_width decides group vs serial execution; smem_max pushes bodies
    out of one CTA's shared memory, to the large-body (cluster) executor, or
    with large_max = 0 to the global-memory executor; the plan still covers
    every link."""
    from bendy2d_gb300 import scenes
    sc = scenes.config2(seed=1, n_bodies=3, box=100.0, n_circles=1, n_polys=1)
    s = sc.to_solver()
    base = s.plan_stats()
    s.set_tuning(serial_width=1e9)
    ser = s.plan_stats()
    assert ser["serial_bodies"] == base["group_bodies"] + base["serial_bodies"]
    assert ser["group_bodies"] == 0
    s2 = sc.to_solver()
    s2.set_tuning(smem_max=1024)
    large = s2.plan_stats()
    assert large["large_bodies"] == large["group_bodies"] == base["group_bodies"]
    assert large["global_bodies"] == 0 and large["ops"] == base["ops"]
    s3 = sc.to_solver()
    s3.set_tuning(smem_max=1024, large_max=0)
    glob = s3.plan_stats()
    assert glob["global_bodies"] == glob["group_bodies"] == base["group_bodies"]
    assert glob["large_bodies"] == 0 and glob["ops"] == base["ops"]


def test_unknown_tunable_is_rejected(native_lib):
    from bendy2d_gb300 import B2DError, Solver
    s = Solver()
    with pytest.raises(B2DError) as e:
        s.set_tuning(no_such_knob=1.0)
    assert "unknown tunable" in str(e.value)



TUNABLES = ["serial_width", "t_min", "t_max", "pack_np", "pack_nl", "free_chunk", "smem_max",
            "warp_groups", "max_groups", "width_per_thread", "resident", "res_max",
            "stage_frac", "bucket_factor", "collide_thread_min", "large_max", "grid_slot_max"]


def test_every_documented_tunable_is_accepted(native_lib):
    """Each tunable is listed in the header's b2d_set_tuning comment and
    accepted by the library; the autotuner searches only known ones."""
    from pathlib import Path
    from bendy2d_gb300 import Solver
    from bendy2d_gb300.autotune import DEFAULTS
    hdr = (Path(__file__).resolve().parents[1] / "include" / "bendy2d.h").read_text()
    block = hdr[hdr.index("/* executor tunables"):hdr.index("int b2d_set_tuning")]
    s = Solver()
    for k in TUNABLES:
        assert k in block, k
        s.set_tuning(**{k: DEFAULTS.get(k, 1.0)})
    assert set(DEFAULTS) <= set(TUNABLES)
