"""The oracle against the hand-derived known answers (CPU only).

The reference has no tests or golden vectors, so these first-principles
cases (tests/golden/make_kats.py) are the only pin on the oracle."""
import numpy as np
import pytest

from helpers import kat_cases, kat_to_oracle, same_bits

CASES = kat_cases()


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_matches_kat(name):
    case = CASES[name]
    o = kat_to_oracle(case["scene"])
    st = 0
    for _ in range(case["steps"]):
        st = o.update(case["scene"]["dt"])
        if st:
            break
    if "expect_status" in case:
        assert st == case["expect_status"]
        return
    assert st == 0
    if "expect_pos" in case:
        pos, prev = o.particles()
        assert same_bits(pos, case["expect_pos"]), (pos, case["expect_pos"])
        assert same_bits(prev, case["expect_prev"])
    if "expect_circles_pos" in case:
        cp, cq = o.circles()
        assert same_bits(cp, case["expect_circles_pos"]), (cp, case["expect_circles_pos"])
        assert same_bits(cq, case["expect_circles_prev"])
    if "expect_polygons" in case:
        got = o.polygons()
        for g, e in zip(got, case["expect_polygons"]):
            assert same_bits(g[0], e["pos"]), (g[0], e["pos"])
            assert same_bits(g[1], e["prev"])
            assert same_bits(g[2], e["center"]), (g[2], e["center"])


def test_substeps_equal_repeated_updates():
    """G3: update(dt) with 8 sub-steps == 8 x update(dt/8) with 1 (1/8 exact)."""
    from bendy2d_gb300 import scenes
    from oracle import load_scene
    sc = scenes.config1(steps=1)
    a = load_scene(sc)
    sc1 = scenes.config1(steps=1)
    sc1.sub_steps = 1
    b = load_scene(sc1)
    for _ in range(3):
        assert a.update(sc.dt) == 0
        for _ in range(8):
            assert b.update(sc.dt / 8) == 0
    assert same_bits(a.particles()[0], b.particles()[0])
    assert same_bits(a.polygons()[0][0], b.polygons()[0][0])


def test_polygon_circle_builder_rejects_small_n():
    """Polygon::circle with n < 3 makes a == b links, which panic at update."""
    from oracle import Oracle
    for n in (1, 2):
        o = Oracle()
        o.add_polygon_circle(5.0, 50.0, 50.0, n, False)
        assert o.update(0.01) == 4
    o = Oracle()
    o.add_polygon_circle(5.0, 50.0, 50.0, 3, False)
    assert o.update(0.01) == 0


def test_polygon_circle_builder_topology():
    """Polygon::circle chords i -> i+2n/3 and i -> i+n/3 (src/polygon.rs:32-73)."""
    from oracle import Oracle
    o = Oracle()
    o.add_polygon_circle(10.0, 50.0, 50.0, 7, False)
    a, b, t = o.polygon_links(0)
    assert len(a) == 14 and np.all(a < b)
    exp = []
    for i in range(7):
        for off in (14 // 3, 7 // 3):
            x, y = i, (i + off) % 7
            exp.append((min(x, y), max(x, y)))
    assert list(zip(a.tolist(), b.tolist())) == exp
