"""The per-object methods of the Python mirror (Particle, Link, Circle,
Polygon, line_intersection) on the CPU.

Solver::update (src/solver.rs:106-188) is nothing but these methods in a
fixed order, so composing them in that order on host objects must give the
oracle's update bit for bit; every method is exercised on a world with
particles, links, circles, circle links and overlapping polygons."""
import numpy as np
import pytest

from helpers import same_bits


def _world(seed):
    from bendy2d_gb300 import scenes
    from bendy2d_gb300.api import Bounds, Circle, CircleLink, Link, Particle, ParticleLink, Polygon
    rng = np.random.default_rng(seed)
    pos, a, b = scenes.grid_body(5, 4, (10.0, 30.0), 1.5, 0.05, rng)
    free = rng.uniform(5.0, 55.0, size=(6, 2)).astype(np.float32)
    pos = np.vstack([pos, free]).astype(np.float32)
    prev = (pos + rng.normal(0.0, 0.05, pos.shape)).astype(np.float32)
    rest = scenes.f32_dist(pos[a.astype(np.int64)], pos[b.astype(np.int64)])
    parts = [Particle(tuple(map(float, p)), tuple(map(float, q))) for p, q in zip(pos, prev)]
    links = [ParticleLink(Link(int(x), int(y), float(t))) for x, y, t in zip(a, b, rest)]
    circles = []
    for k in range(5):
        c = rng.uniform(15.0, 45.0, 2).astype(np.float32)
        circles.append(Circle(Particle(tuple(map(float, c)), tuple(map(float, c))),
                              float(np.float32(rng.uniform(2.0, 5.0)))))
    clinks = [CircleLink(Link(0, 1, 6.0)), CircleLink(Link(2, 4, 5.0))]
    polys = [Polygon.new([tuple(p) for p in scenes.convex_polygon(rng, rng.uniform(25, 35, 2),
                                                                  rng.uniform(4, 8), k)], False)
             for k in (3, 5, 6)]
    polys.append(Polygon.circle(6.0, (30.0, 8.0), 7, True))
    return parts, links, circles, clinks, polys, Bounds((0.0, 0.0), (60.0, 60.0))


def _oracle(parts, links, circles, clinks, polys, bounds, g, sub):
    from oracle import Oracle
    o = Oracle()
    o.set_gravity(*g)
    o.set_bounds(*bounds.pos, *bounds.size)
    o.set_sub_steps(sub)
    o.add_particles(np.asarray([p.pos for p in parts], np.float32),
                    np.asarray([p.prev_pos for p in parts], np.float32))
    o.add_particle_links([l.link.particle_a for l in links], [l.link.particle_b for l in links],
                         [l.link.target_distance for l in links])
    for c in circles:
        o.add_circle(c.point.pos, c.point.prev_pos, c.point.acc, c.radius)
    for l in clinks:
        o.add_circle_link(l.link.particle_a, l.link.particle_b, l.link.target_distance)
    for q in polys:
        o.add_polygon(np.asarray([p.pos for p in q.particles], np.float32),
                      np.asarray([p.prev_pos for p in q.particles], np.float32),
                      np.asarray([p.acc for p in q.particles], np.float32),
                      [(l.link.particle_a, l.link.particle_b, l.link.target_distance)
                       for l in q.particle_links], q.is_static, q.center, q.scale)
    return o


def _host_update(parts, links, circles, clinks, polys, bounds, g, sub, dt):
    """Solver::update from the per-object methods, in the reference's order."""
    delta = np.float32(dt) * (np.float32(1.0) / np.float32(sub))
    for _ in range(sub):
        for p in parts:
            p.add_force_v2(g)
        for c in circles:
            c.point.add_force_v2(g)
        for q in polys:
            q.add_force_v2(g)
        for l in links:
            l.solve(parts)
        for l in clinks:
            l.solve(circles)
        for q in polys:
            q.solve_links()
        for i in range(len(circles)):
            for j in range(i + 1, len(circles)):
                circles[i].solve_circle(circles[j])
        for i in range(len(polys)):
            for j in range(i + 1, len(polys)):
                polys[i].solve_polygon(polys[j])
        for p in parts:
            p.solve_bounds(bounds)
        for c in circles:
            c.solve_bounds(bounds)
        for q in polys:
            q.solve_bounds(bounds)
        for p in parts:
            p.update(float(delta))
        for c in circles:
            c.point.update(float(delta))
        for q in polys:
            q.update(float(delta))


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_per_object_methods_compose_to_the_oracle_update(native_lib, seed):
    world = _world(seed)
    g, sub, dt = (0.0, -9.81), 2, 1.0 / 60.0
    o = _oracle(*world, g, sub)
    parts, links, circles, clinks, polys, bounds = world
    hits = 0
    for step in range(12):
        before = [tuple(p.pos) for q in polys for p in q.particles]
        _host_update(parts, links, circles, clinks, polys, bounds, g, sub, dt)
        assert o.update(dt) == 0
        hits += sum(a != tuple(p.pos) for a, p in zip(before, (p for q in polys for p in q.particles)))
        pos, prev = o.particles()
        assert same_bits(np.asarray([p.pos for p in parts], np.float32), pos), step
        assert same_bits(np.asarray([p.prev_pos for p in parts], np.float32), prev), step
        cp, cq = o.circles()
        assert same_bits(np.asarray([c.point.pos for c in circles], np.float32), cp), step
        assert same_bits(np.asarray([c.point.prev_pos for c in circles], np.float32), cq), step
        for q, (qp, qq, qc) in zip(polys, o.polygons()):
            assert same_bits(np.asarray([p.pos for p in q.particles], np.float32), qp), step
            assert same_bits(np.asarray([p.prev_pos for p in q.particles], np.float32), qq), step
            assert same_bits(np.asarray(q.center, np.float32), qc), step
    assert hits > 0


def test_link_with_bad_indices_raises(native_lib):
    """The reference panics in split_at_mut (src/link.rs:19-21)."""
    from bendy2d_gb300.api import Link, Particle, ParticleLink
    ps = [Particle.new((0.0, 0.0)), Particle.new((1.0, 0.0))]
    for a, b in ((1, 0), (0, 2), (1, 1)):
        with pytest.raises(IndexError):
            ParticleLink(Link(a, b, 1.0)).solve(ps)


def test_line_intersection():
    from bendy2d_gb300.api import line_intersection
    assert line_intersection(((0.0, 0.0), (2.0, 2.0)), ((0.0, 2.0), (2.0, 0.0))) == (1.0, 1.0)
    assert line_intersection(((0.0, 0.0), (1.0, 0.0)), ((0.0, 1.0), (1.0, 1.0))) is None  # parallel
    assert line_intersection(((0.0, 0.0), (1.0, 0.0)), ((2.0, -1.0), (2.0, 1.0))) is None


def test_particle_forces():
    """add_force / add_force_v2 / add_force_towards (src/particle.rs:48-59)
    feed update's acceleration term, which update then clears."""
    from bendy2d_gb300.api import Particle
    p = Particle.new((1.0, 1.0))
    p.add_force(2.0, 0.0)
    p.add_force_v2((0.0, -1.0))
    p.add_force_towards((1.0, 5.0), 4.0)  # unit vector (0, 1) * 4
    assert p.acc == (2.0, 3.0)
    p.update(0.5)
    f = np.float32
    assert p.pos == (float(f(1.0) + f(2.0) * f(0.5) * f(0.5)), float(f(1.0) + f(3.0) * f(0.5) * f(0.5)))
    assert p.prev_pos == (1.0, 1.0) and p.acc == (0.0, 0.0)
