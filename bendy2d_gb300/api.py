"""Python mirror of the reference's public API (src/lib.rs:1-6).

Names, fields and meanings follow bendy2d 0.0.1: ``Solver`` (src/solver.rs),
``Particle`` (src/particle.rs), ``Link`` / ``ParticleLink`` / ``CircleLink``
(src/link.rs), ``Circle`` (src/circle.rs), ``Polygon`` (src/polygon.rs) and
``Bounds`` (src/solver.rs:13-17).  Every call goes through the C ABI of
include/bendy2d.h; ``Solver.update`` runs on the GPU.  Where the reference
panics, the C ABI returns a status and this module raises ``B2DError``;
where it returns ``None`` (``get_particle`` & co.), so does this module.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Iterable, Optional, Sequence

import numpy as np

from . import _native as N
from ._native import B2DError

MODE_REFERENCE = 0
MODE_FAST = 1
COLLIDE_PP = 1
COLLIDE_PC = 2
COLLIDE_PPOLY = 4


def _v(p) -> tuple:
    return (float(p[0]), float(p[1]))


# Host arithmetic of the per-object methods: float32, one rounding per
# operation, in the reference's order (nalgebra: norm = sqrt(x*x + y*y),
# normalize = componentwise division by the norm).
_F = np.float32


def _f2(p) -> tuple:
    return (_F(p[0]), _F(p[1]))


def _py(p) -> tuple:
    return (float(p[0]), float(p[1]))


def _norm(x, y):
    return np.sqrt(x * x + y * y)


def _reflect(pos, prev, lo, hi):
    """One axis of solve_bounds: below lo, else above hi, the coordinate is
    put on the bound and the Verlet velocity reflected."""
    if pos < lo:
        v = prev - pos
        return lo, lo - v
    if pos > hi:
        v = prev - pos
        return hi, hi - v
    return pos, prev


@dataclass
class Particle:
    """src/particle.rs:4-9 (``acc`` is private there; exposed read-only here)."""
    pos: tuple
    prev_pos: tuple
    acc: tuple = (0.0, 0.0)

    @staticmethod
    def new(pos) -> "Particle":  # src/particle.rs:12-18
        p = _v(pos)
        return Particle(p, p, (0.0, 0.0))

    def update(self, dt: float) -> None:
        """src/particle.rs:20-25: pos + velocity + (acc * dt) * dt."""
        (x, y), (qx, qy), (ax, ay), d = _f2(self.pos), _f2(self.prev_pos), _f2(self.acc), _F(dt)
        vx, vy = x - qx, y - qy
        self.prev_pos = _py((x, y))
        self.pos = _py(((x + vx) + (ax * d) * d, (y + vy) + (ay * d) * d))
        self.acc = (0.0, 0.0)

    def solve_bounds(self, bounds: "Bounds") -> None:
        """src/particle.rs:27-46."""
        (x, y), (qx, qy) = _f2(self.pos), _f2(self.prev_pos)
        (bx, by), (bw, bh) = _f2(bounds.pos), _f2(bounds.size)
        x, qx = _reflect(x, qx, bx, bx + bw)
        y, qy = _reflect(y, qy, by, by + bh)
        self.pos, self.prev_pos = _py((x, y)), _py((qx, qy))

    def add_force(self, force_x: float, force_y: float) -> None:  # src/particle.rs:48-50
        self.add_force_v2((force_x, force_y))

    def add_force_v2(self, force) -> None:  # src/particle.rs:52-54
        (ax, ay), (fx, fy) = _f2(self.acc), _f2(force)
        self.acc = _py((ax + fx, ay + fy))

    def add_force_towards(self, point, force: float) -> None:
        """src/particle.rs:56-59: along the unit vector towards point."""
        (px, py), (x, y), f = _f2(point), _f2(self.pos), _F(force)
        dx, dy = px - x, py - y
        n = _norm(dx, dy)
        self.add_force_v2((dx / n * f, dy / n * f))


@dataclass
class Link:
    """src/link.rs:4-10; particle_a must be lower than particle_b."""
    particle_a: int
    particle_b: int
    target_distance: float
    stiffness: float = 1.0  # extension; 1.0 reproduces the reference


def _link_ends(seq, link: Link):
    """The two elements of a link; the reference indexes them through
    split_at_mut and panics unless particle_a < particle_b < len
    (src/link.rs:19-21)."""
    a, b = link.particle_a, link.particle_b
    if not (0 <= a < b < len(seq)):
        raise IndexError(f"link ({a}, {b}) needs a < b < {len(seq)}")
    return seq[a], seq[b]


@dataclass
class ParticleLink:  # src/link.rs:12-15
    link: Link

    def solve(self, particles: list) -> None:
        """src/link.rs:18-27 (the stiffness extension multiplies last; 1.0 is
        exact)."""
        pa, pb = _link_ends(particles, self.link)
        (ax, ay), (bx, by) = _f2(pa.pos), _f2(pb.pos)
        t, k = _F(self.link.target_distance), _F(self.link.stiffness)
        dx, dy = ax - bx, ay - by
        dist = _norm(dx, dy)
        nx, ny = dx / dist, dy / dist
        m = dist - t
        cx, cy = nx * m * _F(0.5) * k, ny * m * _F(0.5) * k
        pa.pos = _py((ax - cx, ay - cy))
        pb.pos = _py((bx + cx, by + cy))


@dataclass
class CircleLink:  # src/link.rs:30-33
    link: Link

    def solve(self, circles: list) -> None:
        """src/link.rs:36-48: the correction split by the squared radii."""
        ca, cb = _link_ends(circles, self.link)
        (ax, ay), (bx, by) = _f2(ca.point.pos), _f2(cb.point.pos)
        t = _F(self.link.target_distance)
        dx, dy = ax - bx, ay - by
        dist = _norm(dx, dy)
        nx, ny = dx / dist, dy / dist
        ra, rb = _F(ca.radius), _F(cb.radius)
        ra2, rb2 = ra * ra, rb * rb
        scale = _F(1.0) / (ra2 + rb2)
        m = dist - t
        ca.point.pos = _py((ax - nx * m * scale * rb2, ay - ny * m * scale * rb2))
        cb.point.pos = _py((bx + nx * m * scale * ra2, by + ny * m * scale * ra2))


@dataclass
class Circle:  # src/circle.rs:4-8
    point: Particle
    radius: float
    is_static: bool = False  # extension

    def solve_bounds(self, bounds: "Bounds") -> None:
        """src/circle.rs:11-30: the particle rule with the bounds shrunk by
        the radius."""
        (x, y), (qx, qy) = _f2(self.point.pos), _f2(self.point.prev_pos)
        (bx, by), (bw, bh), r = _f2(bounds.pos), _f2(bounds.size), _F(self.radius)
        x, qx = _reflect(x, qx, bx + r, bx + bw - r)
        y, qy = _reflect(y, qy, by + r, by + bh - r)
        self.point.pos, self.point.prev_pos = _py((x, y)), _py((qx, qy))

    def solve_circle(self, circle: "Circle") -> None:
        """src/circle.rs:32-45: overlapping discs pushed apart, each by the
        other's share of the squared radii."""
        (ax, ay), (bx, by) = _f2(self.point.pos), _f2(circle.point.pos)
        ra, rb = _F(self.radius), _F(circle.radius)
        dx, dy = ax - bx, ay - by
        d2 = dx * dx + dy * dy
        rs = ra + rb
        if d2 < rs * rs:
            n = _norm(dx, dy)
            nx, ny = dx / n, dy / n
            overlap = rs - np.sqrt(d2)
            ra2, rb2 = ra * ra, rb * rb
            scale = _F(1.0) / (ra2 + rb2)
            self.point.pos = _py((ax + nx * scale * overlap * rb2, ay + ny * scale * overlap * rb2))
            circle.point.pos = _py((bx - nx * scale * overlap * ra2,
                                    by - ny * scale * overlap * ra2))


@dataclass
class Bounds:  # src/solver.rs:13-17
    pos: tuple
    size: tuple


@dataclass
class Polygon:  # src/polygon.rs:7-14
    particles: list
    particle_links: list
    is_static: bool
    center: tuple
    scale: float = 1.0

    @staticmethod
    def circle(radius: float, pos, point_count: int, is_static: bool) -> "Polygon":
        """Polygon::circle, src/polygon.rs:17-82 (built by the native host code)."""
        s = Solver()
        s._chk(s._lib.b2d_add_polygon_circle(s._h, radius, N.Vec2(*_v(pos)), point_count,
                                             int(is_static)))
        return s.get_polygon(0)

    @staticmethod
    def new(points: Sequence, is_static: bool) -> "Polygon":
        """Polygon::new, src/polygon.rs:84-123 (built by the native host code)."""
        s = Solver()
        pts = (N.Vec2 * len(points))(*[N.Vec2(*_v(p)) for p in points])
        s._chk(s._lib.b2d_add_polygon_points(s._h, len(points), pts, int(is_static)))
        return s.get_polygon(0)

    def update(self, dt: float) -> None:
        """src/polygon.rs:125-134: centre, then every vertex, unless static."""
        if self.is_static:
            return
        self._calc_center()
        for p in self.particles:
            p.update(dt)

    def solve_bounds(self, bounds: Bounds) -> None:  # src/polygon.rs:136-140
        for p in self.particles:
            p.solve_bounds(bounds)

    def solve_polygon(self, other: "Polygon") -> None:  # src/polygon.rs:142-145
        self.solve_polygon_single(other)
        other.solve_polygon_single(self)

    def solve_polygon_single(self, other: "Polygon") -> None:
        """src/polygon.rs:147-162: every edge (i, i+1) against every vertex
        of other; the edge's end points are copied when the edge starts and
        the copies serve all of other's vertices, while each hit writes both
        end points and the vertex."""
        n = len(self.particles)
        for i in range(n):
            j = (i + 1) % n
            a, b = _f2(self.particles[i].pos), _f2(self.particles[j].pos)
            for q in other.particles:
                hit = _edge_contact(_f2(self.center), a, b, _f2(q.pos), _f2(other.center))
                if hit is not None:
                    self.particles[i].pos, self.particles[j].pos, q.pos = (_py(v) for v in hit)

    def solve_links(self) -> None:  # src/polygon.rs:218-223
        self._calc_center()
        for link in self.particle_links:
            link.solve(self.particles)

    def add_force_v2(self, force) -> None:  # src/polygon.rs:225-229
        for p in self.particles:
            p.add_force_v2(force)

    def _calc_center(self) -> None:
        """src/polygon.rs:231-237: summed from zero in vertex order, then
        divided by the count."""
        cx, cy = _F(0.0), _F(0.0)
        for p in self.particles:
            px, py = _f2(p.pos)
            cx, cy = cx + px, cy + py
        k = _F(len(self.particles))
        self.center = _py((cx / k, cy / k))


def _edge_contact(center, a, b, q, other_center):
    """src/polygon.rs:164-216: vertex q of a polygon with centre
    other_center against edge a-b of a polygon with centre `center`.  The
    segment q-other_center must cross the edge; the edge then moves two
    thirds of q's depth along the edge's inward normal, shared by a and b in
    proportion to the crossing's distance from the other end, and q moves to
    where a ray from it against that normal (length 10000) crosses the old
    edge.  None when either crossing is missing."""
    hit = line_intersection((a, b), (q, other_center))
    if hit is None:
        return None
    hx, hy = _f2(hit)
    ex, ey = b[0] - a[0], b[1] - a[1]
    en = _norm(ex, ey)
    ux, uy = ex / en, ey / en
    cx, cy = center[0] - hx, center[1] - hy
    s = (ux * cx + uy * cy) / (ux * ux + uy * uy)
    px, py = s * ux, s * uy
    ix, iy = center[0] - (hx + px), center[1] - (hy + py)
    inn = _norm(ix, iy)
    nx, ny = ix / inn, iy / inn
    to_a = _norm(hx - a[0], hy - a[1])
    to_b = _norm(hx - b[0], hy - b[1])
    length = to_a + to_b
    share_a, share_b = to_b / length, to_a / length
    dx, dy = hx - q[0], hy - q[1]
    t = (nx * dx + ny * dy) / (nx * nx + ny * ny)
    ox, oy = t * nx, t * ny
    mx, my = ox / _F(3.0) * _F(2.0), oy / _F(3.0) * _F(2.0)
    new_a = (a[0] - share_a * mx, a[1] - share_a * my)
    new_b = (b[0] - share_b * mx, b[1] - share_b * my)
    far = (q[0] - nx * _F(10000.0), q[1] - ny * _F(10000.0))
    new_q = line_intersection((a, b), (q, far))
    if new_q is None:
        return None
    return new_a, new_b, _f2(new_q)


def line_intersection(line1, line2):
    """common::line_intersection, src/common.rs:3-26: parameters s (along
    line2) and t (along line1) in [0, 1] give p1 + t * (p2 - p1); parallel
    segments give a non-finite s or t and no hit.  f32, the reference's
    operation order (the denominator is evaluated twice)."""
    (p1, p2), (p3, p4) = (_f2(line1[0]), _f2(line1[1])), (_f2(line2[0]), _f2(line2[1]))
    s1x, s1y = p2[0] - p1[0], p2[1] - p1[1]
    s2x, s2y = p4[0] - p3[0], p4[1] - p3[1]
    with np.errstate(divide="ignore", invalid="ignore"):
        s = (-s1y * (p1[0] - p3[0]) + s1x * (p1[1] - p3[1])) / (-s2x * s1y + s1x * s2y)
        t = (s2x * (p1[1] - p3[1]) - s2y * (p1[0] - p3[0])) / (-s2x * s1y + s1x * s2y)
    if _F(0.0) <= s <= _F(1.0) and _F(0.0) <= t <= _F(1.0):
        return _py((p1[0] + t * s1x, p1[1] + t * s1y))
    return None


def _cpart(p: Particle) -> N.CParticle:
    return N.CParticle(N.Vec2(*p.pos), N.Vec2(*p.prev_pos), N.Vec2(*p.acc))


def _ppart(c: N.CParticle) -> Particle:
    return Particle((c.pos.x, c.pos.y), (c.prev_pos.x, c.prev_pos.y), (c.acc.x, c.acc.y))


def _f32p(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_float))


class Solver:
    """src/solver.rs:19-189 — state lives on the GPU between updates."""

    def __init__(self):
        self._lib = N.load()
        h = C.c_void_p()
        N.check(self._lib.b2d_solver_create(C.byref(h)))
        self._h = h

    @staticmethod
    def new() -> "Solver":  # src/solver.rs:34-50
        return Solver()

    def _chk(self, code: int) -> None:
        N.check(code)

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.b2d_solver_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def clone(self) -> "Solver":  # #[derive(Clone)], src/solver.rs:19
        out = Solver.__new__(Solver)
        out._lib = self._lib
        h = C.c_void_p()
        self._chk(self._lib.b2d_solver_clone(self._h, C.byref(h)))
        out._h = h
        return out

    # ---- pub fields (src/solver.rs:21-23)
    @property
    def gravity(self) -> tuple:
        v = N.Vec2()
        self._chk(self._lib.b2d_get_gravity(self._h, C.byref(v)))
        return (v.x, v.y)

    @gravity.setter
    def gravity(self, g) -> None:
        self._chk(self._lib.b2d_set_gravity(self._h, *_v(g)))

    @property
    def bounds(self) -> Bounds:
        p, s = N.Vec2(), N.Vec2()
        self._chk(self._lib.b2d_get_bounds(self._h, C.byref(p), C.byref(s)))
        return Bounds((p.x, p.y), (s.x, s.y))

    @bounds.setter
    def bounds(self, b: Bounds) -> None:
        self._chk(self._lib.b2d_set_bounds(self._h, *_v(b.pos), *_v(b.size)))

    @property
    def bounds_active(self) -> bool:
        v = C.c_int()
        self._chk(self._lib.b2d_get_bounds_active(self._h, C.byref(v)))
        return bool(v.value)

    @bounds_active.setter
    def bounds_active(self, on: bool) -> None:
        self._chk(self._lib.b2d_set_bounds_active(self._h, int(on)))

    # ---- add_* (src/solver.rs:52-67)
    def add_particle(self, pos) -> None:
        self._chk(self._lib.b2d_add_particle(self._h, *_v(pos)))

    def add_circle(self, circle: Circle) -> None:
        c = N.CCircle(_cpart(circle.point), circle.radius, int(circle.is_static))
        self._chk(self._lib.b2d_add_circle(self._h, C.byref(c)))

    def add_polygon(self, polygon: Polygon) -> None:
        nv, nl = len(polygon.particles), len(polygon.particle_links)
        v = (N.CParticle * max(nv, 1))(*[_cpart(p) for p in polygon.particles])
        links = []
        for pl in polygon.particle_links:
            l = pl.link if isinstance(pl, ParticleLink) else pl
            links.append(N.CLink(l.particle_a, l.particle_b, l.target_distance, 1.0))
        la = (N.CLink * max(nl, 1))(*links)
        self._chk(self._lib.b2d_add_polygon(self._h, nv, v, nl, la, int(polygon.is_static),
                                            N.Vec2(*polygon.center), polygon.scale))

    def add_particle_link(self, link) -> None:
        l = link.link if isinstance(link, ParticleLink) else link
        if l.stiffness == 1.0:
            self._chk(self._lib.b2d_add_particle_link(self._h, l.particle_a, l.particle_b,
                                                      l.target_distance))
        else:
            self.add_particle_links([l.particle_a], [l.particle_b], [l.target_distance],
                                    [l.stiffness])

    def add_circle_link(self, link) -> None:
        l = link.link if isinstance(link, CircleLink) else link
        self._chk(self._lib.b2d_add_circle_link(self._h, l.particle_a, l.particle_b,
                                                l.target_distance))

    # ---- extension: bulk and initial velocity
    def add_particle_prev(self, pos, prev) -> None:
        self._chk(self._lib.b2d_add_particle_prev(self._h, *_v(pos), *_v(prev)))

    def add_particles(self, pos: np.ndarray, prev: Optional[np.ndarray] = None) -> None:
        pos = np.ascontiguousarray(pos, dtype=np.float32).reshape(-1, 2)
        if prev is not None:
            prev = np.ascontiguousarray(prev, dtype=np.float32).reshape(-1, 2)
        self._chk(self._lib.b2d_add_particles(self._h, len(pos), _f32p(pos), _f32p(prev)))

    def add_particle_links(self, a, b, target, stiffness=None) -> None:
        a = np.ascontiguousarray(a, dtype=np.uint64)
        b = np.ascontiguousarray(b, dtype=np.uint64)
        t = np.ascontiguousarray(target, dtype=np.float32)
        k = None if stiffness is None else np.ascontiguousarray(stiffness, dtype=np.float32)
        u64 = C.POINTER(C.c_uint64)
        self._chk(self._lib.b2d_add_particle_links(self._h, len(a), a.ctypes.data_as(u64),
                                                   b.ctypes.data_as(u64), _f32p(t), _f32p(k)))

    def add_polygon_circle(self, radius, pos, point_count, is_static) -> None:
        self._chk(self._lib.b2d_add_polygon_circle(self._h, radius, N.Vec2(*_v(pos)),
                                                   point_count, int(is_static)))

    def add_polygon_points(self, points, is_static) -> None:
        pts = (N.Vec2 * max(len(points), 1))(*[N.Vec2(*_v(p)) for p in points])
        self._chk(self._lib.b2d_add_polygon_points(self._h, len(points), pts, int(is_static)))

    # ---- extension knobs
    @property
    def sub_steps(self) -> int:
        v = C.c_uint32()
        self._chk(self._lib.b2d_get_sub_steps(self._h, C.byref(v)))
        return v.value

    def set_sub_steps(self, n: int) -> None:
        self._chk(self._lib.b2d_set_sub_steps(self._h, n))

    def set_link_iters(self, n: int) -> None:
        self._chk(self._lib.b2d_set_link_iters(self._h, n))

    def set_mode(self, mode: int) -> None:
        self._chk(self._lib.b2d_set_mode(self._h, mode))

    def set_collision(self, flags: int, particle_radius: float = 0.5, grid_cell: float = 1.0):
        self._chk(self._lib.b2d_set_collision(self._h, flags, particle_radius, grid_cell))

    def set_circle_static(self, index: int, is_static: bool) -> None:
        self._chk(self._lib.b2d_set_circle_static(self._h, index, int(is_static)))

    def set_tuning(self, **kv) -> None:
        """Executor tunables (see include/bendy2d.h b2d_set_tuning)."""
        for k, v in kv.items():
            self._chk(self._lib.b2d_set_tuning(self._h, k.encode(), float(v)))

    def set_fault(self, kind: int, value: int) -> None:
        """Fault injection for tests of failure detection (FAULT_* of
        _native; value 0 turns it off)."""
        self._chk(self._lib.b2d_set_fault(self._h, int(kind), int(value)))

    # ---- update (src/solver.rs:106-116)
    def update(self, dt: float) -> None:
        self._chk(self._lib.b2d_update(self._h, dt))

    # ---- getters (src/solver.rs:69-104)
    def _len(self, fn) -> int:
        v = C.c_size_t()
        self._chk(fn(self._h, C.byref(v)))
        return v.value

    def get_particle_len(self) -> int:
        return self._len(self._lib.b2d_get_particle_len)

    def get_circles_len(self) -> int:
        return self._len(self._lib.b2d_get_circles_len)

    def get_polygons_len(self) -> int:
        return self._len(self._lib.b2d_get_polygons_len)

    def _links(self, lenfn, getfn, wrap) -> list:
        n = self._len(lenfn)
        buf = (N.CLink * max(n, 1))()
        self._chk(getfn(self._h, buf, n))
        return [wrap(Link(buf[i].particle_a, buf[i].particle_b, buf[i].target_distance,
                          buf[i].stiffness)) for i in range(n)]

    def get_particle_links(self) -> list:
        return self._links(self._lib.b2d_get_particle_links_len, self._lib.b2d_get_particle_links,
                           ParticleLink)

    def get_circle_links(self) -> list:
        return self._links(self._lib.b2d_get_circle_links_len, self._lib.b2d_get_circle_links,
                           CircleLink)

    def get_particles(self) -> list:
        n = self.get_particle_len()
        buf = (N.CParticle * max(n, 1))()
        self._chk(self._lib.b2d_get_particles(self._h, buf, n))
        return [_ppart(buf[i]) for i in range(n)]

    def get_circles(self) -> list:
        n = self.get_circles_len()
        buf = (N.CCircle * max(n, 1))()
        self._chk(self._lib.b2d_get_circles(self._h, buf, n))
        return [Circle(_ppart(buf[i].point), buf[i].radius, bool(buf[i].is_static))
                for i in range(n)]

    def get_polygons(self) -> list:
        return [self.get_polygon(i) for i in range(self.get_polygons_len())]

    def get_particle(self, index: int) -> Optional[Particle]:
        c = N.CParticle()
        code = self._lib.b2d_get_particle(self._h, index, C.byref(c))
        if code == 6:
            return None
        self._chk(code)
        return _ppart(c)

    def get_circle(self, index: int) -> Optional[Circle]:
        c = N.CCircle()
        code = self._lib.b2d_get_circle(self._h, index, C.byref(c))
        if code == 6:
            return None
        self._chk(code)
        return Circle(_ppart(c.point), c.radius, bool(c.is_static))

    def get_polygon(self, index: int) -> Optional[Polygon]:
        nv, nl = C.c_size_t(), C.c_size_t()
        st, ctr, sc = C.c_int(), N.Vec2(), C.c_float()
        code = self._lib.b2d_get_polygon_info(self._h, index, C.byref(nv), C.byref(nl),
                                              C.byref(st), C.byref(ctr), C.byref(sc))
        if code == 6:
            return None
        self._chk(code)
        vb = (N.CParticle * max(nv.value, 1))()
        lb = (N.CLink * max(nl.value, 1))()
        self._chk(self._lib.b2d_get_polygon(self._h, index, vb, nv.value, lb, nl.value))
        parts = [_ppart(vb[i]) for i in range(nv.value)]
        links = [ParticleLink(Link(lb[i].particle_a, lb[i].particle_b, lb[i].target_distance))
                 for i in range(nl.value)]
        return Polygon(parts, links, bool(st.value), (ctr.x, ctr.y), sc.value)

    # ---- bulk state
    def read_state(self) -> tuple[np.ndarray, np.ndarray]:
        n = self.get_particle_len()
        pos = np.empty((n, 2), np.float32)
        prev = np.empty((n, 2), np.float32)
        self._chk(self._lib.b2d_read_state(self._h, _f32p(pos), _f32p(prev)))
        return pos, prev

    def write_state(self, pos: np.ndarray, prev: np.ndarray) -> None:
        pos = np.ascontiguousarray(pos, dtype=np.float32)
        prev = np.ascontiguousarray(prev, dtype=np.float32)
        self._chk(self._lib.b2d_write_state(self._h, _f32p(pos), _f32p(prev)))

    # ---- execution control
    def set_stream(self, stream_ptr: int) -> None:
        self._chk(self._lib.b2d_set_stream(self._h, C.c_void_p(stream_ptr)))

    def synchronize(self) -> None:
        self._chk(self._lib.b2d_synchronize(self._h))

    def set_graphs(self, on: bool) -> None:
        self._chk(self._lib.b2d_set_graphs(self._h, int(on)))

    def set_profiling(self, on: bool) -> None:
        self._chk(self._lib.b2d_set_profiling(self._h, int(on)))

    def profile(self) -> dict:
        return _profile(self._lib.b2d_get_profile, self._h)

    def launch_count(self) -> int:
        v = C.c_uint32()
        self._chk(self._lib.b2d_get_launch_count(self._h, C.byref(v)))
        return v.value

    def state_bytes(self) -> int:
        return self._len(self._lib.b2d_state_bytes)

    def state_upload_async(self, host_ptr: int) -> None:
        self._chk(self._lib.b2d_state_upload_async(self._h, C.c_void_p(host_ptr)))

    def state_download_async(self, host_ptr: int) -> None:
        self._chk(self._lib.b2d_state_download_async(self._h, C.c_void_p(host_ptr)))

    def plan_stats(self) -> dict:
        s = N.CPlanStats()
        self._chk(self._lib.b2d_get_plan_stats(self._h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in N.CPlanStats._fields_}

    def link_order(self) -> np.ndarray:
        n = self._len(self._lib.b2d_get_particle_links_len)
        out = np.empty(n, np.uint64)
        self._chk(self._lib.b2d_get_link_order(self._h, out.ctypes.data_as(C.POINTER(C.c_uint64)),
                                               n))
        return out


def _profile(fn, h) -> dict:
    names = C.create_string_buffer(4096)
    ms = (C.c_float * 64)()
    cnt = C.c_size_t()
    N.check(fn(h, names, 4096, ms, 64, C.byref(cnt)))
    keys = names.value.decode().split("\n") if cnt.value else []
    return {k: ms[i] for i, k in enumerate(keys)}


class Batch:
    """Many independent solvers stepped by one launch sequence (extension)."""

    def __init__(self, solvers: Iterable[Solver] = ()):
        self._lib = N.load()
        h = C.c_void_p()
        N.check(self._lib.b2d_batch_create(C.byref(h)))
        self._h = h
        self.members: list[Solver] = []
        for s in solvers:
            self.add(s)

    def add(self, s: Solver) -> None:
        N.check(self._lib.b2d_batch_add(self._h, s._h))
        self.members.append(s)

    def remove(self, s: Solver) -> None:
        N.check(self._lib.b2d_batch_remove(self._h, s._h))
        self.members.remove(s)

    def update(self, dt: float) -> None:
        N.check(self._lib.b2d_batch_update(self._h, dt))

    def synchronize(self) -> None:
        N.check(self._lib.b2d_batch_synchronize(self._h))

    def set_stream(self, stream_ptr: int) -> None:
        N.check(self._lib.b2d_batch_set_stream(self._h, C.c_void_p(stream_ptr)))

    def set_profiling(self, on: bool) -> None:
        N.check(self._lib.b2d_batch_set_profiling(self._h, int(on)))

    def profile(self) -> dict:
        return _profile(self._lib.b2d_batch_get_profile, self._h)

    def launch_count(self) -> int:
        v = C.c_uint32()
        N.check(self._lib.b2d_batch_get_launch_count(self._h, C.byref(v)))
        return v.value

    def set_tuning(self, **kv) -> None:
        for k, v in kv.items():
            N.check(self._lib.b2d_batch_set_tuning(self._h, k.encode(), float(v)))

    def set_plain(self, on: bool) -> None:
        """One-world-per-launch baseline: no batching, no CUDA graph."""
        N.check(self._lib.b2d_batch_set_plain(self._h, int(on)))

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.b2d_batch_destroy(self._h)
            self._h = None
            self.members = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
