"""Seeded synthetic scenes for the five benchmark configurations.

No public dataset exists for this path; every scene is generated from a
numpy PCG64 stream with the shapes, sizes and distributions of the
configuration it stands for.  All state is float32.  Particle links are
emitted in a natural builder order: structural links row-major (right, then
down, per particle), then shear links row-major (both diagonals per cell);
rest length = initial distance computed in float32 as the reference would,
``(a - b).magnitude()``.

A Scene is plain data; ``Scene.to_solver()`` loads it through the public API.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from .api import COLLIDE_PC, COLLIDE_PP, COLLIDE_PPOLY, MODE_FAST, MODE_REFERENCE, Solver

F32 = np.float32


def f32_dist(pa: np.ndarray, pb: np.ndarray) -> np.ndarray:
    """nalgebra magnitude in float32: sqrt(0 + (dx*dx + dy*dy))."""
    d = (pa - pb).astype(F32)
    return np.sqrt(F32(0.0) + (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1])).astype(F32)


@dataclass
class Scene:
    name: str
    pos: np.ndarray                      # (N,2) f32
    prev: np.ndarray                     # (N,2) f32
    la: np.ndarray                       # (L,) u64
    lb: np.ndarray
    rest: np.ndarray                     # (L,) f32
    stiff: np.ndarray                    # (L,) f32
    circles: list = field(default_factory=list)       # dicts: pos, prev, acc, radius, static
    circle_links: list = field(default_factory=list)  # (a, b, rest)
    polygons: list = field(default_factory=list)      # dicts: points (n,2) f32, static
    gravity: tuple = (0.0, -9.81)
    bounds: tuple = (0.0, 0.0, 100.0, 100.0)
    sub_steps: int = 8
    link_iters: int = 4
    mode: int = MODE_REFERENCE
    collide: int = 0
    radius: float = 0.5
    cell: float = 1.0
    dt: float = 1.0 / 60.0
    steps: int = 1

    @property
    def n_particles(self) -> int:
        return len(self.pos)

    def to_solver(self, solver: Optional[Solver] = None) -> Solver:
        s = solver or Solver()
        s.gravity = self.gravity
        from .api import Bounds
        s.bounds = Bounds(self.bounds[:2], self.bounds[2:])
        s.set_sub_steps(self.sub_steps)
        s.set_link_iters(self.link_iters)
        s.set_mode(self.mode)
        s.set_collision(self.collide, self.radius, self.cell)
        s.add_particles(self.pos, self.prev)
        if len(self.la):
            s.add_particle_links(self.la, self.lb, self.rest,
                                 None if np.all(self.stiff == 1.0) else self.stiff)
        from .api import Circle, CircleLink, Link, Particle
        for c in self.circles:
            s.add_circle(Circle(Particle(tuple(c["pos"]), tuple(c["prev"]), tuple(c["acc"])),
                                float(c["radius"]), bool(c["static"])))
        for a, b, r in self.circle_links:
            s.add_circle_link(CircleLink(Link(int(a), int(b), float(r))))
        for g in self.polygons:
            s.add_polygon_points([tuple(p) for p in g["points"]], bool(g["static"]))
        return s


# ---------------------------------------------------------------- builders
def grid_body(w: int, h: int, origin, spacing: float, jitter: float, rng):
    """w x h cloth grid: positions, structural then shear links (row-major)."""
    ys, xs = np.mgrid[0:h, 0:w]
    pos = np.stack([origin[0] + spacing * xs.ravel(), origin[1] + spacing * ys.ravel()], 1)
    pos = pos + rng.uniform(-jitter, jitter, size=pos.shape)
    pos = pos.astype(F32)
    idx = lambda x, y: y * w + x  # noqa: E731
    a, b = [], []
    for y in range(h):
        for x in range(w):
            if x + 1 < w:
                a.append(idx(x, y)); b.append(idx(x + 1, y))
            if y + 1 < h:
                a.append(idx(x, y)); b.append(idx(x, y + 1))
    for y in range(h - 1):
        for x in range(w - 1):
            a.append(idx(x, y)); b.append(idx(x + 1, y + 1))
            a.append(idx(x + 1, y)); b.append(idx(x, y + 1))
    a = np.asarray(a, np.uint64)
    b = np.asarray(b, np.uint64)
    return pos, a, b


def partial_grid(n: int, w: int, origin, spacing, jitter, rng):
    """First n particles of a w-wide grid (last row may be partial)."""
    h = (n + w - 1) // w
    pos, a, b = grid_body(w, h, origin, spacing, jitter, rng)
    keep = (a < n) & (b < n)
    return pos[:n], a[keep], b[keep]


def ring_body(n_rim: int, center, radius: float):
    """n rim particles on a circle plus a centre particle (last); rim links
    i -> i+1 (mod n, a<b), then spokes i -> centre."""
    th = 2.0 * np.pi * np.arange(n_rim) / n_rim
    rim = np.stack([center[0] + radius * np.cos(th), center[1] + radius * np.sin(th)], 1)
    pos = np.vstack([rim, [center]]).astype(F32)
    a, b = [], []
    for i in range(n_rim):
        j = (i + 1) % n_rim
        a.append(min(i, j)); b.append(max(i, j))
    for i in range(n_rim):
        a.append(i); b.append(n_rim)
    return pos, np.asarray(a, np.uint64), np.asarray(b, np.uint64)


def convex_polygon(rng, center, radius, k):
    th = np.sort(rng.uniform(0.0, 2.0 * np.pi, size=k))
    pts = np.stack([center[0] + radius * np.cos(th), center[1] + radius * np.sin(th)], 1)
    return pts.astype(F32)


def _assemble(name, bodies, **kw) -> Scene:
    pos, la, lb = [], [], []
    off = 0
    for p, a, b in bodies:
        pos.append(p)
        la.append(a + off)
        lb.append(b + off)
        off += len(p)
    pos = np.vstack(pos).astype(F32) if pos else np.zeros((0, 2), F32)
    la = np.concatenate(la).astype(np.uint64) if la else np.zeros(0, np.uint64)
    lb = np.concatenate(lb).astype(np.uint64) if lb else np.zeros(0, np.uint64)
    rest = f32_dist(pos[la.astype(np.int64)], pos[lb.astype(np.int64)]) if len(la) else \
        np.zeros(0, F32)
    prev = kw.pop("prev", None)
    stiff = kw.pop("stiff", None)
    return Scene(name=name, pos=pos, prev=pos.copy() if prev is None else prev.astype(F32),
                 la=la, lb=lb, rest=rest,
                 stiff=np.ones(len(la), F32) if stiff is None else stiff.astype(F32), **kw)


def _circle(pos, radius, static, prev=None):
    p = np.asarray(pos, F32)
    return {"pos": p, "prev": p.copy() if prev is None else np.asarray(prev, F32),
            "acc": np.zeros(2, F32), "radius": F32(radius), "static": bool(static)}


def _velocity_prev(pos, rng, sigma, h):
    v = rng.normal(0.0, sigma, size=pos.shape)
    return (pos - v * h).astype(F32)


# ---------------------------------------------------------------- configs
def config1(seed: int = 0, steps: int = 600) -> Scene:
    """32x32 cloth (1024 particles, 1984 structural + 1922 shear links), 4 static
    circles r=5, a static rectangular floor polygon, box 100^2, g=(0,-9.81),
    dt=1/60, 8 sub-steps, 4 link iterations; reference semantics (no
    extension collisions)."""
    rng = np.random.default_rng(seed)
    body = grid_body(32, 32, (34.0, 50.0), 1.0, 0.01, rng)
    circles = [_circle(rng.uniform(0.0, 100.0, 2), 5.0, True) for _ in range(4)]
    floor = {"points": np.array([[0, 0], [100, 0], [100, 4], [0, 4]], F32), "static": True}
    return _assemble("config1_cloth", [body], circles=circles, polygons=[floor],
                     bounds=(0.0, 0.0, 100.0, 100.0), sub_steps=8, link_iters=4, steps=steps)


def config2(seed: int = 0, n_bodies: int = 64, box: float = 2000.0, n_circles: int = 16,
            n_polys: int = 8, collide: int = COLLIDE_PP | COLLIDE_PC | COLLIDE_PPOLY,
            mode: int = MODE_REFERENCE) -> Scene:
    """64 cloth grids of 32x32 (65,536 particles, 249,984 links) at seeded
    uniform offsets in a 2000^2 box, initial velocities N(0, 0.5), particle
    collisions on (r=0.5, cell 1.0), 16 circles r~U[5,30], 8 convex polygons
    (4-8 vertices, hull radius U[10,50]); 8 sub-steps, 4 link iterations."""
    rng = np.random.default_rng(seed)
    bodies = [grid_body(32, 32, rng.uniform(0.0, box - 32.0, 2), 1.0, 0.01, rng)
              for _ in range(n_bodies)]
    h = (1.0 / 60.0) / 8.0
    circles = [_circle(rng.uniform(0.0, box, 2), rng.uniform(5.0, 30.0), False)
               for _ in range(n_circles)]
    m = min(50.0, 0.25 * box)  # small test boxes shrink the hull radius range
    polys = [{"points": convex_polygon(rng, rng.uniform(m, box - m, 2),
                                       rng.uniform(min(10.0, 0.5 * m), m),
                                       int(rng.integers(4, 9))),
              "static": False} for _ in range(n_polys)]
    sc = _assemble("config2_64grids", bodies, circles=circles, polygons=polys,
                   bounds=(0.0, 0.0, box, box), sub_steps=8, link_iters=4, collide=collide,
                   mode=mode)
    sc.prev = _velocity_prev(sc.pos, rng, 0.5, h)
    return sc


def config3_world(rng, n_target: int, box: float = 1000.0, link_iters: int = 1) -> Scene:
    """One batched world: 1-8 rings (n rim + centre, rim + spoke links,
    stiffness U[0.3,1]), 2 circles and a floor polygon."""
    n_rings = int(rng.integers(1, 9))
    n_rings = max(1, min(n_rings, n_target // 4))
    sizes = np.full(n_rings, n_target // n_rings)
    sizes[: n_target - sizes.sum()] += 1
    bodies, stiff = [], []
    for sz in sizes:
        r = rng.uniform(5.0, 20.0)
        c = rng.uniform(r + 5.0, box - r - 5.0, 2)
        p, a, b = ring_body(int(sz) - 1, c, r)
        bodies.append((p, a, b))
        stiff.append(np.full(len(a), rng.uniform(0.3, 1.0)))
    circles = [_circle(rng.uniform(50.0, box - 50.0, 2), rng.uniform(5.0, 20.0), False)
               for _ in range(2)]
    floor = {"points": np.array([[0, 0], [box, 0], [box, 10], [0, 10]], F32), "static": True}
    return _assemble("config3_world", bodies, circles=circles, polygons=[floor],
                     bounds=(0.0, 0.0, box, box), sub_steps=8, link_iters=link_iters,
                     stiff=np.concatenate(stiff))


def config3(seed: int = 0, n_worlds: int = 4096, lo: int = 64, hi: int = 4096,
            link_iters: int = 1) -> list:
    """4096 independent worlds, particle counts log-uniform in [64, 4096]."""
    rng = np.random.default_rng(seed)
    ns = np.exp(rng.uniform(np.log(lo), np.log(hi), size=n_worlds)).astype(int)
    return [config3_world(rng, int(n), link_iters=link_iters) for n in ns]


def config4_request(rng, n: int, box: float = 2000.0) -> Scene:
    """A serving request: a config-2-style world of n particles (32-wide grids,
    the last one partial), particle collisions on."""
    bodies = []
    left = n
    while left > 0:
        k = min(left, 1024)
        bodies.append(partial_grid(k, 32, rng.uniform(0.0, box - 32.0, 2), 1.0, 0.01, rng))
        left -= k
    h = (1.0 / 60.0) / 8.0
    sc = _assemble("config4_request", bodies, bounds=(0.0, 0.0, box, box), sub_steps=8,
                   link_iters=4, collide=COLLIDE_PP)
    sc.prev = _velocity_prev(sc.pos, rng, 0.5, h)
    return sc


def config5(seed: int = 0, n_side: int = 32, box: float = 4000.0,
            mode: int = MODE_FAST) -> Scene:
    """1024 cloth grids (1,048,576 particles, 3,999,744 links) packed on a
    lattice in a 4000^2 box, 20 sub-steps, 8 link iterations, particle
    collisions on, 64 static circles r=5 and 32 convex polygons."""
    rng = np.random.default_rng(seed)
    pitch = (box - 100.0) / n_side
    bodies = []
    for gy in range(n_side):
        for gx in range(n_side):
            o = (50.0 + gx * pitch, 50.0 + gy * pitch)
            bodies.append(grid_body(32, 32, o, 1.0, 0.01, rng))
    circles = [_circle(rng.uniform(0.0, box, 2), 5.0, True) for _ in range(64)]
    polys = [{"points": convex_polygon(rng, rng.uniform(50.0, box - 50.0, 2),
                                       rng.uniform(10.0, 50.0), int(rng.integers(4, 9))),
              "static": True} for _ in range(32)]
    return _assemble("config5_1024grids", bodies, circles=circles, polygons=polys,
                     bounds=(0.0, 0.0, box, box), sub_steps=20, link_iters=8,
                     collide=COLLIDE_PP | COLLIDE_PC | COLLIDE_PPOLY, mode=mode)
