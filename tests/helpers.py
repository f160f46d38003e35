"""Shared test helpers: load known-answer scenes into the oracle or the GPU
solver, and compare states bit for bit (NaN-aware)."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"


def kat_cases() -> dict:
    return json.loads((GOLDEN / "kat_reference.json").read_text())


def kat_to_oracle(sc: dict):
    from oracle import Oracle
    o = Oracle()
    o.set_gravity(*sc["gravity"])
    o.set_bounds(*sc["bounds"])
    o.set_sub_steps(sc["sub_steps"])
    o.set_link_iters(sc["link_iters"])
    if sc["particles"]:
        o.add_particles(np.asarray(sc["particles"], np.float32), np.asarray(sc["prev"], np.float32))
    if sc["links"]:
        L = np.asarray(sc["links"], np.float64)
        o.add_particle_links(L[:, 0].astype(np.uint64), L[:, 1].astype(np.uint64), L[:, 2], L[:, 3])
    for c in sc["circles"]:
        o.add_circle(c["pos"], c["prev"], c["acc"], c["radius"], c["static"])
    for a, b, r in sc["circle_links"]:
        o.add_circle_link(int(a), int(b), float(r))
    for g in sc["polygons"]:
        o.add_polygon_points(np.asarray(g["points"], np.float32), g["static"])
    for g in sc.get("polygons_full", []):  # Solver::add_polygon with given links and centre
        o.add_polygon(np.asarray(g["pos"], np.float32), np.asarray(g["prev"], np.float32),
                      np.asarray(g["acc"], np.float32), [tuple(l) for l in g["links"]],
                      g["static"], tuple(g["center"]))
    for g in sc.get("polygon_circles", []):  # Polygon::circle
        o.add_polygon_circle(g["radius"], g["pos"][0], g["pos"][1], g["n"], g["static"])
    return o


def kat_to_solver(sc: dict):
    from bendy2d_gb300 import Bounds, Circle, CircleLink, Link, Particle, ParticleLink, Solver
    s = Solver()
    s.gravity = tuple(sc["gravity"])
    s.bounds = Bounds(tuple(sc["bounds"][:2]), tuple(sc["bounds"][2:]))
    s.set_sub_steps(sc["sub_steps"])
    s.set_link_iters(sc["link_iters"])
    if sc["particles"]:
        s.add_particles(np.asarray(sc["particles"], np.float32), np.asarray(sc["prev"], np.float32))
    if sc["links"]:
        L = np.asarray(sc["links"], np.float64)
        s.add_particle_links(L[:, 0].astype(np.uint64), L[:, 1].astype(np.uint64), L[:, 2], L[:, 3])
    for c in sc["circles"]:
        s.add_circle(Circle(Particle(tuple(c["pos"]), tuple(c["prev"]), tuple(c["acc"])),
                            c["radius"], c["static"]))
    for a, b, r in sc["circle_links"]:
        s.add_circle_link(CircleLink(Link(int(a), int(b), float(r))))
    for g in sc["polygons"]:
        s.add_polygon_points([tuple(p) for p in g["points"]], g["static"])
    from bendy2d_gb300 import Polygon
    for g in sc.get("polygons_full", []):
        pos, prev, acc = (np.asarray(g[k], np.float32).reshape(-1, 2) for k in ("pos", "prev", "acc"))
        s.add_polygon(Polygon([Particle(tuple(map(float, a)), tuple(map(float, b)),
                                        tuple(map(float, c))) for a, b, c in zip(pos, prev, acc)],
                              [ParticleLink(Link(int(a), int(b), float(t))) for a, b, t in g["links"]],
                              g["static"], tuple(g["center"])))
    for g in sc.get("polygon_circles", []):
        s.add_polygon_circle(g["radius"], tuple(g["pos"]), g["n"], g["static"])
    return s


def same_bits(a, b) -> bool:
    """Bit-exact float32 equality, with every NaN equal to every NaN."""
    a = np.asarray(a, np.float32).ravel()
    b = np.asarray(b, np.float32).ravel()
    if a.shape != b.shape:
        return False
    na, nb = np.isnan(a), np.isnan(b)
    if not np.array_equal(na, nb):
        return False
    return np.array_equal(a[~na].view(np.uint32), b[~nb].view(np.uint32))


def rel_err(x, ref) -> float:
    """max |x - ref| / max(|ref|, 1) per component."""
    x = np.asarray(x, np.float64)
    ref = np.asarray(ref, np.float64)
    if x.size == 0:
        return 0.0
    return float(np.max(np.abs(x - ref) / np.maximum(np.abs(ref), 1.0)))


def solver_state(s):
    """(pos, prev, circles_pos, circles_prev, [(poly_pos, poly_prev, centre)])"""
    pos, prev = s.read_state()
    cs = s.get_circles()
    cp = np.asarray([c.point.pos for c in cs], np.float32).reshape(-1, 2)
    cq = np.asarray([c.point.prev_pos for c in cs], np.float32).reshape(-1, 2)
    polys = []
    for g in s.get_polygons():
        polys.append((np.asarray([p.pos for p in g.particles], np.float32).reshape(-1, 2),
                      np.asarray([p.prev_pos for p in g.particles], np.float32).reshape(-1, 2),
                      np.asarray(g.center, np.float32)))
    return pos, prev, cp, cq, polys


def oracle_state(o):
    pos, prev = o.particles()
    cp, cq = o.circles()
    return pos, prev, cp, cq, o.polygons()


def assert_same_state(gpu_state, orc_state, what=""):
    names = ["particle pos", "particle prev", "circle pos", "circle prev"]
    for k in range(4):
        assert same_bits(gpu_state[k], orc_state[k]), f"{what}: {names[k]} differs " \
            f"(max rel err {rel_err(gpu_state[k], orc_state[k]):.3g})"
    assert len(gpu_state[4]) == len(orc_state[4])
    for i, (g, o) in enumerate(zip(gpu_state[4], orc_state[4])):
        for k, nm in enumerate(["pos", "prev", "centre"]):
            assert same_bits(g[k], o[k]), f"{what}: polygon {i} {nm} differs"
