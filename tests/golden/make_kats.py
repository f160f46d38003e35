"""Generate tests/golden/kat_reference.json: known-answer cases for the
bendy2d solver step, derived by hand from the reference source.

Each case is a tiny scene whose expected state after N updates follows from
the reference formulas evaluated step by step in float32 (numpy scalars, one
rounding per operation, no fused multiply-add) — written out below in the
order the reference evaluates them.  This is independent of the C oracle and
of the CUDA kernels; both are checked against it.

Run: python tests/golden/make_kats.py
"""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np

f = np.float32
OUT = Path(__file__).resolve().parent / "kat_reference.json"


def v(x, y):
    return np.array([x, y], dtype=f)


def norm(d):  # nalgebra magnitude: sqrt(0 + (x*x + y*y))
    return np.sqrt(f(0) + (d[0] * d[0] + d[1] * d[1]))


def normalize(d):  # component-wise division by the norm
    n = norm(d)
    return np.array([d[0] / n, d[1] / n], dtype=f)


def dot(a, b):
    return a[0] * b[0] + a[1] * b[1]


def integrate(p, q, acc, h):  # src/particle.rs:20-25
    vel = p - q
    return (p + vel) + ((acc * h) * h), p.copy()


def line_intersection(p1, p2, p3, p4):  # src/common.rs:3-26
    s1x, s1y = p2[0] - p1[0], p2[1] - p1[1]
    s2x, s2y = p4[0] - p3[0], p4[1] - p3[1]
    with np.errstate(divide="ignore", invalid="ignore"):  # parallel: inf/NaN, no hit
        s = (-s1y * (p1[0] - p3[0]) + s1x * (p1[1] - p3[1])) / (-s2x * s1y + s1x * s2y)
        t = (s2x * (p1[1] - p3[1]) - s2y * (p1[0] - p3[0])) / (-s2x * s1y + s1x * s2y)
    if s >= 0 and s <= 1 and t >= 0 and t <= 1:
        return np.array([p1[0] + t * s1x, p1[1] + t * s1y], dtype=f)
    return None


def base(**kw):
    c = {"gravity": [0.0, 0.0], "bounds": [0.0, 0.0, 100.0, 100.0], "sub_steps": 1,
         "link_iters": 1, "dt": 1.0, "particles": [], "prev": [], "links": [],
         "circles": [], "circle_links": [], "polygons": []}
    c.update(kw)
    return c


def flat(a):
    return [float(x) for x in np.asarray(a, dtype=f).ravel()]


cases = {}

# 1. free fall from rest (src/particle.rs:20-25): y_k = y0 + g*h^2*k(k+1)/2,
#    g = -8, h = 0.25 -> g*h*h = -0.5 exactly.
p, q = v(50, 50), v(50, 50)
g = v(0, -8)
for _ in range(5):
    acc = f(0) + g                      # apply_gravity on a zeroed acc
    p, q = integrate(p, q, acc, f(0.25))
assert p[1] == f(50 - 0.5 * 15)
cases["free_fall"] = dict(scene=base(gravity=[0.0, -8.0], dt=0.25, particles=[[50, 50]],
                                     prev=[[50, 50]]),
                          steps=5, expect_pos=flat([p]), expect_prev=flat([q]))

# 2. bounds reflection (src/particle.rs:27-46), both sides of x, g = 0, dt = 1.
def bounds_step(p, q, lo, hi):
    p, q = p.copy(), q.copy()
    for ax in range(2):
        if p[ax] < lo[ax]:
            vel = q[ax] - p[ax]; q[ax] = lo[ax] - vel; p[ax] = lo[ax]
        elif p[ax] > lo[ax] + hi[ax]:
            vel = q[ax] - p[ax]; q[ax] = lo[ax] + hi[ax] - vel; p[ax] = lo[ax] + hi[ax]
    return p, q


P = [v(1, 50), v(99, 50)]
Q = [v(3, 50), v(97, 50)]
for _ in range(2):
    for i in range(2):
        P[i], Q[i] = bounds_step(P[i], Q[i], v(0, 0), v(100, 100))
        P[i], Q[i] = integrate(P[i], Q[i], f(0) + v(0, 0), f(1))
assert list(P[0]) == [2, 50] and list(Q[0]) == [0, 50]
assert list(P[1]) == [98, 50] and list(Q[1]) == [100, 50]
cases["bounds_reflect"] = dict(scene=base(particles=[[1, 50], [99, 50]], prev=[[3, 50], [97, 50]]),
                               steps=2, expect_pos=flat(P), expect_prev=flat(Q))

# 3. one particle link, then coincident endpoints -> NaN (src/link.rs:18-27)
def link(a, b, rest, stiff=f(1)):
    d = a - b
    dist = norm(d)
    n = normalize(d)
    corr = ((n * (dist - rest)) * f(0.5)) * stiff
    return a - corr, b + corr


a, b = v(10, 10), v(12, 10)
qa, qb = a.copy(), b.copy()
a, b = link(a, b, f(1))
assert list(a) == [10.5, 10] and list(b) == [11.5, 10]
a, qa = integrate(a, qa, f(0) + v(0, 0), f(1))
b, qb = integrate(b, qb, f(0) + v(0, 0), f(1))
cases["link_pair"] = dict(scene=base(particles=[[10, 10], [12, 10]], prev=[[10, 10], [12, 10]],
                                     links=[[0, 1, 1.0, 1.0]]),
                          steps=1, expect_pos=flat([a, b]), expect_prev=flat([qa, qb]))
with np.errstate(invalid="ignore", divide="ignore"):
    a2, b2 = link(a, b, f(1))
    a2, qa2 = integrate(a2, a.copy(), f(0) + v(0, 0), f(1))
    b2, qb2 = integrate(b2, b.copy(), f(0) + v(0, 0), f(1))
assert np.isnan(a2).all()
cases["link_coincident_nan"] = dict(
    scene=base(particles=[[10, 10], [12, 10]], prev=[[10, 10], [12, 10]],
               links=[[0, 1, 1.0, 1.0]]),
    steps=2, expect_pos=flat([a2, b2]), expect_prev=flat([qa2, qb2]))

# 4. link with stiffness 0.5 (extension: correction scaled last)
a, b = v(10, 10), v(13, 14)
qa, qb = a.copy(), b.copy()
a, b = link(a, b, f(2), f(0.5))
a, qa = integrate(a, qa, f(0) + v(0, 0), f(1))
b, qb = integrate(b, qb, f(0) + v(0, 0), f(1))
cases["link_stiffness"] = dict(scene=base(particles=[[10, 10], [13, 14]], prev=[[10, 10], [13, 14]],
                                          links=[[0, 1, 2.0, 0.5]]),
                               steps=1, expect_pos=flat([a, b]), expect_prev=flat([qa, qb]))

# 5. circle pair overlap (src/circle.rs:32-45), equal radii 2, centres 3 apart
c1, c2 = v(10, 10), v(13, 10)
r1, r2 = f(2), f(2)
d = c1 - c2
d2 = f(0) + (d[0] * d[0] + d[1] * d[1])
rs = r1 + r2
assert d2 < rs * rs
n = normalize(d)
overlap = rs - np.sqrt(d2)
scale = f(1) / (r1 * r1 + r2 * r2)
c1 = c1 + ((n * scale) * overlap) * (r2 * r2)
c2 = c2 - ((n * scale) * overlap) * (r1 * r1)
assert list(c1) == [9.5, 10] and list(c2) == [13.5, 10]
p1, q1 = integrate(c1, v(10, 10), f(0) + v(0, 0), f(1))
p2, q2 = integrate(c2, v(13, 10), f(0) + v(0, 0), f(1))
cases["circle_pair"] = dict(
    scene=base(circles=[{"pos": [10, 10], "prev": [10, 10], "acc": [0, 0], "radius": 2.0,
                         "static": False},
                        {"pos": [13, 10], "prev": [13, 10], "acc": [0, 0], "radius": 2.0,
                         "static": False}]),
    steps=1, expect_circles_pos=flat([p1, p2]), expect_circles_prev=flat([q1, q2]))

# 6. circle link, radius^2-weighted (src/link.rs:36-48); after the link the
#    circles are 3 apart with radius sum 2.5, so the pair test misses.
ca, cb = v(10, 10), v(14, 10)
ra, rb = f(1), f(1.5)
d = ca - cb
dist = norm(d)
n = normalize(d)
ra2, rb2 = ra * ra, rb * rb
scale = f(1) / (ra2 + rb2)
ca = ca - (((n * (dist - f(3))) * scale) * rb2)
cb = cb + (((n * (dist - f(3))) * scale) * ra2)
assert norm(ca - cb) ** 2 >= (ra + rb) ** 2
pa, qa = integrate(ca, v(10, 10), f(0) + v(0, 0), f(1))
pb, qb = integrate(cb, v(14, 10), f(0) + v(0, 0), f(1))
cases["circle_link"] = dict(
    scene=base(circles=[{"pos": [10, 10], "prev": [10, 10], "acc": [0, 0], "radius": 1.0,
                         "static": False},
                        {"pos": [14, 10], "prev": [14, 10], "acc": [0, 0], "radius": 1.5,
                         "static": False}],
               circle_links=[[0, 1, 3.0]]),
    steps=1, expect_circles_pos=flat([pa, pb]), expect_circles_prev=flat([qa, qb]))

# 7. polygon edge hit (src/polygon.rs:142-216): static square A, triangle B
#    whose vertex (15,18) pokes through A's top edge (20,20)-(10,20).
A = [v(10, 10), v(20, 10), v(20, 20), v(10, 20)]
B = [v(15, 18), v(12, 30), v(18, 30)]
Bprev = [x.copy() for x in B]
cA = (((A[0] + A[1]) + A[2]) + A[3]) / f(4)   # calc_center in solve_links
cB = ((B[0] + B[1]) + B[2]) / f(3)
pa, pb, qq = A[2], A[3], B[0]
I = line_intersection(pa, pb, qq, cB)
assert I is not None and list(I) == [15, 20]
nl = normalize(pb - pa)
cp = nl * (dot(nl, cA - I) / dot(nl, nl))
ni = normalize(cA - (I + cp))
da, db = norm(I - pa), norm(I - pb)
dab = da + db
ia, ib = db / dab, da / dab
ion = ni * (dot(ni, I - qq) / dot(ni, ni))
dl = (ion / f(3)) * f(2)
new_a, new_b = pa - dl * ia, pb - dl * ib
hit = line_intersection(pa, pb, qq, qq - ni * f(10000))
assert hit is not None
A[2], A[3], B[0] = new_a, new_b, hit
# remaining edge tests miss (checked by the oracle); bounds no-op; B integrates
cB2 = ((B[0] + B[1]) + B[2]) / f(3)           # Polygon::update calc_center
Bn, Bq = [], []
for x, xq in zip(B, Bprev):
    pn, qn = integrate(x, xq, f(0) + v(0, 0), f(1))
    Bn.append(pn); Bq.append(qn)
cases["polygon_edge_hit"] = dict(
    scene=base(polygons=[{"points": [[10, 10], [20, 10], [20, 20], [10, 20]], "static": True},
                         {"points": [[15, 18], [12, 30], [18, 30]], "static": False}]),
    steps=1,
    expect_polygons=[{"pos": flat(A), "prev": flat([[10, 10], [20, 10], [20, 20], [10, 20]]),
                      "center": flat(cA)},
                     {"pos": flat(Bn), "prev": flat(Bq), "center": flat(cB2)}])

# 8. reference panics -> status codes (src/link.rs:19-21, :37-39)
cases["bad_link_a_ge_b"] = dict(scene=base(particles=[[1, 1], [2, 2]], prev=[[1, 1], [2, 2]],
                                           links=[[1, 0, 1.0, 1.0]]), steps=1, expect_status=2)
cases["bad_link_b_oob"] = dict(scene=base(particles=[[1, 1], [2, 2]], prev=[[1, 1], [2, 2]],
                                          links=[[0, 2, 1.0, 1.0]]), steps=1, expect_status=2)
cases["bad_circle_link"] = dict(
    scene=base(circles=[{"pos": [10, 10], "prev": [10, 10], "acc": [0, 0], "radius": 1.0,
                         "static": False}], circle_links=[[0, 1, 1.0]]),
    steps=1, expect_status=3)

# ---------------------------------------------------------------------------
# A whole Solver::update in float32 (src/solver.rs:106-188), written from the
# reference text for the cases below: each phase in the reference's loop
# order, every polygon edge with its pre-loop copies (src/polygon.rs:147-162).
def calc_center(pts):  # src/polygon.rs:231-237
    c = v(0, 0)
    for p in pts:
        c = c + p
    return c / f(len(pts))


def resolve(self_center, pa, pb, q, other_center):  # src/polygon.rs:164-216
    inter = line_intersection(pa, pb, q, other_center)
    if inter is None:
        return None
    nl = normalize(pb - pa)
    cp = (dot(nl, self_center - inter) / dot(nl, nl)) * nl
    ni = normalize(self_center - (inter + cp))
    da, db = norm(inter - pa), norm(inter - pb)
    dab = da + db
    ia, ib = db / dab, da / dab
    ion = (dot(ni, inter - q) / dot(ni, ni)) * ni
    dl = (ion / f(3)) * f(2)
    new_a, new_b = pa - ia * dl, pb - ib * dl
    hit = line_intersection(pa, pb, q, q - ni * f(10000))
    if hit is None:
        return None
    return new_a, new_b, hit


def solve_polygon_single(S, O, hits):  # src/polygon.rs:147-162
    n = len(S["pos"])
    for i in range(n):
        b = (i + 1) % n
        pa, pb = S["pos"][i].copy(), S["pos"][b].copy()
        for k in range(len(O["pos"])):
            r = resolve(S["center"], pa, pb, O["pos"][k], O["center"])
            if r is not None:
                S["pos"][i], S["pos"][b], O["pos"][k] = r
                hits.append((S["id"], i, O["id"], k))


def circle_bounds(p, q, r, lo, size):  # src/circle.rs:11-30
    p, q = p.copy(), q.copy()
    for ax in range(2):
        if p[ax] < lo[ax] + r:
            vel = q[ax] - p[ax]; q[ax] = lo[ax] + r - vel; p[ax] = lo[ax] + r
        elif p[ax] > lo[ax] + size[ax] - r:
            vel = q[ax] - p[ax]; q[ax] = lo[ax] + size[ax] - r - vel; p[ax] = lo[ax] + size[ax] - r
    return p, q


def world_update(W, dt, hits=None):
    """One Solver::update of a world dict: particles {pos, prev}, links
    [(a, b, rest)], circles {pos, prev, acc, r}, polygons {pos, prev, acc,
    links, static, center}."""
    hits = [] if hits is None else hits
    S = W["sub_steps"]
    delta = f(dt) * (f(1) / f(S))  # src/solver.rs:107-108
    g, lo, size = W["g"], W["lo"], W["size"]
    for _ in range(S):
        pacc = [f(0) + g for _ in W["particles"]]  # acc is zero at each update's start
        for c in W["circles"]:
            c["acc"] = c["acc"] + g
        for P in W["polygons"]:
            P["acc"] = [a + g for a in P["acc"]]
        for a_, b_, rest in W["links"]:
            A, B = W["particles"][a_], W["particles"][b_]
            A["pos"], B["pos"] = link(A["pos"], B["pos"], f(rest))
        for P in W["polygons"]:  # Polygon::solve_links, src/polygon.rs:218-223
            P["center"] = calc_center(P["pos"])
            for a_, b_, rest in P["links"]:
                P["pos"][a_], P["pos"][b_] = link(P["pos"][a_], P["pos"][b_], f(rest))
        C = W["circles"]
        for i in range(len(C)):
            for j in range(i + 1, len(C)):
                d = C[i]["pos"] - C[j]["pos"]
                d2 = f(0) + (d[0] * d[0] + d[1] * d[1])
                rs = C[i]["r"] + C[j]["r"]
                if d2 < rs * rs:
                    n = normalize(d)
                    ov = rs - np.sqrt(d2)
                    ri2, rj2 = C[i]["r"] * C[i]["r"], C[j]["r"] * C[j]["r"]
                    sc = f(1) / (ri2 + rj2)
                    C[i]["pos"] = C[i]["pos"] + ((n * sc) * ov) * rj2
                    C[j]["pos"] = C[j]["pos"] - ((n * sc) * ov) * ri2
        G = W["polygons"]
        for i in range(len(G)):
            for j in range(i + 1, len(G)):
                solve_polygon_single(G[i], G[j], hits)
                solve_polygon_single(G[j], G[i], hits)
        for P_ in W["particles"]:
            P_["pos"], P_["prev"] = bounds_step(P_["pos"], P_["prev"], lo, size)
        for c in C:
            c["pos"], c["prev"] = circle_bounds(c["pos"], c["prev"], c["r"], lo, size)
        for P in G:
            for k in range(len(P["pos"])):
                P["pos"][k], P["prev"][k] = bounds_step(P["pos"][k], P["prev"][k], lo, size)
        for P_, acc in zip(W["particles"], pacc):
            P_["pos"], P_["prev"] = integrate(P_["pos"], P_["prev"], acc, delta)
        for c in C:
            c["pos"], c["prev"] = integrate(c["pos"], c["prev"], c["acc"], delta)
            c["acc"] = v(0, 0)
        for P in G:  # Polygon::update, src/polygon.rs:125-134
            if P["static"]:
                continue
            P["center"] = calc_center(P["pos"])
            for k in range(len(P["pos"])):
                P["pos"][k], P["prev"][k] = integrate(P["pos"][k], P["prev"][k], P["acc"][k], delta)
                P["acc"][k] = v(0, 0)
    return hits


def new_world(g=(0, 0), sub_steps=1, lo=(0, 0), size=(100, 100)):
    return {"g": v(*g), "sub_steps": sub_steps, "lo": v(*lo), "size": v(*size),
            "particles": [], "links": [], "circles": [], "polygons": []}


def polygon_new(points, static, pid):  # Polygon::new, src/polygon.rs:84-123
    pos = [v(*p) for p in points]
    center = v(0, 0)
    for p in pos:
        center = center + p
    center = center / f(len(pos))
    links = []
    for i in range(len(pos)):
        a_, b_ = i, (i + 1) % len(pos)
        if a_ > b_:
            a_, b_ = b_, a_
        links.append((a_, b_, norm(pos[a_] - pos[b_])))
    return {"id": pid, "pos": pos, "prev": [p.copy() for p in pos],
            "acc": [v(0, 0) for _ in pos], "links": links, "static": static, "center": center}


def polygon_expect(P):
    return {"pos": flat(P["pos"]), "prev": flat(P["prev"]), "center": flat(P["center"])}


def circle_scene(c):
    return {"pos": flat(c["pos"]), "prev": flat(c["prev"]), "acc": flat(c["acc"]),
            "radius": float(c["r"]), "static": False}


# 9. Circle::solve_bounds insets the walls by the radius (src/circle.rs:11-30):
#    a circle moving into each of three walls, radii 2, 3 and 1.5.
W = new_world()
W["circles"] = [{"pos": v(1.5, 50), "prev": v(2.5, 50), "acc": v(0, 0), "r": f(2)},
                {"pos": v(98, 20), "prev": v(97, 20), "acc": v(0, 0), "r": f(3)},
                {"pos": v(50, 1), "prev": v(50, 1.25), "acc": v(0, 0), "r": f(1.5)}]
scene = base(circles=[circle_scene(c) for c in W["circles"]])
world_update(W, 1.0)
assert list(W["circles"][0]["pos"]) == [3, 50] and list(W["circles"][0]["prev"]) == [2, 50]
assert list(W["circles"][1]["pos"]) == [96, 20] and list(W["circles"][1]["prev"]) == [97, 20]
assert W["circles"][2]["prev"][1] == f(1.5)
cases["circle_bounds_inset"] = dict(
    scene=scene, steps=1,
    expect_circles_pos=flat([c["pos"] for c in W["circles"]]),
    expect_circles_prev=flat([c["prev"] for c in W["circles"]]))

# 10. Two vertices of one polygon cross the same edge of another: the edge's
#     end points are copied before the vertex loop, so the second hit is
#     computed from the copies and overwrites the first (src/polygon.rs:148-160).
W = new_world()
A = polygon_new([(10, 10), (20, 10), (20, 20), (10, 20)], True, 0)
B = polygon_new([(13, 18.5), (17, 18), (15, 30)], False, 1)
W["polygons"] = [A, B]
copies = (A["pos"][2].copy(), A["pos"][3].copy())
hits = world_update(W, 1.0)
edge_hits = [h for h in hits if h[0] == 0 and h[1] == 2]
assert [h[3] for h in edge_hits] == [0, 1], hits
second = resolve(calc_center([v(10, 10), v(20, 10), v(20, 20), v(10, 20)]), copies[0], copies[1],
                 v(17, 18), calc_center([v(13, 18.5), v(17, 18), v(15, 30)]))
assert np.array_equal(A["pos"][2], second[0]) and np.array_equal(A["pos"][3], second[1])
cases["polygon_two_hits_one_edge"] = dict(
    scene=base(polygons=[{"points": [[10, 10], [20, 10], [20, 20], [10, 20]], "static": True},
                         {"points": [[13, 18.5], [17, 18], [15, 30]], "static": False}]),
    steps=1, expect_polygons=[polygon_expect(A), polygon_expect(B)])

# 11. An acceleration set on a circle before it is added is consumed by the
#     first sub-step only: update clears acc (src/particle.rs:20-25) and
#     gravity is added afresh each sub-step (src/solver.rs:130-141).
W = new_world(g=(0, -2), sub_steps=2)
W["circles"] = [{"pos": v(50, 50), "prev": v(50, 50), "acc": v(3, 4), "r": f(1)}]
scene = base(gravity=[0.0, -2.0], sub_steps=2, circles=[circle_scene(W["circles"][0])])
world_update(W, 1.0)
assert list(W["circles"][0]["pos"]) == [51.5, 50.5], W["circles"][0]["pos"]
cases["circle_preset_acc_first_substep"] = dict(
    scene=scene, steps=1, expect_circles_pos=flat([W["circles"][0]["pos"]]),
    expect_circles_prev=flat([W["circles"][0]["prev"]]))

# 12. A static polygon is moved by its links (a link shorter than the edge)
#     and by a collision, but never integrated: its prev stays, its centre is
#     the one solve_links computed (src/polygon.rs:125-128, :218-223).
W = new_world(g=(0, -1))
T = polygon_new([(20, 20), (30, 20), (25, 30)], True, 0)
T["links"][0] = (0, 1, f(8))  # pulls vertices 0 and 1 together
Q = polygon_new([(24, 28), (21, 35), (28, 36)], False, 1)
W["polygons"] = [T, Q]
prev0 = [p.copy() for p in T["prev"]]
hits = world_update(W, 1.0)
assert any(0 in (h[0], h[2]) for h in hits), hits     # the static triangle takes a hit
assert all(np.array_equal(a, b) for a, b in zip(T["prev"], prev0))
assert not np.array_equal(T["pos"][0], v(20, 20))     # moved by its short link
full = lambda P: {"pos": flat(P["pos"]), "prev": flat(P["prev"]), "acc": [0.0] * (2 * len(P["pos"])),
                  "links": [[a_, b_, float(t)] for a_, b_, t in P["links"]],
                  "static": P["static"], "center": flat(P["center"])}
T0 = polygon_new([(20, 20), (30, 20), (25, 30)], True, 0)
T0["links"][0] = (0, 1, f(8))
Q0 = polygon_new([(24, 28), (21, 35), (28, 36)], False, 1)
cases["static_polygon_moved_not_integrated"] = dict(
    scene=base(gravity=[0.0, -1.0], polygons_full=[full(T0), full(Q0)]),
    steps=1, expect_polygons=[polygon_expect(T), polygon_expect(Q)])

# 13. 20 sub-steps: delta = dt * (1/20) (src/solver.rs:107-108), which is not
#     dt / 20 for this dt; a particle falling from y = 0 (the box is centred
#     on the origin) after one update, chosen so that stepping with dt / 20
#     would end on different bits.
def fall20(dt, h_of):
    W = new_world(g=(0, -9.81), sub_steps=20, lo=(-100, -100), size=(200, 200))
    W["particles"] = [{"pos": v(0, 0), "prev": v(0, 0)}]
    if h_of == "solver":
        world_update(W, dt)
    else:
        W["sub_steps"] = 1
        for _ in range(20):
            world_update(W, dt / f(20))
    return W["particles"][0]


dt20 = None
for k in range(1, 400):
    cand = f(k / 600.0)
    if cand * (f(1) / f(20)) == cand / f(20):
        continue
    a_, b_ = fall20(cand, "solver"), fall20(cand, "divided")
    if not np.array_equal(a_["pos"], b_["pos"]):
        dt20, P20 = cand, a_
        break
assert dt20 is not None
cases["substeps_20_delta"] = dict(
    scene=base(gravity=[0.0, -9.81], sub_steps=20, dt=float(dt20),
               bounds=[-100.0, -100.0, 200.0, 200.0], particles=[[0, 0]], prev=[[0, 0]]),
    steps=1, expect_pos=flat([P20["pos"]]), expect_prev=flat([P20["prev"]]))

# 14. Polygon::circle(10, (50, 50), 6, false) (src/polygon.rs:17-82): vertices
#     from f32 cos/sin of an accumulated f32 angle (the platform libm, as the
#     reference's f32::cos/sin), chords i -> i + 2n/3 and i -> i + n/3, which
#     for n = 6 solve every chord twice; one update under gravity.
import ctypes
_libm = ctypes.CDLL("libm.so.6")
for _fn in ("cosf", "sinf"):
    getattr(_libm, _fn).restype = ctypes.c_float
    getattr(_libm, _fn).argtypes = [ctypes.c_float]
n6, r6, c6 = 6, f(10), v(50, 50)
ang = f(0)
pts = []
for _ in range(n6):
    x, y = r6 * f(_libm.cosf(ang)), r6 * f(_libm.sinf(ang))
    pts.append(c6 + v(x, y))
    ang = ang + (f(2) * f(np.pi)) / f(n6)
P6 = polygon_new([tuple(p) for p in pts], False, 0)
P6["pos"] = pts
P6["prev"] = [p.copy() for p in pts]
links6 = []
for i in range(n6):
    for off in (2 * n6 // 3, n6 // 3):
        a_, b_ = i, (i + off) % n6
        if a_ > b_:
            a_, b_ = b_, a_
        links6.append((a_, b_, norm(pts[a_] - pts[b_])))
assert len(set((a_, b_) for a_, b_, _ in links6)) == 6  # every chord twice
P6["links"] = links6
W = new_world(g=(0, -1))
W["polygons"] = [P6]
world_update(W, 1.0)
cases["polygon_circle_6"] = dict(
    scene=base(gravity=[0.0, -1.0],
               polygon_circles=[{"radius": 10.0, "pos": [50.0, 50.0], "n": 6, "static": False}]),
    steps=1, expect_polygons=[polygon_expect(P6)])

OUT.write_text(json.dumps(cases, indent=1))
print(f"wrote {OUT} ({len(cases)} cases)")
