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

OUT.write_text(json.dumps(cases, indent=1))
print(f"wrote {OUT} ({len(cases)} cases)")
