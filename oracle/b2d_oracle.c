/*
 * b2d_oracle.c — CPU oracle for the bendy2d solver step (TEST INFRASTRUCTURE).
 *
 * A plain-C restatement of Murrent/bendy2d 0.0.1, src/*.rs, op for op, in the
 * reference's array-of-structs layout and loop order.  Only the test-suite,
 * the smoke check and the benchmark's CPU-baseline leg use it, as the checker.
 * PARITY UNPINNED (no reference tests, no Rust toolchain); see b2d_oracle.h.
 *
 * Build: gcc -O2 -std=c11 -ffp-contract=off -fno-fast-math -fPIC -shared
 * (recipe in oracle/build.py).  No FMA contraction anywhere: rustc emits none.
 */
#include "b2d_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ---------------------------------------------------------------- Vector2 */
typedef struct { float x, y; } V2;
static inline V2 v2(float x, float y) { V2 r; r.x = x; r.y = y; return r; }
static inline V2 vadd(V2 a, V2 b) { return v2(a.x + b.x, a.y + b.y); }
static inline V2 vsub(V2 a, V2 b) { return v2(a.x - b.x, a.y - b.y); }
static inline V2 vmul(V2 a, float s) { return v2(a.x * s, a.y * s); }
static inline V2 vdiv(V2 a, float s) { return v2(a.x / s, a.y / s); }
static inline float vdot(V2 a, V2 b) { return a.x * b.x + a.y * b.y; }
/* nalgebra norm_squared: res = 0; res += dotc(col, col) */
static inline float vnorm_sq(V2 a) { return 0.0f + (a.x * a.x + a.y * a.y); }
static inline float vnorm(V2 a) { return sqrtf(vnorm_sq(a)); }
static inline V2 vnormalize(V2 a) { return vdiv(a, vnorm(a)); }

/* ---------------------------------------------------------------- types */
typedef struct { V2 pos, prev, acc; } Particle;            /* src/particle.rs:4-9 */
typedef struct { size_t a, b; float target, stiff; } Link;  /* src/link.rs:4-10 (+stiff ext) */
typedef struct { Particle point; float radius; int is_static; } Circle; /* src/circle.rs:4-8 */
typedef struct {                                           /* src/polygon.rs:7-14 */
  Particle* particles; size_t np;
  Link* links; size_t nl;
  int is_static; V2 center; float scale;
} Polygon;
typedef struct { V2 pos, size; } Bounds;                   /* src/solver.rs:13-17 */

struct orc_world {                                         /* src/solver.rs:19-31 */
  V2 gravity; Bounds bounds; int bounds_active;
  Particle* particles; size_t np, cap_p;
  Link* plinks; size_t npl, cap_pl;
  Circle* circles; size_t nc, cap_c;
  Link* clinks; size_t ncl, cap_cl;
  Polygon* polys; size_t npoly, cap_poly;
  uint32_t sub_steps; float sub_steps_multiplier;
  /* extensions (defaults reproduce the reference) */
  uint32_t link_iters; uint32_t collide; float radius; float cell;
};

#define GROW(ptr, n, cap, add, T)                                   \
  do {                                                              \
    if ((n) + (add) > (cap)) {                                      \
      size_t nc_ = (cap) ? (cap) : 16;                              \
      while (nc_ < (n) + (add)) nc_ *= 2;                           \
      (ptr) = (T*)realloc((ptr), nc_ * sizeof(T));                  \
      (cap) = nc_;                                                  \
    }                                                               \
  } while (0)

/* src/particle.rs:12-18 */
static Particle particle_new(V2 pos) {
  Particle p; p.pos = pos; p.prev = pos; p.acc = v2(0.0f, 0.0f); return p;
}

/* src/particle.rs:20-25: pos = pos + vel + acc*dt*dt */
static void particle_update(Particle* p, float dt) {
  V2 vel = vsub(p->pos, p->prev);
  p->prev = p->pos;
  p->pos = vadd(vadd(p->pos, vel), vmul(vmul(p->acc, dt), dt));
  p->acc = v2(0.0f, 0.0f);
}

/* src/particle.rs:27-46: per axis, min side else-if max side */
static void particle_solve_bounds(Particle* p, Bounds b) {
  if (p->pos.x < b.pos.x) {
    float vel_x = p->prev.x - p->pos.x;
    p->prev.x = b.pos.x - vel_x;
    p->pos.x = b.pos.x;
  } else if (p->pos.x > b.pos.x + b.size.x) {
    float vel_x = p->prev.x - p->pos.x;
    p->prev.x = b.pos.x + b.size.x - vel_x;
    p->pos.x = b.pos.x + b.size.x;
  }
  if (p->pos.y < b.pos.y) {
    float vel_y = p->prev.y - p->pos.y;
    p->prev.y = b.pos.y - vel_y;
    p->pos.y = b.pos.y;
  } else if (p->pos.y > b.pos.y + b.size.y) {
    float vel_y = p->prev.y - p->pos.y;
    p->prev.y = b.pos.y + b.size.y - vel_y;
    p->pos.y = b.pos.y + b.size.y;
  }
}

/* src/particle.rs:52-54 */
static void particle_add_force(Particle* p, V2 f) { p->acc = vadd(p->acc, f); }

/* src/link.rs:18-27 (ParticleLink::solve).  Extension: the correction is
 * multiplied by the link stiffness last; stiffness 1 is an exact identity. */
static void particle_link_solve(const Link* l, Particle* ps) {
  Particle* a = &ps[l->a];
  Particle* b = &ps[l->b];
  V2 dist_vec = vsub(a->pos, b->pos);
  float dist = vnorm(dist_vec);
  V2 normal = vnormalize(dist_vec);
  V2 corr = vmul(vmul(vmul(normal, dist - l->target), 0.5f), l->stiff);
  a->pos = vsub(a->pos, corr);
  b->pos = vadd(b->pos, corr);
}

/* src/link.rs:36-48 (CircleLink::solve), radius^2 weights */
static void circle_link_solve(const Link* l, Circle* cs) {
  Circle* ca = &cs[l->a];
  Circle* cb = &cs[l->b];
  V2 dist_vec = vsub(ca->point.pos, cb->point.pos);
  float dist = vnorm(dist_vec);
  V2 normal = vnormalize(dist_vec);
  float ra2 = ca->radius * ca->radius;
  float rb2 = cb->radius * cb->radius;
  float scale = 1.0f / (ra2 + rb2);
  ca->point.pos = vsub(ca->point.pos, vmul(vmul(vmul(normal, dist - l->target), scale), rb2));
  cb->point.pos = vadd(cb->point.pos, vmul(vmul(vmul(normal, dist - l->target), scale), ra2));
}

/* src/circle.rs:11-30 */
static void circle_solve_bounds(Circle* c, Bounds b) {
  Particle* p = &c->point;
  float r = c->radius;
  if (p->pos.x < b.pos.x + r) {
    float vel_x = p->prev.x - p->pos.x;
    p->prev.x = b.pos.x + r - vel_x;
    p->pos.x = b.pos.x + r;
  } else if (p->pos.x > b.pos.x + b.size.x - r) {
    float vel_x = p->prev.x - p->pos.x;
    p->prev.x = b.pos.x + b.size.x - r - vel_x;
    p->pos.x = b.pos.x + b.size.x - r;
  }
  if (p->pos.y < b.pos.y + r) {
    float vel_y = p->prev.y - p->pos.y;
    p->prev.y = b.pos.y + r - vel_y;
    p->pos.y = b.pos.y + r;
  } else if (p->pos.y > b.pos.y + b.size.y - r) {
    float vel_y = p->prev.y - p->pos.y;
    p->prev.y = b.pos.y + b.size.y - r - vel_y;
    p->pos.y = b.pos.y + b.size.y - r;
  }
}

/* src/circle.rs:32-45 */
static void circle_solve_circle(Circle* s, Circle* o) {
  V2 dist = vsub(s->point.pos, o->point.pos);
  float dist_sqr = vnorm_sq(dist);
  float radius_sum = s->radius + o->radius;
  if (dist_sqr < radius_sum * radius_sum) {
    V2 normal = vnormalize(dist);
    float overlap = radius_sum - sqrtf(dist_sqr);
    float self_rad_sqr = s->radius * s->radius;
    float circle_rad_sqr = o->radius * o->radius;
    float scale = 1.0f / (self_rad_sqr + circle_rad_sqr);
    s->point.pos = vadd(s->point.pos, vmul(vmul(vmul(normal, scale), overlap), circle_rad_sqr));
    o->point.pos = vsub(o->point.pos, vmul(vmul(vmul(normal, scale), overlap), self_rad_sqr));
  }
}

/* src/common.rs:3-26 */
static int line_intersection(V2 p1, V2 p2, V2 p3, V2 p4, V2* out) {
  float s1_x = p2.x - p1.x;
  float s1_y = p2.y - p1.y;
  float s2_x = p4.x - p3.x;
  float s2_y = p4.y - p3.y;
  float s = (-s1_y * (p1.x - p3.x) + s1_x * (p1.y - p3.y)) / (-s2_x * s1_y + s1_x * s2_y);
  float t = (s2_x * (p1.y - p3.y) - s2_y * (p1.x - p3.x)) / (-s2_x * s1_y + s1_x * s2_y);
  if (s >= 0.0f && s <= 1.0f && t >= 0.0f && t <= 1.0f) {
    out->x = p1.x + (t * s1_x);
    out->y = p1.y + (t * s1_y);
    return 1;
  }
  return 0;
}

/* src/polygon.rs:231-237 */
static void polygon_calc_center(Polygon* p) {
  V2 c = v2(0.0f, 0.0f);
  for (size_t i = 0; i < p->np; ++i) c = vadd(c, p->particles[i].pos);
  p->center = vdiv(c, (float)p->np);
}

/* src/polygon.rs:125-134 */
static void polygon_update(Polygon* p, float dt) {
  if (p->is_static) return;
  polygon_calc_center(p);
  for (size_t i = 0; i < p->np; ++i) particle_update(&p->particles[i], dt);
}

/* src/polygon.rs:164-216.  Returns 1 and the three new positions on a hit. */
static int resolve_line_intersection(const Polygon* self, V2 pa, V2 pb, V2 q, V2 other_center,
                                     V2* new_a, V2* new_b, V2* new_q) {
  V2 intersection;
  if (!line_intersection(pa, pb, q, other_center, &intersection)) return 0;
  V2 normal_line = vnormalize(vsub(pb, pa));
  V2 center_proj = vmul(normal_line, vdot(normal_line, vsub(self->center, intersection)) /
                                         vdot(normal_line, normal_line));
  V2 normal_in = vnormalize(vsub(self->center, vadd(intersection, center_proj)));
  float dist_to_a = vnorm(vsub(intersection, pa));
  float dist_to_b = vnorm(vsub(intersection, pb));
  float dist_a_to_b = dist_to_a + dist_to_b;
  float influence_a = dist_to_b / dist_a_to_b;
  float influence_b = dist_to_a / dist_a_to_b;
  V2 diff_int_to_point = vsub(intersection, q);
  V2 intersection_on_normal =
      vmul(normal_in, vdot(normal_in, diff_int_to_point) / vdot(normal_in, normal_in));
  V2 displace_third = vdiv(intersection_on_normal, 3.0f);
  V2 displace_line = vmul(displace_third, 2.0f);
  V2 displacement_a = vmul(displace_line, influence_a);
  V2 displacement_b = vmul(displace_line, influence_b);
  V2 na = vsub(pa, displacement_a);
  V2 nb = vsub(pb, displacement_b);
  V2 hit;
  if (line_intersection(pa, pb, q, vsub(q, vmul(normal_in, 10000.0f)), &hit)) {
    *new_a = na; *new_b = nb; *new_q = hit;
    return 1;
  }
  return 0;
}

/* src/polygon.rs:147-162: point_a/point_b are copies taken before the inner
 * loop, so later hits on the same edge overwrite earlier ones. */
static void polygon_solve_single(Polygon* self, Polygon* other) {
  size_t n = self->np;
  for (size_t i = 0; i < n; ++i) {
    V2 pa = self->particles[i].pos;
    size_t b_id = (i + 1) % n;
    V2 pb = self->particles[b_id].pos;
    for (size_t k = 0; k < other->np; ++k) {
      V2 na, nb, nq;
      if (resolve_line_intersection(self, pa, pb, other->particles[k].pos, other->center,
                                    &na, &nb, &nq)) {
        self->particles[i].pos = na;
        self->particles[b_id].pos = nb;
        other->particles[k].pos = nq;
      }
    }
  }
}

/* src/polygon.rs:142-145 */
static void polygon_solve_polygon(Polygon* a, Polygon* b) {
  polygon_solve_single(a, b);
  polygon_solve_single(b, a);
}

/* src/polygon.rs:218-223 */
static void polygon_solve_links(Polygon* p) {
  polygon_calc_center(p);
  for (size_t i = 0; i < p->nl; ++i) particle_link_solve(&p->links[i], p->particles);
}

/* ------------------------------------------------ extension collisions
 * Not in the reference (it has no particle radius and no broadphase,
 * src/solver.rs:167-188).  The spec below is this project's own; the CUDA
 * path implements the same rules in the same summation order.
 */
static int32_t cell_coord(float p, float origin, float cell) {
  float v = floorf((p - origin) / cell);
  if (!(v > -1.0e9f)) v = -1.0e9f;
  if (v > 1.0e9f) v = 1.0e9f;
  return (int32_t)v;
}

typedef struct { int32_t cy, cx; uint32_t idx; } CellEnt;
static int cellent_cmp(const void* x, const void* y) {
  const CellEnt* a = (const CellEnt*)x;
  const CellEnt* b = (const CellEnt*)y;
  if (a->cy != b->cy) return a->cy < b->cy ? -1 : 1;
  if (a->cx != b->cx) return a->cx < b->cx ? -1 : 1;
  return a->idx < b->idx ? -1 : (a->idx > b->idx);
}
static size_t cell_lower(const CellEnt* e, size_t n, int32_t cy, int32_t cx) {
  size_t lo = 0, hi = n;
  while (lo < hi) {
    size_t mid = (lo + hi) / 2;
    if (e[mid].cy < cy || (e[mid].cy == cy && e[mid].cx < cx)) lo = mid + 1; else hi = mid;
  }
  return lo;
}

/* particle-particle: Jacobi over the pre-collision snapshot.  For particle
 * i, every other particle j whose cell is one of the 9 cells around i's cell
 * is a candidate; contact when 0 < |d|^2 < (2r)^2, d = p_i - p_j:
 *   corr = ((d/|d|) * (2r - |d|)) * 0.5
 * The corrections are summed in 64-bit fixed point (units of 2^-32, each
 * component rounded to nearest-even), so the sum does not depend on the order
 * neighbours are visited in; then pos = pos + (float)(sum * 2^-32). */
static int64_t fix32(float c) { return llrintf(c * 4294967296.0f); }
static float unfix32(int64_t s) { return (float)((double)s * 0x1p-32); }

static void ext_collide_pp(orc_world* w) {
  size_t n = w->np;
  if (n == 0) return;
  V2* snap = (V2*)malloc(n * sizeof(V2));
  CellEnt* ent = (CellEnt*)malloc(n * sizeof(CellEnt));
  for (size_t i = 0; i < n; ++i) {
    snap[i] = w->particles[i].pos;
    ent[i].cx = cell_coord(snap[i].x, w->bounds.pos.x, w->cell);
    ent[i].cy = cell_coord(snap[i].y, w->bounds.pos.y, w->cell);
    ent[i].idx = (uint32_t)i;
  }
  CellEnt* sorted = (CellEnt*)malloc(n * sizeof(CellEnt));
  memcpy(sorted, ent, n * sizeof(CellEnt));
  qsort(sorted, n, sizeof(CellEnt), cellent_cmp);
  float D = w->radius + w->radius;
  float D2 = D * D;
  for (size_t i = 0; i < n; ++i) {
    V2 p = snap[i];
    int64_t sx = 0, sy = 0;
    int hit = 0;
    for (int dy = -1; dy <= 1; ++dy) {
      for (int dx = -1; dx <= 1; ++dx) {
        int32_t cy = ent[i].cy + dy, cx = ent[i].cx + dx;
        size_t k = cell_lower(sorted, n, cy, cx);
        for (; k < n && sorted[k].cy == cy && sorted[k].cx == cx; ++k) {
          uint32_t j = sorted[k].idx;
          if (j == i) continue;
          V2 d = vsub(p, snap[j]);
          float d2 = d.x * d.x + d.y * d.y;
          if (d2 < D2 && d2 > 0.0f) {
            float dist = sqrtf(d2);
            V2 nrm = vdiv(d, dist);
            V2 corr = vmul(vmul(nrm, D - dist), 0.5f);
            sx += fix32(corr.x);
            sy += fix32(corr.y);
            hit = 1;
          }
        }
      }
    }
    if (hit) w->particles[i].pos = vadd(p, v2(unfix32(sx), unfix32(sy)));
  }
  free(snap); free(ent); free(sorted);
}

/* particle-Circle: circles are kinematic for particles (one-way).  Circles are
 * visited in index order; contact when |d|^2 < (r+R)^2 and |d|^2 > 0:
 *   pos = pos + (d/|d|) * ((r+R) - |d|) */
static V2 ext_particle_circles(const orc_world* w, V2 p) {
  for (size_t k = 0; k < w->nc; ++k) {
    V2 d = vsub(p, w->circles[k].point.pos);
    float d2 = d.x * d.x + d.y * d.y;
    float R = w->radius + w->circles[k].radius;
    if (d2 < R * R && d2 > 0.0f) {
      float dist = sqrtf(d2);
      V2 nrm = vdiv(d, dist);
      p = vadd(p, vmul(nrm, R - dist));
    }
  }
  return p;
}

/* particle-Polygon edge projection (one-way).  For each polygon with >= 3
 * vertices, in index order, skipped when p lies outside the vertex bounding
 * box grown by r:
 *   inside  = crossing-number test over edges (v[e], v[e+1 mod n]);
 *   q       = closest point over edges, t = clamp(dot(p-a,ab)/dot(ab,ab),0,1),
 *             first minimum of |p-q|^2 wins;
 *   inside          -> pos = q + ((q-p)/|q-p|) * r   (pos = q if |q-p| = 0)
 *   outside, d < r  -> pos = q + ((p-q)/|p-q|) * r                        */
static V2 ext_particle_polygon(const Polygon* poly, float r, V2 p) {
  size_t n = poly->np;
  if (n < 3) return p;
  const Particle* v = poly->particles;
  float minx = v[0].pos.x, maxx = v[0].pos.x, miny = v[0].pos.y, maxy = v[0].pos.y;
  for (size_t e = 1; e < n; ++e) {
    if (v[e].pos.x < minx) minx = v[e].pos.x;
    if (v[e].pos.x > maxx) maxx = v[e].pos.x;
    if (v[e].pos.y < miny) miny = v[e].pos.y;
    if (v[e].pos.y > maxy) maxy = v[e].pos.y;
  }
  if (!(p.x >= minx - r && p.x <= maxx + r && p.y >= miny - r && p.y <= maxy + r)) return p;
  int inside = 0;
  float best = INFINITY;
  V2 bq = p;
  for (size_t e = 0; e < n; ++e) {
    V2 a = v[e].pos, b = v[(e + 1) % n].pos;
    if ((a.y > p.y) != (b.y > p.y)) {
      float t = (p.y - a.y) / (b.y - a.y);
      float xint = a.x + t * (b.x - a.x);
      if (p.x < xint) inside = !inside;
    }
    V2 ab = vsub(b, a);
    float l2 = ab.x * ab.x + ab.y * ab.y;
    float t = 0.0f;
    if (l2 > 0.0f) t = ((p.x - a.x) * ab.x + (p.y - a.y) * ab.y) / l2;
    t = fminf(fmaxf(t, 0.0f), 1.0f);
    V2 q = vadd(a, vmul(ab, t));
    V2 dq = vsub(p, q);
    float d2 = dq.x * dq.x + dq.y * dq.y;
    if (d2 < best) { best = d2; bq = q; }
  }
  if (inside) {
    float dist = sqrtf(best);
    if (dist > 0.0f) {
      V2 nrm = vdiv(vsub(bq, p), dist);
      return vadd(bq, vmul(nrm, r));
    }
    return bq;
  }
  if (best < r * r) {
    float dist = sqrtf(best);
    if (dist > 0.0f) {
      V2 nrm = vdiv(vsub(p, bq), dist);
      return vadd(bq, vmul(nrm, r));
    }
  }
  return p;
}

/* ---------------------------------------------------------------- solver */
orc_world* orc_new(void) {                                  /* src/solver.rs:34-50 */
  orc_world* w = (orc_world*)calloc(1, sizeof(orc_world));
  w->gravity = v2(0.0f, 98.2f);
  w->bounds.pos = v2(0.0f, 0.0f);
  w->bounds.size = v2(100.0f, 100.0f);
  w->bounds_active = 1;
  w->sub_steps = 1;
  w->sub_steps_multiplier = 0.0f;
  w->link_iters = 1;
  w->collide = 0;
  w->radius = 0.5f;
  w->cell = 1.0f;
  return w;
}

static void polygon_free(Polygon* p) { free(p->particles); free(p->links); }

void orc_free(orc_world* w) {
  if (!w) return;
  free(w->particles); free(w->plinks); free(w->circles); free(w->clinks);
  for (size_t i = 0; i < w->npoly; ++i) polygon_free(&w->polys[i]);
  free(w->polys);
  free(w);
}

static void* dup(const void* src, size_t bytes) {
  if (!bytes) return NULL;
  void* d = malloc(bytes);
  memcpy(d, src, bytes);
  return d;
}

orc_world* orc_clone(const orc_world* w) {
  orc_world* c = (orc_world*)malloc(sizeof(orc_world));
  *c = *w;
  c->particles = (Particle*)dup(w->particles, w->np * sizeof(Particle)); c->cap_p = w->np;
  c->plinks = (Link*)dup(w->plinks, w->npl * sizeof(Link)); c->cap_pl = w->npl;
  c->circles = (Circle*)dup(w->circles, w->nc * sizeof(Circle)); c->cap_c = w->nc;
  c->clinks = (Link*)dup(w->clinks, w->ncl * sizeof(Link)); c->cap_cl = w->ncl;
  c->polys = (Polygon*)dup(w->polys, w->npoly * sizeof(Polygon)); c->cap_poly = w->npoly;
  for (size_t i = 0; i < w->npoly; ++i) {
    c->polys[i].particles = (Particle*)dup(w->polys[i].particles, w->polys[i].np * sizeof(Particle));
    c->polys[i].links = (Link*)dup(w->polys[i].links, w->polys[i].nl * sizeof(Link));
  }
  return c;
}

void orc_set_gravity(orc_world* w, float x, float y) { w->gravity = v2(x, y); }
void orc_set_bounds(orc_world* w, float px, float py, float sx, float sy) {
  w->bounds.pos = v2(px, py); w->bounds.size = v2(sx, sy);
}
void orc_set_sub_steps(orc_world* w, uint32_t n) { w->sub_steps = n; }
void orc_set_link_iters(orc_world* w, uint32_t n) { w->link_iters = n; }
void orc_set_collide(orc_world* w, uint32_t flags, float r, float cell) {
  w->collide = flags; w->radius = r; w->cell = cell;
}

void orc_add_particles(orc_world* w, size_t n, const float* pos, const float* prev) {
  GROW(w->particles, w->np, w->cap_p, n, Particle);
  for (size_t i = 0; i < n; ++i) {
    Particle p = particle_new(v2(pos[2 * i], pos[2 * i + 1]));
    if (prev) p.prev = v2(prev[2 * i], prev[2 * i + 1]);
    w->particles[w->np++] = p;
  }
}

void orc_add_particle_links(orc_world* w, size_t n, const uint64_t* a, const uint64_t* b,
                            const float* target, const float* stiff) {
  GROW(w->plinks, w->npl, w->cap_pl, n, Link);
  for (size_t i = 0; i < n; ++i) {
    Link l; l.a = (size_t)a[i]; l.b = (size_t)b[i]; l.target = target[i];
    l.stiff = stiff ? stiff[i] : 1.0f;
    w->plinks[w->npl++] = l;
  }
}

void orc_add_circle(orc_world* w, const float* pos, const float* prev, const float* acc,
                    float radius, int is_static) {
  GROW(w->circles, w->nc, w->cap_c, 1, Circle);
  Circle c;
  c.point = particle_new(v2(pos[0], pos[1]));
  if (prev) c.point.prev = v2(prev[0], prev[1]);
  if (acc) c.point.acc = v2(acc[0], acc[1]);
  c.radius = radius;
  c.is_static = is_static;
  w->circles[w->nc++] = c;
}

void orc_add_circle_link(orc_world* w, uint64_t a, uint64_t b, float target) {
  GROW(w->clinks, w->ncl, w->cap_cl, 1, Link);
  Link l; l.a = (size_t)a; l.b = (size_t)b; l.target = target; l.stiff = 1.0f;
  w->clinks[w->ncl++] = l;
}

void orc_add_polygon(orc_world* w, size_t nv, const float* pos, const float* prev,
                     const float* acc, size_t nl, const uint64_t* la, const uint64_t* lb,
                     const float* lt, int is_static, float cx, float cy, float scale) {
  GROW(w->polys, w->npoly, w->cap_poly, 1, Polygon);
  Polygon p;
  p.np = nv;
  p.particles = (Particle*)malloc((nv ? nv : 1) * sizeof(Particle));
  for (size_t i = 0; i < nv; ++i) {
    p.particles[i] = particle_new(v2(pos[2 * i], pos[2 * i + 1]));
    if (prev) p.particles[i].prev = v2(prev[2 * i], prev[2 * i + 1]);
    if (acc) p.particles[i].acc = v2(acc[2 * i], acc[2 * i + 1]);
  }
  p.nl = nl;
  p.links = (Link*)malloc((nl ? nl : 1) * sizeof(Link));
  for (size_t i = 0; i < nl; ++i) {
    p.links[i].a = (size_t)la[i]; p.links[i].b = (size_t)lb[i];
    p.links[i].target = lt[i]; p.links[i].stiff = 1.0f;
  }
  p.is_static = is_static; p.center = v2(cx, cy); p.scale = scale;
  w->polys[w->npoly++] = p;
}

/* Polygon::circle, src/polygon.rs:17-82: chords i -> i+2n/3 and i -> i+n/3,
 * ids swapped so a < b, target = initial distance. */
void orc_add_polygon_circle(orc_world* w, float radius, float x, float y, size_t n,
                            int is_static) {
  float* pos = (float*)malloc((2 * n + 2) * sizeof(float));
  V2 center = v2(0.0f, 0.0f);
  float angle = 0.0f;
  for (size_t i = 0; i < n; ++i) {
    float px = radius * cosf(angle);
    float py = radius * sinf(angle);
    V2 pt = vadd(v2(x, y), v2(px, py));
    pos[2 * i] = pt.x; pos[2 * i + 1] = pt.y;
    center = vadd(center, pt);
    angle += 2.0f * 3.14159265358979323846f / (float)n;
  }
  center = vdiv(center, (float)n);
  uint64_t* la = (uint64_t*)malloc((2 * n + 1) * sizeof(uint64_t));
  uint64_t* lb = (uint64_t*)malloc((2 * n + 1) * sizeof(uint64_t));
  float* lt = (float*)malloc((2 * n + 1) * sizeof(float));
  size_t nl = 0;
  for (size_t i = 0; i < n; ++i) {
    size_t offs[2] = {2 * n / 3, n / 3};
    for (int k = 0; k < 2; ++k) {
      size_t a = i, b = (i + offs[k]) % n;
      if (a > b) { size_t t = a; a = b; b = t; }
      V2 d = vsub(v2(pos[2 * a], pos[2 * a + 1]), v2(pos[2 * b], pos[2 * b + 1]));
      la[nl] = a; lb[nl] = b; lt[nl] = vnorm(d); ++nl;
    }
  }
  orc_add_polygon(w, n, pos, NULL, NULL, nl, la, lb, lt, is_static, center.x, center.y, 1.0f);
  free(pos); free(la); free(lb); free(lt);
}

/* Polygon::new, src/polygon.rs:84-123: perimeter links i -> (i+1) mod n */
void orc_add_polygon_points(orc_world* w, size_t n, const float* pts, int is_static) {
  V2 center = v2(0.0f, 0.0f);
  for (size_t i = 0; i < n; ++i) center = vadd(center, v2(pts[2 * i], pts[2 * i + 1]));
  center = vdiv(center, (float)n);
  uint64_t* la = (uint64_t*)malloc((n + 1) * sizeof(uint64_t));
  uint64_t* lb = (uint64_t*)malloc((n + 1) * sizeof(uint64_t));
  float* lt = (float*)malloc((n + 1) * sizeof(float));
  for (size_t i = 0; i < n; ++i) {
    size_t a = i, b = (i + 1) % n;
    if (a > b) { size_t t = a; a = b; b = t; }
    V2 d = vsub(v2(pts[2 * a], pts[2 * a + 1]), v2(pts[2 * b], pts[2 * b + 1]));
    la[i] = a; lb[i] = b; lt[i] = vnorm(d);
  }
  orc_add_polygon(w, n, pts, NULL, NULL, n, la, lb, lt, is_static, center.x, center.y, 1.0f);
  free(la); free(lb); free(lt);
}

/* The reference panics inside update on a bad link (split_at_mut(b) needs
 * b <= len, split.1[0] needs b < len, split.0[a] needs a < b,
 * src/link.rs:19-21, :37-39).  The oracle reports it before touching state. */
static int validate(const orc_world* w) {
  for (size_t i = 0; i < w->npl; ++i)
    if (!(w->plinks[i].a < w->plinks[i].b && w->plinks[i].b < w->np)) return ORC_ERR_LINK_INDEX;
  for (size_t i = 0; i < w->ncl; ++i)
    if (!(w->clinks[i].a < w->clinks[i].b && w->clinks[i].b < w->nc))
      return ORC_ERR_CIRCLE_LINK_INDEX;
  for (size_t p = 0; p < w->npoly; ++p)
    for (size_t i = 0; i < w->polys[p].nl; ++i)
      if (!(w->polys[p].links[i].a < w->polys[p].links[i].b &&
            w->polys[p].links[i].b < w->polys[p].np))
        return ORC_ERR_POLY_LINK_INDEX;
  return ORC_OK;
}

/* src/solver.rs:130-141 */
static void apply_gravity(orc_world* w) {
  V2 g = w->gravity;
  for (size_t i = 0; i < w->np; ++i) particle_add_force(&w->particles[i], g);
  for (size_t i = 0; i < w->nc; ++i) particle_add_force(&w->circles[i].point, g);
  for (size_t p = 0; p < w->npoly; ++p)                  /* src/polygon.rs:225-229 */
    for (size_t i = 0; i < w->polys[p].np; ++i) particle_add_force(&w->polys[p].particles[i], g);
}

/* src/solver.rs:143-153 */
static void apply_links(orc_world* w) {
  for (size_t i = 0; i < w->npl; ++i) particle_link_solve(&w->plinks[i], w->particles);
  for (size_t i = 0; i < w->ncl; ++i) circle_link_solve(&w->clinks[i], w->circles);
  for (size_t p = 0; p < w->npoly; ++p) polygon_solve_links(&w->polys[p]);
}

/* src/solver.rs:167-188 (+ extension particle collisions after polygons) */
static void solve_dynamic_collisions(orc_world* w) {
  for (size_t i = 0; i < w->nc; ++i)
    for (size_t j = i + 1; j < w->nc; ++j) circle_solve_circle(&w->circles[i], &w->circles[j]);
  for (size_t i = 0; i < w->npoly; ++i)
    for (size_t j = i + 1; j < w->npoly; ++j) polygon_solve_polygon(&w->polys[i], &w->polys[j]);
  if (w->collide & ORC_COLLIDE_PP) ext_collide_pp(w);
  if (w->collide & (ORC_COLLIDE_PC | ORC_COLLIDE_PPOLY)) {
    for (size_t i = 0; i < w->np; ++i) {
      V2 p = w->particles[i].pos;
      if (w->collide & ORC_COLLIDE_PC) p = ext_particle_circles(w, p);
      if (w->collide & ORC_COLLIDE_PPOLY)
        for (size_t k = 0; k < w->npoly; ++k) p = ext_particle_polygon(&w->polys[k], w->radius, p);
      w->particles[i].pos = p;
    }
  }
}

/* src/solver.rs:155-165 (bounds_active is never read, src/solver.rs:23) */
static void solve_boundary_collisions(orc_world* w) {
  for (size_t i = 0; i < w->np; ++i) particle_solve_bounds(&w->particles[i], w->bounds);
  for (size_t i = 0; i < w->nc; ++i) circle_solve_bounds(&w->circles[i], w->bounds);
  for (size_t p = 0; p < w->npoly; ++p)                  /* src/polygon.rs:136-140 */
    for (size_t i = 0; i < w->polys[p].np; ++i)
      particle_solve_bounds(&w->polys[p].particles[i], w->bounds);
}

/* src/solver.rs:118-128.  Extension: a static circle is not integrated (its
 * acceleration keeps accumulating, like a static polygon's). */
static void update_positions(orc_world* w, float dt) {
  for (size_t i = 0; i < w->np; ++i) particle_update(&w->particles[i], dt);
  for (size_t i = 0; i < w->nc; ++i)
    if (!w->circles[i].is_static) particle_update(&w->circles[i].point, dt);
  for (size_t p = 0; p < w->npoly; ++p) polygon_update(&w->polys[p], dt);
}

/* src/solver.rs:106-116.  Extension: apply_links is repeated link_iters times. */
int orc_update(orc_world* w, float dt) {
  int st = validate(w);
  if (st != ORC_OK) return st;
  w->sub_steps_multiplier = 1.0f / (float)w->sub_steps;
  float delta = dt * w->sub_steps_multiplier;
  for (uint32_t s = 0; s < w->sub_steps; ++s) {
    apply_gravity(w);
    for (uint32_t k = 0; k < w->link_iters; ++k) apply_links(w);
    solve_dynamic_collisions(w);
    solve_boundary_collisions(w);
    update_positions(w, delta);
  }
  return ORC_OK;
}

size_t orc_particle_len(const orc_world* w) { return w->np; }
size_t orc_circle_len(const orc_world* w) { return w->nc; }
size_t orc_polygon_len(const orc_world* w) { return w->npoly; }
size_t orc_polygon_vertex_len(const orc_world* w, size_t i) { return w->polys[i].np; }
size_t orc_polygon_link_len(const orc_world* w, size_t i) { return w->polys[i].nl; }

void orc_read_particles(const orc_world* w, float* pos, float* prev) {
  for (size_t i = 0; i < w->np; ++i) {
    if (pos) { pos[2 * i] = w->particles[i].pos.x; pos[2 * i + 1] = w->particles[i].pos.y; }
    if (prev) { prev[2 * i] = w->particles[i].prev.x; prev[2 * i + 1] = w->particles[i].prev.y; }
  }
}
void orc_read_circles(const orc_world* w, float* pos, float* prev) {
  for (size_t i = 0; i < w->nc; ++i) {
    if (pos) { pos[2 * i] = w->circles[i].point.pos.x; pos[2 * i + 1] = w->circles[i].point.pos.y; }
    if (prev) { prev[2 * i] = w->circles[i].point.prev.x; prev[2 * i + 1] = w->circles[i].point.prev.y; }
  }
}
void orc_read_polygon(const orc_world* w, size_t k, float* pos, float* prev, float* center) {
  const Polygon* p = &w->polys[k];
  for (size_t i = 0; i < p->np; ++i) {
    if (pos) { pos[2 * i] = p->particles[i].pos.x; pos[2 * i + 1] = p->particles[i].pos.y; }
    if (prev) { prev[2 * i] = p->particles[i].prev.x; prev[2 * i + 1] = p->particles[i].prev.y; }
  }
  if (center) { center[0] = p->center.x; center[1] = p->center.y; }
}
void orc_read_polygon_links(const orc_world* w, size_t k, uint64_t* a, uint64_t* b, float* t) {
  const Polygon* p = &w->polys[k];
  for (size_t i = 0; i < p->nl; ++i) { a[i] = p->links[i].a; b[i] = p->links[i].b; t[i] = p->links[i].target; }
}

double orc_link_residual(const orc_world* w) {
  double worst = 0.0;
  for (size_t i = 0; i < w->npl; ++i) {
    const Link* l = &w->plinks[i];
    double dx = (double)w->particles[l->a].pos.x - w->particles[l->b].pos.x;
    double dy = (double)w->particles[l->a].pos.y - w->particles[l->b].pos.y;
    double len = sqrt(dx * dx + dy * dy);
    double r = fabs(len - l->target) / (l->target > 0 ? l->target : 1.0);
    if (r > worst) worst = r;
  }
  return worst;
}
