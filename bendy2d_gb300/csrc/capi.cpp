// capi.cpp — the extern "C" boundary declared in include/bendy2d.h.
//
// A b2d_solver keeps a host mirror of the reference's Solver (WorldHost) and
// places the world in an Engine (its own, or a batch's) on the first update.
// Device state is authoritative between updates; getters copy it back.
#include <cuda_runtime_api.h>

#include <algorithm>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/bendy2d.h"
#include "engine.hpp"
#include "server.hpp"

using namespace b2d;

static thread_local std::string g_err;

static int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

namespace b2d {
void set_last_error(const std::string& msg) { g_err = msg; }
}  // namespace b2d

struct b2d_solver {
  WorldHost w;
  std::unique_ptr<Engine> own;
  Engine* eng = nullptr;
  b2d_batch* batch = nullptr;
  uint32_t slot = 0;
  bool placed = false;
  bool topo_dirty = true;
  bool params_dirty = false;
  bool host_stale = false;
  cudaStream_t stream = nullptr;
  bool graphs = true;
  bool profiling = false;
  PlanTuning tune;
  bool tune_set = false;
};

struct b2d_server {
  std::unique_ptr<Server> sv;
  std::vector<uint64_t> pending;  // finished ids not yet handed out
};

struct b2d_batch {
  std::recursive_mutex mu;  // every b2d_batch_* call holds it
  std::unique_ptr<Engine> eng;
  std::vector<b2d_solver*> members;
  cudaStream_t stream = nullptr;
  bool profiling = false;
  bool plain = false;
  PlanTuning tune;
  bool tune_set = false;
};

static int have_gpu() {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return 0;
  return 1;
}

static int engine_for(b2d_solver* s, Engine** out) {
  if (s->batch) {
    if (!s->batch->eng) {
      if (!have_gpu()) return fail(ERR_CUDA, "no CUDA device: bendy2d-gb300 has no CPU path");
      s->batch->eng = std::make_unique<Engine>(s->batch->stream);
      s->batch->eng->set_plain(s->batch->plain);
      if (s->batch->tune_set) s->batch->eng->set_tuning(s->batch->tune);
    }
    *out = s->batch->eng.get();
    return OK;
  }
  if (!s->own) {
    if (!have_gpu()) return fail(ERR_CUDA, "no CUDA device: bendy2d-gb300 has no CPU path");
    s->own = std::make_unique<Engine>(s->stream);
    s->own->set_use_graph(s->graphs);
    s->own->set_profile(s->profiling);
    if (s->tune_set) s->own->set_tuning(s->tune);
  }
  *out = s->own.get();
  return OK;
}

static int sync_host(b2d_solver* s) {
  if (s->host_stale && s->placed) {
    int st = s->eng->download(s->slot);
    if (st != OK) return fail(st, s->eng->last_error);
  }
  s->host_stale = false;
  return OK;
}

static int unplace(b2d_solver* s) {
  int st = sync_host(s);
  if (st != OK) return st;
  if (s->placed) {
    st = s->eng->remove(s->slot);
    if (st != OK) return fail(st, s->eng->last_error);
  }
  s->placed = false;
  s->topo_dirty = true;
  return OK;
}

static int ensure_placed(b2d_solver* s) {
  Engine* e = nullptr;
  int st = engine_for(s, &e);
  if (st != OK) return st;
  if (s->placed && s->eng != e) {
    st = unplace(s);
    if (st != OK) return st;
  }
  if (s->topo_dirty || !s->placed) {
    st = sync_host(s);
    if (st != OK) return st;
    if (s->placed) {
      st = s->eng->remove(s->slot);
      if (st != OK) return fail(st, s->eng->last_error);
      s->placed = false;
    }
    std::string why;
    st = e->add(&s->w, &s->slot, &why);
    if (st != OK) return fail(st, why.empty() ? e->last_error : why);
    s->eng = e;
    s->placed = true;
    s->topo_dirty = false;
    s->params_dirty = false;
  } else if (s->params_dirty) {
    st = e->set_params(s->slot);
    if (st != OK) return fail(st, e->last_error);
    s->params_dirty = false;
  }
  return OK;
}

#define CHECK_S(s) \
  if (!(s)) return fail(ERR_NULL, "null solver")
#define MUTATE(s)                        \
  do {                                   \
    int st_ = sync_host(s);              \
    if (st_ != OK) return st_;           \
    (s)->topo_dirty = true;              \
  } while (0)

extern "C" {

const char* b2d_last_error(void) { return g_err.c_str(); }
const char* b2d_version(void) { return "bendy2d-gb300 0.1.0 (reference: bendy2d 0.0.1)"; }

int b2d_solver_create(b2d_solver** out) {
  if (!out) return fail(ERR_NULL, "null out");
  *out = new b2d_solver();
  return OK;
}

int b2d_batch_remove(b2d_batch* b, b2d_solver* s);

int b2d_solver_destroy(b2d_solver* s) {
  if (!s) return OK;
  if (s->batch) b2d_batch_remove(s->batch, s);
  if (s->placed && s->eng) s->eng->remove(s->slot);
  delete s;
  return OK;
}

int b2d_solver_clone(b2d_solver* s, b2d_solver** out) {
  CHECK_S(s);
  if (!out) return fail(ERR_NULL, "null out");
  int st = sync_host(s);
  if (st != OK) return st;
  b2d_solver* c = new b2d_solver();
  c->w = s->w;
  c->graphs = s->graphs;
  *out = c;
  return OK;
}

int b2d_set_gravity(b2d_solver* s, float x, float y) {
  CHECK_S(s);
  s->w.gravity = Vec2{x, y};
  s->params_dirty = true;
  return OK;
}
int b2d_get_gravity(b2d_solver* s, b2d_vec2* out) {
  CHECK_S(s);
  out->x = s->w.gravity.x;
  out->y = s->w.gravity.y;
  return OK;
}
int b2d_set_bounds(b2d_solver* s, float px, float py, float sx, float sy) {
  CHECK_S(s);
  s->w.bounds = Bounds{{px, py}, {sx, sy}};
  s->params_dirty = true;
  return OK;
}
int b2d_get_bounds(b2d_solver* s, b2d_vec2* pos, b2d_vec2* size) {
  CHECK_S(s);
  if (pos) { pos->x = s->w.bounds.pos.x; pos->y = s->w.bounds.pos.y; }
  if (size) { size->x = s->w.bounds.size.x; size->y = s->w.bounds.size.y; }
  return OK;
}
int b2d_set_bounds_active(b2d_solver* s, int a) {
  CHECK_S(s);
  s->w.bounds_active = a != 0;
  return OK;
}
int b2d_get_bounds_active(b2d_solver* s, int* out) {
  CHECK_S(s);
  *out = s->w.bounds_active ? 1 : 0;
  return OK;
}

int b2d_add_particle(b2d_solver* s, float x, float y) {
  CHECK_S(s);
  MUTATE(s);
  s->w.particles.push_back(Particle{{x, y}, {x, y}, {0.0f, 0.0f}});
  return OK;
}
int b2d_add_particle_prev(b2d_solver* s, float x, float y, float px, float py) {
  CHECK_S(s);
  MUTATE(s);
  s->w.particles.push_back(Particle{{x, y}, {px, py}, {0.0f, 0.0f}});
  return OK;
}
int b2d_add_particles(b2d_solver* s, size_t n, const float* pos, const float* prev) {
  CHECK_S(s);
  if (n && !pos) return fail(ERR_NULL, "null positions");
  MUTATE(s);
  s->w.particles.reserve(s->w.particles.size() + n);
  for (size_t i = 0; i < n; ++i) {
    Vec2 p{pos[2 * i], pos[2 * i + 1]};
    Vec2 q = prev ? Vec2{prev[2 * i], prev[2 * i + 1]} : p;
    s->w.particles.push_back(Particle{p, q, {0.0f, 0.0f}});
  }
  return OK;
}
int b2d_add_particle_link(b2d_solver* s, uint64_t a, uint64_t b, float t) {
  CHECK_S(s);
  MUTATE(s);
  s->w.particle_links.push_back(Link{a, b, t, 1.0f});
  return OK;
}
int b2d_add_particle_links(b2d_solver* s, size_t n, const uint64_t* a, const uint64_t* b,
                           const float* t, const float* k) {
  CHECK_S(s);
  if (n && (!a || !b || !t)) return fail(ERR_NULL, "null link arrays");
  MUTATE(s);
  s->w.particle_links.reserve(s->w.particle_links.size() + n);
  for (size_t i = 0; i < n; ++i) s->w.particle_links.push_back(Link{a[i], b[i], t[i], k ? k[i] : 1.0f});
  return OK;
}
int b2d_add_circle(b2d_solver* s, const b2d_circle* c) {
  CHECK_S(s);
  if (!c) return fail(ERR_NULL, "null circle");
  MUTATE(s);
  Circle cc;
  std::memcpy(&cc.point, &c->point, sizeof(Particle));
  cc.radius = c->radius;
  cc.is_static = c->is_static;
  s->w.circles.push_back(cc);
  return OK;
}
int b2d_add_circle_link(b2d_solver* s, uint64_t a, uint64_t b, float t) {
  CHECK_S(s);
  MUTATE(s);
  s->w.circle_links.push_back(Link{a, b, t, 1.0f});
  return OK;
}
int b2d_add_polygon(b2d_solver* s, size_t nv, const b2d_particle* v, size_t nl,
                    const b2d_link* l, int is_static, b2d_vec2 center, float scale) {
  CHECK_S(s);
  if ((nv && !v) || (nl && !l)) return fail(ERR_NULL, "null polygon arrays");
  MUTATE(s);
  Polygon p;
  p.particles.resize(nv);
  if (nv) std::memcpy(p.particles.data(), v, nv * sizeof(Particle));
  for (size_t i = 0; i < nl; ++i)
    p.particle_links.push_back(Link{l[i].particle_a, l[i].particle_b, l[i].target_distance, 1.0f});
  p.is_static = is_static != 0;
  p.center = Vec2{center.x, center.y};
  p.scale = scale;
  s->w.polygons.push_back(std::move(p));
  return OK;
}
int b2d_add_polygon_circle(b2d_solver* s, float r, b2d_vec2 pos, size_t n, int is_static) {
  CHECK_S(s);
  MUTATE(s);
  s->w.polygons.push_back(Polygon::circle(r, Vec2{pos.x, pos.y}, n, is_static != 0));
  return OK;
}
int b2d_add_polygon_points(b2d_solver* s, size_t n, const b2d_vec2* pts, int is_static) {
  CHECK_S(s);
  if (n && !pts) return fail(ERR_NULL, "null points");
  MUTATE(s);
  std::vector<Vec2> v(n);
  for (size_t i = 0; i < n; ++i) v[i] = Vec2{pts[i].x, pts[i].y};
  s->w.polygons.push_back(Polygon::from_points(v, is_static != 0));
  return OK;
}

int b2d_set_sub_steps(b2d_solver* s, uint32_t n) {
  CHECK_S(s);
  MUTATE(s);
  s->w.sub_steps = n;
  return OK;
}
int b2d_get_sub_steps(b2d_solver* s, uint32_t* out) {
  CHECK_S(s);
  *out = s->w.sub_steps;
  return OK;
}
int b2d_set_link_iters(b2d_solver* s, uint32_t n) {
  CHECK_S(s);
  MUTATE(s);
  s->w.link_iters = n;
  return OK;
}
int b2d_set_mode(b2d_solver* s, int mode) {
  CHECK_S(s);
  if (mode != B2D_MODE_REFERENCE && mode != B2D_MODE_FAST) return fail(ERR_ARG, "unknown mode");
  MUTATE(s);
  s->w.mode = (uint32_t)mode;
  return OK;
}
int b2d_set_collision(b2d_solver* s, uint32_t flags, float r, float cell) {
  CHECK_S(s);
  if (flags & ~7u) return fail(ERR_ARG, "unknown collision flags");
  if (flags && !(r >= 0.0f && cell > 0.0f && cell >= 2.0f * r))
    return fail(ERR_ARG, "collisions need radius >= 0 and grid cell >= 2 * radius");
  MUTATE(s);
  s->w.collide = flags;
  s->w.particle_radius = r;
  s->w.grid_cell = cell;
  return OK;
}
int b2d_set_circle_static(b2d_solver* s, size_t i, int on) {
  CHECK_S(s);
  int st = sync_host(s);
  if (st != OK) return st;
  if (i >= s->w.circles.size()) return fail(ERR_INDEX, "circle index out of range");
  s->topo_dirty = true;
  s->w.circles[i].is_static = on ? 1u : 0u;
  return OK;
}

int b2d_set_tuning(b2d_solver* s, const char* key, double value) {
  CHECK_S(s);
  if (!key) return fail(ERR_NULL, "null key");
  if (!s->tune.set(key, value)) return fail(ERR_ARG, std::string("unknown tunable: ") + key);
  s->tune_set = true;
  MUTATE(s);
  if (s->own) s->own->set_tuning(s->tune);
  return OK;
}

int b2d_set_fault(b2d_solver* s, int kind, uint64_t value) {
  CHECK_S(s);
  if (s->batch) return fail(ERR_STATE, "solver belongs to a batch");
  Engine* e = nullptr;
  int st = engine_for(s, &e);
  if (st != OK) return st;
  st = e->set_fault(kind, value);
  return st == OK ? OK : fail(st, e->last_error);
}

int b2d_update(b2d_solver* s, float dt) {
  CHECK_S(s);
  if (s->batch) return fail(ERR_STATE, "solver belongs to a batch: use b2d_batch_update");
  int st = ensure_placed(s);
  if (st != OK) return st;
  st = s->eng->set_dt(s->slot, dt);
  if (st != OK) return fail(st, s->eng->last_error);
  st = s->eng->step();
  if (st != OK) return fail(st, s->eng->last_error);
  s->host_stale = true;
  return OK;
}

#define LEN_GETTER(fn, expr)            \
  int fn(b2d_solver* s, size_t* out) {  \
    CHECK_S(s);                         \
    if (!out) return fail(ERR_NULL, "null out"); \
    *out = (expr);                      \
    return OK;                          \
  }
LEN_GETTER(b2d_get_particle_len, s->w.particles.size())
LEN_GETTER(b2d_get_circles_len, s->w.circles.size())
LEN_GETTER(b2d_get_polygons_len, s->w.polygons.size())
LEN_GETTER(b2d_get_particle_links_len, s->w.particle_links.size())
LEN_GETTER(b2d_get_circle_links_len, s->w.circle_links.size())

static void put_link(const Link& l, b2d_link* d) {
  d->particle_a = l.particle_a;
  d->particle_b = l.particle_b;
  d->target_distance = l.target_distance;
  d->stiffness = l.stiffness;
}

int b2d_get_particle_links(b2d_solver* s, b2d_link* dst, size_t cap) {
  CHECK_S(s);
  if (cap < s->w.particle_links.size()) return fail(ERR_CAPACITY, "buffer too small");
  for (size_t i = 0; i < s->w.particle_links.size(); ++i) put_link(s->w.particle_links[i], dst + i);
  return OK;
}
int b2d_get_circle_links(b2d_solver* s, b2d_link* dst, size_t cap) {
  CHECK_S(s);
  if (cap < s->w.circle_links.size()) return fail(ERR_CAPACITY, "buffer too small");
  for (size_t i = 0; i < s->w.circle_links.size(); ++i) put_link(s->w.circle_links[i], dst + i);
  return OK;
}
int b2d_get_particles(b2d_solver* s, b2d_particle* dst, size_t cap) {
  CHECK_S(s);
  int st = sync_host(s);
  if (st != OK) return st;
  if (cap < s->w.particles.size()) return fail(ERR_CAPACITY, "buffer too small");
  if (!s->w.particles.empty())
    std::memcpy(dst, s->w.particles.data(), s->w.particles.size() * sizeof(Particle));
  return OK;
}
int b2d_get_particle(b2d_solver* s, size_t i, b2d_particle* out) {
  CHECK_S(s);
  int st = sync_host(s);
  if (st != OK) return st;
  if (i >= s->w.particles.size()) return fail(ERR_INDEX, "particle index out of range");
  std::memcpy(out, &s->w.particles[i], sizeof(Particle));
  return OK;
}
int b2d_get_circles(b2d_solver* s, b2d_circle* dst, size_t cap) {
  CHECK_S(s);
  int st = sync_host(s);
  if (st != OK) return st;
  if (cap < s->w.circles.size()) return fail(ERR_CAPACITY, "buffer too small");
  for (size_t i = 0; i < s->w.circles.size(); ++i) {
    std::memcpy(&dst[i].point, &s->w.circles[i].point, sizeof(Particle));
    dst[i].radius = s->w.circles[i].radius;
    dst[i].is_static = s->w.circles[i].is_static;
  }
  return OK;
}
int b2d_get_circle(b2d_solver* s, size_t i, b2d_circle* out) {
  CHECK_S(s);
  int st = sync_host(s);
  if (st != OK) return st;
  if (i >= s->w.circles.size()) return fail(ERR_INDEX, "circle index out of range");
  std::memcpy(&out->point, &s->w.circles[i].point, sizeof(Particle));
  out->radius = s->w.circles[i].radius;
  out->is_static = s->w.circles[i].is_static;
  return OK;
}
int b2d_get_polygon_info(b2d_solver* s, size_t i, size_t* nv, size_t* nl, int* is_static,
                         b2d_vec2* center, float* scale) {
  CHECK_S(s);
  int st = sync_host(s);
  if (st != OK) return st;
  if (i >= s->w.polygons.size()) return fail(ERR_INDEX, "polygon index out of range");
  const Polygon& p = s->w.polygons[i];
  if (nv) *nv = p.particles.size();
  if (nl) *nl = p.particle_links.size();
  if (is_static) *is_static = p.is_static ? 1 : 0;
  if (center) { center->x = p.center.x; center->y = p.center.y; }
  if (scale) *scale = p.scale;
  return OK;
}
int b2d_get_polygon(b2d_solver* s, size_t i, b2d_particle* v, size_t cap_v, b2d_link* l,
                    size_t cap_l) {
  CHECK_S(s);
  int st = sync_host(s);
  if (st != OK) return st;
  if (i >= s->w.polygons.size()) return fail(ERR_INDEX, "polygon index out of range");
  const Polygon& p = s->w.polygons[i];
  if ((v && cap_v < p.particles.size()) || (l && cap_l < p.particle_links.size()))
    return fail(ERR_CAPACITY, "buffer too small");
  if (v && !p.particles.empty()) std::memcpy(v, p.particles.data(), p.particles.size() * sizeof(Particle));
  if (l)
    for (size_t k = 0; k < p.particle_links.size(); ++k) put_link(p.particle_links[k], l + k);
  return OK;
}

int b2d_read_state(b2d_solver* s, float* pos, float* prev) {
  CHECK_S(s);
  int st = sync_host(s);
  if (st != OK) return st;
  for (size_t i = 0; i < s->w.particles.size(); ++i) {
    if (pos) { pos[2 * i] = s->w.particles[i].pos.x; pos[2 * i + 1] = s->w.particles[i].pos.y; }
    if (prev) { prev[2 * i] = s->w.particles[i].prev_pos.x; prev[2 * i + 1] = s->w.particles[i].prev_pos.y; }
  }
  return OK;
}
int b2d_write_state(b2d_solver* s, const float* pos, const float* prev) {
  CHECK_S(s);
  int st = sync_host(s);
  if (st != OK) return st;
  for (size_t i = 0; i < s->w.particles.size(); ++i) {
    if (pos) s->w.particles[i].pos = Vec2{pos[2 * i], pos[2 * i + 1]};
    if (prev) s->w.particles[i].prev_pos = Vec2{prev[2 * i], prev[2 * i + 1]};
  }
  if (s->placed && !s->topo_dirty) {
    st = s->eng->upload_state(s->slot);
    if (st != OK) return fail(st, s->eng->last_error);
  }
  return OK;
}

int b2d_set_stream(b2d_solver* s, void* stream) {
  CHECK_S(s);
  s->stream = static_cast<cudaStream_t>(stream);
  if (s->own) s->own->set_stream(s->stream);
  return OK;
}
int b2d_synchronize(b2d_solver* s) {
  CHECK_S(s);
  if (!s->eng) return OK;
  int st = s->eng->sync();
  return st == OK ? OK : fail(st, s->eng->last_error);
}
int b2d_set_graphs(b2d_solver* s, int on) {
  CHECK_S(s);
  s->graphs = on != 0;
  if (s->own) s->own->set_use_graph(s->graphs);
  return OK;
}
int b2d_set_profiling(b2d_solver* s, int on) {
  CHECK_S(s);
  s->profiling = on != 0;
  if (s->own) s->own->set_profile(s->profiling);
  return OK;
}

static int put_profile(Engine* e, char* names, size_t names_cap, float* ms, size_t cap,
                       size_t* count) {
  if (!e) {
    if (count) *count = 0;
    return OK;
  }
  const auto& p = e->last_profile();
  if (count) *count = p.size();
  std::string joined;
  for (size_t i = 0; i < p.size(); ++i) {
    if (i) joined += '\n';
    joined += p[i].first;
    if (ms && i < cap) ms[i] = p[i].second;
  }
  if (names && names_cap) {
    size_t n = std::min(names_cap - 1, joined.size());
    std::memcpy(names, joined.data(), n);
    names[n] = 0;
  }
  return OK;
}
int b2d_get_profile(b2d_solver* s, char* names, size_t names_cap, float* ms, size_t cap,
                    size_t* count) {
  CHECK_S(s);
  return put_profile(s->eng, names, names_cap, ms, cap, count);
}
int b2d_get_launch_count(b2d_solver* s, uint32_t* out) {
  CHECK_S(s);
  *out = s->eng ? s->eng->launches_per_step() : 0;
  return OK;
}

int b2d_state_bytes(b2d_solver* s, size_t* out) {
  CHECK_S(s);
  int st = ensure_placed(s);
  if (st != OK) return st;
  void* d;
  return s->eng->state_span(s->slot, &d, out);
}
int b2d_state_upload_async(b2d_solver* s, const void* src) {
  CHECK_S(s);
  int st = ensure_placed(s);
  if (st != OK) return st;
  void* d;
  size_t n;
  st = s->eng->state_span(s->slot, &d, &n);
  if (st != OK) return st;
  if (cudaMemcpyAsync(d, src, n, cudaMemcpyHostToDevice, s->eng->stream()) != cudaSuccess)
    return fail(ERR_CUDA, "state upload failed");
  s->host_stale = true;
  return OK;
}
int b2d_state_download_async(b2d_solver* s, void* dst) {
  CHECK_S(s);
  int st = ensure_placed(s);
  if (st != OK) return st;
  void* d;
  size_t n;
  st = s->eng->state_span(s->slot, &d, &n);
  if (st != OK) return st;
  if (cudaMemcpyAsync(dst, d, n, cudaMemcpyDeviceToHost, s->eng->stream()) != cudaSuccess)
    return fail(ERR_CUDA, "state download failed");
  return OK;
}

int b2d_get_plan_stats(b2d_solver* s, b2d_plan_stats* out) {
  CHECK_S(s);
  if (!out) return fail(ERR_NULL, "null out");
  std::memset(out, 0, sizeof(*out));
  const WorldImage* im = (s->placed && !s->topo_dirty) ? s->eng->image(s->slot) : nullptr;
  WorldImage tmp;
  if (!im) {  // plan on the host only (works without a GPU)
    int st = sync_host(s);
    if (st != OK) return st;
    SchedRegistry reg;
    std::string why;
    st = plan_world(s->w, s->tune, reg, tmp, &why);  // the solver's own tunables
    if (st != OK) return fail(st, why);
    im = &tmp;
  } else {
    out->device_bytes = s->eng->device_bytes();
  }
  out->bodies = im->stats.bodies;
  out->group_bodies = im->stats.group_bodies;
  out->serial_bodies = im->stats.serial_bodies;
  out->global_bodies = im->stats.global_bodies;
  out->levels = im->stats.levels;
  out->ops = im->stats.ops;
  out->colours = im->stats.colours;
  out->large_bodies = im->stats.large_bodies;
  return OK;
}
int b2d_get_link_order(b2d_solver* s, uint64_t* order, size_t cap) {
  CHECK_S(s);
  const size_t nl = s->w.particle_links.size();
  if (cap < nl) return fail(ERR_CAPACITY, "buffer too small");
  if (s->w.mode == MODE_FAST) {
    std::vector<uint32_t> o = colour_link_order(s->w, nullptr);
    for (size_t i = 0; i < nl; ++i) order[i] = o[i];
  } else {
    for (size_t i = 0; i < nl; ++i) order[i] = i;
  }
  return OK;
}

// ---- batch ---------------------------------------------------------------
int b2d_batch_create(b2d_batch** out) {
  if (!out) return fail(ERR_NULL, "null out");
  *out = new b2d_batch();
  return OK;
}
int b2d_batch_destroy(b2d_batch* b) {
  if (!b) return OK;
  {
    std::lock_guard<std::recursive_mutex> lk(b->mu);
    while (!b->members.empty()) b2d_batch_remove(b, b->members.back());
  }
  delete b;
  return OK;
}
int b2d_batch_add(b2d_batch* b, b2d_solver* s) {
  if (!b || !s) return fail(ERR_NULL, "null argument");
  std::lock_guard<std::recursive_mutex> lk(b->mu);
  if (s->batch) return fail(ERR_STATE, "solver already belongs to a batch");
  int st = unplace(s);
  if (st != OK) return st;
  s->batch = b;
  b->members.push_back(s);
  return OK;
}
int b2d_batch_remove(b2d_batch* b, b2d_solver* s) {
  if (!b || !s) return fail(ERR_NULL, "null argument");
  std::lock_guard<std::recursive_mutex> lk(b->mu);
  auto it = std::find(b->members.begin(), b->members.end(), s);
  if (it == b->members.end()) return fail(ERR_STATE, "solver is not in this batch");
  int st = unplace(s);
  if (st != OK) return st;
  b->members.erase(it);
  s->batch = nullptr;
  s->eng = nullptr;
  return OK;
}
int b2d_batch_update(b2d_batch* b, float dt) {
  if (!b) return fail(ERR_NULL, "null batch");
  std::lock_guard<std::recursive_mutex> lk(b->mu);
  for (b2d_solver* s : b->members) {
    int st = ensure_placed(s);
    if (st != OK) return st;
    st = s->eng->set_dt(s->slot, dt);
    if (st != OK) return fail(st, s->eng->last_error);
  }
  if (!b->eng) return OK;
  b->eng->set_profile(b->profiling);
  int st = b->eng->step();
  if (st != OK) return fail(st, b->eng->last_error);
  for (b2d_solver* s : b->members) s->host_stale = true;
  return OK;
}
int b2d_batch_synchronize(b2d_batch* b) {
  if (!b) return fail(ERR_NULL, "null batch");
  std::lock_guard<std::recursive_mutex> lk(b->mu);
  if (!b->eng) return OK;
  int st = b->eng->sync();
  return st == OK ? OK : fail(st, b->eng->last_error);
}
int b2d_batch_set_stream(b2d_batch* b, void* stream) {
  if (!b) return fail(ERR_NULL, "null batch");
  std::lock_guard<std::recursive_mutex> lk(b->mu);
  b->stream = static_cast<cudaStream_t>(stream);
  if (b->eng) b->eng->set_stream(b->stream);
  return OK;
}
int b2d_batch_set_profiling(b2d_batch* b, int on) {
  if (!b) return fail(ERR_NULL, "null batch");
  std::lock_guard<std::recursive_mutex> lk(b->mu);
  b->profiling = on != 0;
  return OK;
}
int b2d_batch_get_profile(b2d_batch* b, char* names, size_t names_cap, float* ms, size_t cap,
                          size_t* count) {
  if (!b) return fail(ERR_NULL, "null batch");
  std::lock_guard<std::recursive_mutex> lk(b->mu);
  return put_profile(b->eng.get(), names, names_cap, ms, cap, count);
}
int b2d_batch_set_tuning(b2d_batch* b, const char* key, double value) {
  if (!b || !key) return fail(ERR_NULL, "null argument");
  std::lock_guard<std::recursive_mutex> lk(b->mu);
  if (!b->tune.set(key, value)) return fail(ERR_ARG, std::string("unknown tunable: ") + key);
  b->tune_set = true;
  if (b->eng) {
    for (b2d_solver* s : b->members) {
      int st = unplace(s);
      if (st != OK) return st;
    }
    b->eng->set_tuning(b->tune);
  }
  return OK;
}
int b2d_batch_set_plain(b2d_batch* b, int on) {
  if (!b) return fail(ERR_NULL, "null batch");
  std::lock_guard<std::recursive_mutex> lk(b->mu);
  b->plain = on != 0;
  if (b->eng) b->eng->set_plain(b->plain);
  return OK;
}
int b2d_batch_get_launch_count(b2d_batch* b, uint32_t* out) {
  if (!b) return fail(ERR_NULL, "null batch");
  std::lock_guard<std::recursive_mutex> lk(b->mu);
  *out = b->eng ? b->eng->launches_per_step() : 0;
  return OK;
}

// ---- serving ---------------------------------------------------------------
int b2d_server_create(uint64_t budget_bytes, b2d_server** out) {
  if (!out) return fail(ERR_NULL, "null out");
  if (!have_gpu()) return fail(ERR_CUDA, "no CUDA device: bendy2d-gb300 has no CPU path");
  *out = new b2d_server();
  (*out)->sv = std::make_unique<Server>(budget_bytes);
  return OK;
}
int b2d_server_destroy(b2d_server* sv) {
  if (!sv) return OK;
  sv->sv->stop();
  delete sv;
  return OK;
}
int b2d_server_start(b2d_server* sv) {
  if (!sv) return fail(ERR_NULL, "null server");
  return sv->sv->start();
}
int b2d_server_stop(b2d_server* sv) {
  if (!sv) return fail(ERR_NULL, "null server");
  return sv->sv->stop();
}
int b2d_server_submit(b2d_server* sv, b2d_solver* world, uint32_t steps, float dt, uint64_t* id) {
  if (!sv || !world || !id) return fail(ERR_NULL, "null argument");
  int st = sync_host(world);
  if (st != OK) return st;
  std::string why;
  st = sv->sv->submit(world->w, steps, dt, id, &why);
  return st == OK ? OK : fail(st, why);
}
int b2d_server_cancel(b2d_server* sv, uint64_t id) {
  if (!sv) return fail(ERR_NULL, "null server");
  const int st = sv->sv->cancel(id);
  if (st == ERR_INDEX) return fail(st, "unknown request id");
  if (st == ERR_STATE) return fail(st, "request already finished");
  return st;
}
int b2d_server_set_max_resident_particles(b2d_server* sv, uint64_t n) {
  if (!sv) return fail(ERR_NULL, "null server");
  sv->sv->set_max_resident_particles(n);
  return OK;
}
int b2d_server_set_fault(b2d_server* sv, int kind, uint64_t value) {
  if (!sv) return fail(ERR_NULL, "null server");
  if (kind != FAULT_WAIT_TIMEOUT && kind != FAULT_GRID_CAP && kind != FAULT_ALLOC)
    return fail(ERR_ARG, "unknown fault kind " + std::to_string(kind));
  sv->sv->set_fault(kind, value);
  return OK;
}
int b2d_server_poll(b2d_server* sv, uint64_t id, int* state) {
  if (!sv || !state) return fail(ERR_NULL, "null argument");
  int st = sv->sv->poll(id, state);
  return st == OK ? OK : fail(st, "unknown request id");
}
int b2d_server_take(b2d_server* sv, uint64_t id, b2d_solver* dst, double* latency_s,
                    double* queue_s) {
  if (!sv || !dst) return fail(ERR_NULL, "null argument");
  int st = unplace(dst);
  if (st != OK) return st;
  std::string why;
  st = sv->sv->take(id, &dst->w, latency_s, queue_s, &why);
  if (st != OK) return fail(st, why);
  dst->topo_dirty = true;
  dst->host_stale = false;
  return OK;
}
int b2d_server_finished(b2d_server* sv, uint64_t* ids, size_t cap, size_t* n) {
  if (!sv || !n) return fail(ERR_NULL, "null argument");
  std::vector<uint64_t>& pend = sv->pending;
  std::vector<uint64_t> more = sv->sv->finished();
  pend.insert(pend.end(), more.begin(), more.end());
  const size_t k = std::min(cap, pend.size());
  if (k && ids) std::memcpy(ids, pend.data(), k * sizeof(uint64_t));
  pend.erase(pend.begin(), pend.begin() + k);
  *n = k;
  return OK;
}
int b2d_server_get_stats(b2d_server* sv, b2d_server_stats* out) {
  if (!sv || !out) return fail(ERR_NULL, "null argument");
  const ServerStats s = sv->sv->stats();
  out->submitted = s.submitted;
  out->admitted = s.admitted;
  out->completed = s.completed;
  out->failed = s.failed;
  out->queued = s.queued;
  out->active = s.active;
  out->ticks = s.ticks;
  out->particle_substeps = s.particle_substeps;
  out->resident_bytes = s.resident_bytes;
  out->admit_ns = s.admit_ns;
  out->step_ns = s.step_ns;
  out->retire_ns = s.retire_ns;
  out->cancelled = s.cancelled;
  out->resident_particles = s.resident_particles;
  return OK;
}

}  // extern "C"
