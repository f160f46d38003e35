// host.cpp — polygon builders, validation and fast-mode link colouring.
// Compiled with -ffp-contract=off: the builders' float arithmetic follows the
// reference op for op (rustc never contracts).
#include "host.hpp"

#include <algorithm>
#include <cmath>

namespace b2d {

static inline Vec2 vsub(Vec2 a, Vec2 b) { return {a.x - b.x, a.y - b.y}; }
static inline float vnorm(Vec2 a) { return std::sqrt(0.0f + (a.x * a.x + a.y * a.y)); }

static Particle particle_new(Vec2 p) { return Particle{p, p, {0.0f, 0.0f}}; }

// src/polygon.rs:17-82: vertices from an accumulated angle; chord links
// i -> i + 2n/3 and i -> i + n/3 (mod n), endpoints swapped so a < b,
// target = initial distance.
Polygon Polygon::circle(float radius, Vec2 pos, size_t n, bool is_static) {
  Polygon p;
  Vec2 center{0.0f, 0.0f};
  float angle = 0.0f;
  for (size_t i = 0; i < n; ++i) {
    float x = radius * std::cos(angle);
    float y = radius * std::sin(angle);
    Particle pt = particle_new(Vec2{pos.x + x, pos.y + y});
    p.particles.push_back(pt);
    center.x = center.x + pt.pos.x;
    center.y = center.y + pt.pos.y;
    angle += 2.0f * 3.14159265358979323846f / (float)n;
  }
  center.x = center.x / (float)n;
  center.y = center.y / (float)n;
  for (size_t i = 0; i < n; ++i) {
    const size_t offs[2] = {2 * n / 3, n / 3};
    for (size_t k = 0; k < 2; ++k) {
      size_t a = i, b = (i + offs[k]) % n;
      if (a > b) std::swap(a, b);
      Vec2 d = vsub(p.particles[a].pos, p.particles[b].pos);
      p.particle_links.push_back(Link{a, b, vnorm(d), 1.0f});
    }
  }
  p.is_static = is_static;
  p.center = center;
  p.scale = 1.0f;
  return p;
}

// src/polygon.rs:84-123: perimeter links i -> (i+1) mod n.
Polygon Polygon::from_points(const std::vector<Vec2>& pts, bool is_static) {
  Polygon p;
  Vec2 center{0.0f, 0.0f};
  for (const Vec2& v : pts) {
    p.particles.push_back(particle_new(v));
    center.x = center.x + v.x;
    center.y = center.y + v.y;
  }
  center.x = center.x / (float)pts.size();
  center.y = center.y / (float)pts.size();
  const size_t n = pts.size();
  for (size_t i = 0; i < n; ++i) {
    size_t a = i, b = (i + 1) % n;
    if (a > b) std::swap(a, b);
    Vec2 d = vsub(p.particles[a].pos, p.particles[b].pos);
    p.particle_links.push_back(Link{a, b, vnorm(d), 1.0f});
  }
  p.is_static = is_static;
  p.center = center;
  p.scale = 1.0f;
  return p;
}

int validate_world(const WorldHost& w, std::string* why) {
  const uint64_t np = w.particles.size();
  for (size_t i = 0; i < w.particle_links.size(); ++i) {
    const Link& l = w.particle_links[i];
    if (!(l.particle_a < l.particle_b && l.particle_b < np)) {
      if (why) *why = "particle link " + std::to_string(i) + " needs a < b < particle count";
      return ERR_LINK_INDEX;
    }
  }
  const uint64_t nc = w.circles.size();
  for (size_t i = 0; i < w.circle_links.size(); ++i) {
    const Link& l = w.circle_links[i];
    if (!(l.particle_a < l.particle_b && l.particle_b < nc)) {
      if (why) *why = "circle link " + std::to_string(i) + " needs a < b < circle count";
      return ERR_CIRCLE_LINK_INDEX;
    }
  }
  for (size_t p = 0; p < w.polygons.size(); ++p) {
    const Polygon& g = w.polygons[p];
    for (size_t i = 0; i < g.particle_links.size(); ++i) {
      const Link& l = g.particle_links[i];
      if (!(l.particle_a < l.particle_b && l.particle_b < g.particles.size())) {
        if (why)
          *why = "polygon " + std::to_string(p) + " link " + std::to_string(i) +
                 " needs a < b < vertex count";
        return ERR_POLY_LINK_INDEX;
      }
    }
  }
  if (w.mode != MODE_REFERENCE && w.mode != MODE_FAST) {
    if (why) *why = "unknown mode";
    return ERR_ARG;
  }
  return OK;
}

std::vector<uint32_t> colour_link_order(const WorldHost& w, uint32_t* ncolours) {
  const size_t nl = w.particle_links.size();
  std::vector<std::vector<uint32_t>> used(w.particles.size());
  std::vector<uint32_t> colour(nl);
  uint32_t maxc = 0;
  for (size_t k = 0; k < nl; ++k) {
    const auto& ua = used[w.particle_links[k].particle_a];
    const auto& ub = used[w.particle_links[k].particle_b];
    uint32_t c = 0;
    for (;; ++c) {
      if (std::find(ua.begin(), ua.end(), c) != ua.end()) continue;
      if (std::find(ub.begin(), ub.end(), c) != ub.end()) continue;
      break;
    }
    colour[k] = c;
    used[w.particle_links[k].particle_a].push_back(c);
    used[w.particle_links[k].particle_b].push_back(c);
    maxc = std::max(maxc, c + 1);
  }
  std::vector<uint32_t> order(nl);
  for (size_t k = 0; k < nl; ++k) order[k] = (uint32_t)k;
  std::stable_sort(order.begin(), order.end(),
                   [&](uint32_t x, uint32_t y) { return colour[x] < colour[y]; });
  if (ncolours) *ncolours = maxc;
  return order;
}

}  // namespace b2d
