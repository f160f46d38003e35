// host.hpp — host-side mirror of the reference's public types and the world
// description the planner consumes.  Layout and defaults follow
// src/particle.rs:4-9, src/link.rs:4-33, src/circle.rs:4-8,
// src/polygon.rs:7-14 and src/solver.rs:13-50.
#pragma once
#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

namespace b2d {

enum Status : int {
  OK = 0,
  ERR_NULL = 1,
  ERR_LINK_INDEX = 2,         // reference panics: src/link.rs:19-21
  ERR_CIRCLE_LINK_INDEX = 3,  // reference panics: src/link.rs:37-39
  ERR_POLY_LINK_INDEX = 4,    // reference panics inside Polygon::solve_links
  ERR_ARG = 5,
  ERR_INDEX = 6,              // getter index out of range (Option::None)
  ERR_CUDA = 7,
  ERR_DEVICE = 8,
  ERR_BUDGET = 9,
  ERR_CAPACITY = 10,
  ERR_STATE = 11,
};

enum Mode : uint32_t { MODE_REFERENCE = 0, MODE_FAST = 1 };

struct Vec2 { float x, y; };
struct Particle { Vec2 pos, prev_pos, acc; };
struct Link { uint64_t particle_a, particle_b; float target_distance; float stiffness; };
struct Circle { Particle point; float radius; uint32_t is_static; };
struct Bounds { Vec2 pos, size; };

struct Polygon {
  std::vector<Particle> particles;
  std::vector<Link> particle_links;
  bool is_static = false;
  Vec2 center{0.0f, 0.0f};
  float scale = 1.0f;
  // Polygon::circle, src/polygon.rs:17-82
  static Polygon circle(float radius, Vec2 pos, size_t point_count, bool is_static);
  // Polygon::new, src/polygon.rs:84-123
  static Polygon from_points(const std::vector<Vec2>& points, bool is_static);
};

// One Solver's world (src/solver.rs:19-31) plus the extension knobs, whose
// defaults reproduce the reference.
struct WorldHost {
  Vec2 gravity{0.0f, 98.2f};
  Bounds bounds{{0.0f, 0.0f}, {100.0f, 100.0f}};
  bool bounds_active = true;  // accepted and ignored, like the reference (src/solver.rs:23)
  std::vector<Particle> particles;
  std::vector<Link> particle_links;
  std::vector<Circle> circles;
  std::vector<Link> circle_links;
  std::vector<Polygon> polygons;
  uint32_t sub_steps = 1;
  uint32_t link_iters = 1;
  uint32_t mode = MODE_REFERENCE;
  uint32_t collide = 0;
  float particle_radius = 0.5f;
  float grid_cell = 1.0f;
};

// Validation with the reference's panic conditions (a < b < len).
int validate_world(const WorldHost& w, std::string* why);

// Greedy edge colouring of the particle links in insertion order; returns
// the fast-mode link order (colour-major, insertion order within a colour).
std::vector<uint32_t> colour_link_order(const WorldHost& w, uint32_t* ncolours);

}  // namespace b2d
