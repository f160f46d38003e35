/*
 * b2d_oracle.h — CPU oracle for the bendy2d solver step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * Rust crate Murrent/bendy2d 0.0.1 (src/*.rs), used by the test-suite, the
 * smoke check and the CPU-baseline leg of the benchmark to check the CUDA
 * product path.  The product never links, loads or calls it.
 *
 * PARITY UNPINNED: the reference has no tests, fixtures or golden vectors, it
 * cannot be compiled here (no Rust toolchain), and its only dependency,
 * nalgebra "^0.32.2" (Cargo.toml:17-18), is not vendored.  This restatement is
 * anchored by source reading plus first-principles known-answer tests
 * (tests/golden/kat_*.json), nothing more.
 *
 * nalgebra 0.32 semantics assumed for Vector2<f32> (documented behaviour):
 *   norm_squared(v) = 0 + (x*x + y*y)   (zero-initialised sum of dotc)
 *   norm(v)         = sqrt(norm_squared(v))
 *   normalize(v)    = v / norm(v)       (component-wise division)
 *   dot(a, b)       = a.x*b.x + a.y*b.y
 *   v * s, v / s    = component-wise; expressions evaluate left to right.
 * Compiled with -ffp-contract=off: rustc never fuses multiply-add.
 *
 * Extensions that the reference does not have (sub-step setter, link
 * iterations, stiffness, static circles, particle collisions) are switched
 * off by default; with defaults the oracle is the reference algorithm.
 */
#ifndef B2D_ORACLE_H
#define B2D_ORACLE_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_world orc_world;

/* status codes (same values as the product's B2D_* codes) */
#define ORC_OK 0
#define ORC_ERR_LINK_INDEX 2     /* reference panics: split_at_mut / index OOB, src/link.rs:19-21 */
#define ORC_ERR_CIRCLE_LINK_INDEX 3
#define ORC_ERR_POLY_LINK_INDEX 4
#define ORC_ERR_ARG 5

/* extension collision flags */
#define ORC_COLLIDE_PP 1u      /* particle-particle, uniform grid */
#define ORC_COLLIDE_PC 2u      /* particle-Circle */
#define ORC_COLLIDE_PPOLY 4u   /* particle-Polygon edge projection */

orc_world* orc_new(void);                                   /* Solver::new, src/solver.rs:34-50 */
void orc_free(orc_world* w);
orc_world* orc_clone(const orc_world* w);                   /* #[derive(Clone)], src/solver.rs:19 */

void orc_set_gravity(orc_world* w, float x, float y);       /* pub gravity, src/solver.rs:21 */
void orc_set_bounds(orc_world* w, float px, float py, float sx, float sy); /* pub bounds :22 */
void orc_set_sub_steps(orc_world* w, uint32_t n);           /* ext: private field :29 */
void orc_set_link_iters(orc_world* w, uint32_t n);          /* ext */
void orc_set_collide(orc_world* w, uint32_t flags, float particle_radius, float cell);

/* Solver::add_particle (src/solver.rs:52-54) is n=1, prev=NULL. prev: ext. */
void orc_add_particles(orc_world* w, size_t n, const float* pos_xy, const float* prev_xy);
/* Solver::add_particle_link (src/solver.rs:62-64); stiffness may be NULL (=1). */
void orc_add_particle_links(orc_world* w, size_t n, const uint64_t* a, const uint64_t* b,
                            const float* target, const float* stiffness);
/* Solver::add_circle (src/solver.rs:55-57) */
void orc_add_circle(orc_world* w, const float* pos, const float* prev, const float* acc,
                    float radius, int is_static);
/* Solver::add_circle_link (src/solver.rs:65-67) */
void orc_add_circle_link(orc_world* w, uint64_t a, uint64_t b, float target);
/* Solver::add_polygon (src/solver.rs:58-60) with explicit polygon contents */
void orc_add_polygon(orc_world* w, size_t nv, const float* pos, const float* prev,
                     const float* acc, size_t nl, const uint64_t* la, const uint64_t* lb,
                     const float* ltarget, int is_static, float cx, float cy, float scale);
/* Polygon::circle (src/polygon.rs:17-82) / Polygon::new (src/polygon.rs:84-123), added to w */
void orc_add_polygon_circle(orc_world* w, float radius, float x, float y, size_t n, int is_static);
void orc_add_polygon_points(orc_world* w, size_t n, const float* pts, int is_static);

/* Solver::update, src/solver.rs:106-116 */
int orc_update(orc_world* w, float dt);

size_t orc_particle_len(const orc_world* w);
size_t orc_circle_len(const orc_world* w);
size_t orc_polygon_len(const orc_world* w);
size_t orc_polygon_vertex_len(const orc_world* w, size_t i);
size_t orc_polygon_link_len(const orc_world* w, size_t i);
/* xy pairs */
void orc_read_particles(const orc_world* w, float* pos, float* prev);
void orc_read_circles(const orc_world* w, float* pos, float* prev);
void orc_read_polygon(const orc_world* w, size_t i, float* pos, float* prev, float* center);
void orc_read_polygon_links(const orc_world* w, size_t i, uint64_t* a, uint64_t* b, float* target);

/* diagnostics used by long-run tests */
double orc_link_residual(const orc_world* w);   /* max |len - rest| / rest over particle links */

#ifdef __cplusplus
}
#endif
#endif
