/*
 * bendy2d.h — C ABI of bendy2d-gb300, a GB300 (sm_103a) implementation of
 * the Murrent/bendy2d 0.0.1 solver step.
 *
 * Every entry point returns an int status (B2D_OK = 0); b2d_last_error()
 * gives a message for the last failure on the calling thread.  The caller
 * owns host buffers; the library owns device memory.  A solver is used from
 * one thread at a time (the reference's update takes &mut self,
 * src/solver.rs:106).  Batch calls hold the batch's lock, so several threads
 * may call b2d_batch_* on one batch; calls on a member solver share the
 * batch's engine and must not overlap batch calls.  Servers synchronise
 * internally.
 *
 * Reference citations are file:line within the bendy2d crate (src/...).
 */
#ifndef BENDY2D_H
#define BENDY2D_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define B2D_OK 0
#define B2D_ERR_NULL 1
#define B2D_ERR_LINK_INDEX 2        /* a particle link breaks a < b < len; the reference panics in
                                       ParticleLink::solve (src/link.rs:19-21) */
#define B2D_ERR_CIRCLE_LINK_INDEX 3 /* same for circle links (src/link.rs:37-39) */
#define B2D_ERR_POLY_LINK_INDEX 4   /* same inside Polygon::solve_links (src/polygon.rs:218-223) */
#define B2D_ERR_ARG 5
#define B2D_ERR_INDEX 6             /* getter index out of range: the reference returns None
                                       (src/solver.rs:96-104) */
#define B2D_ERR_CUDA 7
#define B2D_ERR_DEVICE 8
#define B2D_ERR_BUDGET 9            /* serving: request exceeds the device-memory budget */
#define B2D_ERR_CAPACITY 10         /* caller buffer too small */
#define B2D_ERR_STATE 11            /* call not valid in the object's current state */

/* ---- modes and extension flags (not in the reference) ------------------ */
#define B2D_MODE_REFERENCE 0 /* replays the reference's sequential link order exactly */
#define B2D_MODE_FAST 1      /* links re-ordered by greedy colouring at build time */
#define B2D_COLLIDE_PP 1u    /* particle-particle, hashed uniform grid */
#define B2D_COLLIDE_PC 2u    /* particle-Circle */
#define B2D_COLLIDE_PPOLY 4u /* particle-Polygon edge projection */

/* ---- plain data, same fields as the reference -------------------------- */
typedef struct { float x, y; } b2d_vec2;                    /* nalgebra Vector2<f32> */
typedef struct { b2d_vec2 pos, prev_pos, acc; } b2d_particle; /* src/particle.rs:4-9 */
typedef struct {                                           /* src/link.rs:4-10 */
  uint64_t particle_a, particle_b; /* particle_a < particle_b (src/link.rs:6) */
  float target_distance;
  float stiffness; /* extension; 1.0 reproduces the reference */
} b2d_link;
typedef struct {                                           /* src/circle.rs:4-8 */
  b2d_particle point;
  float radius;
  uint32_t is_static; /* extension: a static circle is not integrated */
} b2d_circle;

typedef struct b2d_solver b2d_solver;
typedef struct b2d_batch b2d_batch;
typedef struct b2d_server b2d_server;

const char* b2d_last_error(void);
const char* b2d_version(void);

/* ---- Solver (src/solver.rs:19-189) ------------------------------------- */
int b2d_solver_create(b2d_solver** out);                    /* Solver::new, src/solver.rs:34-50 */
int b2d_solver_destroy(b2d_solver* s);
int b2d_solver_clone(b2d_solver* s, b2d_solver** out);      /* #[derive(Clone)], src/solver.rs:19 */

int b2d_set_gravity(b2d_solver* s, float x, float y);       /* pub gravity, src/solver.rs:21 */
int b2d_get_gravity(b2d_solver* s, b2d_vec2* out);
int b2d_set_bounds(b2d_solver* s, float px, float py, float sx, float sy); /* pub bounds, :22 */
int b2d_get_bounds(b2d_solver* s, b2d_vec2* pos, b2d_vec2* size);
int b2d_set_bounds_active(b2d_solver* s, int active);       /* pub bounds_active, :23 (never read) */
int b2d_get_bounds_active(b2d_solver* s, int* out);

int b2d_add_particle(b2d_solver* s, float x, float y);      /* Solver::add_particle, :52-54 */
int b2d_add_circle(b2d_solver* s, const b2d_circle* c);     /* Solver::add_circle, :55-57 */
int b2d_add_polygon(b2d_solver* s, size_t n_vertices, const b2d_particle* vertices,
                    size_t n_links, const b2d_link* links, int is_static, b2d_vec2 center,
                    float scale);                           /* Solver::add_polygon, :58-60 */
int b2d_add_particle_link(b2d_solver* s, uint64_t a, uint64_t b, float target_distance);
                                                            /* Solver::add_particle_link, :62-64 */
int b2d_add_circle_link(b2d_solver* s, uint64_t a, uint64_t b, float target_distance);
                                                            /* Solver::add_circle_link, :65-67 */

/* extension: initial velocity (prev_pos) and bulk uploads; prev_xy may be NULL */
int b2d_add_particle_prev(b2d_solver* s, float x, float y, float prev_x, float prev_y);
int b2d_add_particles(b2d_solver* s, size_t n, const float* pos_xy, const float* prev_xy);
int b2d_add_particle_links(b2d_solver* s, size_t n, const uint64_t* a, const uint64_t* b,
                           const float* target_distance, const float* stiffness /* NULL = 1 */);

/* Polygon::circle (src/polygon.rs:17-82) and Polygon::new (src/polygon.rs:84-123) added
 * directly to the solver */
int b2d_add_polygon_circle(b2d_solver* s, float radius, b2d_vec2 pos, size_t point_count,
                           int is_static);
int b2d_add_polygon_points(b2d_solver* s, size_t n, const b2d_vec2* points, int is_static);

/* extension knobs (private or absent in the reference; defaults reproduce it) */
int b2d_set_sub_steps(b2d_solver* s, uint32_t n);           /* private sub_steps = 1, :29,:47 */
int b2d_get_sub_steps(b2d_solver* s, uint32_t* out);
int b2d_set_link_iters(b2d_solver* s, uint32_t n);          /* apply_links repeated n times */
int b2d_set_mode(b2d_solver* s, int mode);                  /* B2D_MODE_* */
int b2d_set_collision(b2d_solver* s, uint32_t flags, float particle_radius, float grid_cell);
int b2d_set_circle_static(b2d_solver* s, size_t index, int is_static);
/* executor tunables (the autotuner sets these): serial_width, t_min, t_max,
 * pack_np, pack_nl, free_chunk, smem_max, warp_groups, max_groups,
 * width_per_thread, resident, res_max, stage_frac, bucket_factor,
 * collide_thread_min, large_max, grid_slot_max (collision particles up to
 * which the grid is built by slot inserts, above by a counting sort); they move
 * work between executors and never change results; take effect at the next
 * update; B2D_ERR_ARG for an unknown key */
int b2d_set_tuning(b2d_solver* s, const char* key, double value);

int b2d_update(b2d_solver* s, float dt);                    /* Solver::update, :106-116 */

/* fault injection, for tests of failure detection (no counterpart in the
 * reference, which has no failure handling): nothing here faults, traps or
 * hangs a GPU.  B2D_FAULT_WAIT_TIMEOUT (value != 0): every executor group
 * takes the timeout path of its first bulk-copy wait (device error word,
 * the copy in flight still lands, the group leaves), so b2d_synchronize
 * reports B2D_ERR_DEVICE.  B2D_FAULT_GRID_CAP (value > 0): the collision
 * grid holds at most `value` overflow entries per sub-step (the entries of a
 * bucket past its fixed slots; for the sorted grid, all entries); an
 * insert past that is refused instead of written past the array
 * (B2D_ERR_DEVICE).  B2D_FAULT_ALLOC: the next `value` world-block
 * allocations fail as if cudaMallocAsync had (B2D_ERR_CUDA).  Value 0 turns
 * a fault off; the solver's state after a reported failure is unspecified
 * until it is rewritten (b2d_write_state). */
#define B2D_FAULT_WAIT_TIMEOUT 1
#define B2D_FAULT_GRID_CAP 2
#define B2D_FAULT_ALLOC 3
int b2d_set_fault(b2d_solver* s, int kind, uint64_t value);

int b2d_get_particle_len(b2d_solver* s, size_t* out);       /* :69-71 */
int b2d_get_circles_len(b2d_solver* s, size_t* out);        /* :72-74 */
int b2d_get_polygons_len(b2d_solver* s, size_t* out);       /* :75-77 */
int b2d_get_particle_links_len(b2d_solver* s, size_t* out);
int b2d_get_circle_links_len(b2d_solver* s, size_t* out);
int b2d_get_particle_links(b2d_solver* s, b2d_link* dst, size_t cap);   /* :79-81 */
int b2d_get_circle_links(b2d_solver* s, b2d_link* dst, size_t cap);     /* :82-84 */
int b2d_get_particles(b2d_solver* s, b2d_particle* dst, size_t cap);    /* :86-88 */
int b2d_get_circles(b2d_solver* s, b2d_circle* dst, size_t cap);        /* :89-91 */
int b2d_get_particle(b2d_solver* s, size_t index, b2d_particle* out);   /* :96-98 */
int b2d_get_circle(b2d_solver* s, size_t index, b2d_circle* out);       /* :99-101 */
/* get_polygons / get_polygon (:92-94, :102-104) */
int b2d_get_polygon_info(b2d_solver* s, size_t index, size_t* n_vertices, size_t* n_links,
                         int* is_static, b2d_vec2* center, float* scale);
int b2d_get_polygon(b2d_solver* s, size_t index, b2d_particle* vertices, size_t cap_vertices,
                    b2d_link* links, size_t cap_links);

/* SoA state access (pos then prev, x/y interleaved, insertion order) */
int b2d_read_state(b2d_solver* s, float* pos_xy, float* prev_xy);
int b2d_write_state(b2d_solver* s, const float* pos_xy, const float* prev_xy);

/* execution control */
int b2d_set_stream(b2d_solver* s, void* cuda_stream);       /* NULL = library-owned stream */
int b2d_synchronize(b2d_solver* s);
int b2d_set_graphs(b2d_solver* s, int on);                  /* CUDA-graph replay (default on) */
int b2d_set_profiling(b2d_solver* s, int on);               /* per-kernel CUDA-event timing */
/* per-kernel times (ms) of the last profiled update: names joined by '\n' */
int b2d_get_profile(b2d_solver* s, char* names, size_t names_cap, float* ms, size_t cap,
                    size_t* count);
int b2d_get_launch_count(b2d_solver* s, uint32_t* out);     /* kernel launches per update */

/* end-to-end state transfer: the device state prefix of the solver (pos,
 * prev, circles, polygons) from/to host memory (pinned for speed) */
int b2d_state_bytes(b2d_solver* s, size_t* out);
int b2d_state_upload_async(b2d_solver* s, const void* host_src);
int b2d_state_download_async(b2d_solver* s, void* host_dst);

/* planning introspection */
typedef struct {
  uint32_t bodies, group_bodies, serial_bodies, global_bodies;
  uint64_t levels, ops;
  uint32_t colours;
  uint64_t device_bytes;
  /* group bodies over one CTA's shared memory that the large-body executor
   * runs from the shared memory of a thread-block cluster (global_bodies
   * counts the ones run from global memory) */
  uint32_t large_bodies;
} b2d_plan_stats;
int b2d_get_plan_stats(b2d_solver* s, b2d_plan_stats* out);
/* fast mode: the link order actually executed (world link ids) */
int b2d_get_link_order(b2d_solver* s, uint64_t* order, size_t cap);

/* ---- particle-collision sub-steps without allocation ------------------- */
/* No counterpart in the reference.  For callers that may not allocate GPU
 * memory while running (frame loops that reserve all device memory at
 * start-up, hosts that own and hand over every device buffer): runs
 * `sub_steps` sub-steps of particle-particle collision (hashed grid,
 * fixed-point Jacobi sum), bounds and Verlet integration on n link-free
 * particles held in the caller's device arrays (pos/prev, x/y interleaved),
 * in place, on `cuda_stream` -- the same arithmetic b2d_update applies to a
 * solver holding only these particles with B2D_COLLIDE_PP.  Allocates
 * nothing: all scratch lives in one static device array of about 3.6 MB,
 * mapped on a device when the library's kernels are first loaded there (at
 * the latest on the first call) and held until exit, so n is limited to
 * 65536 (B2D_ERR_CAPACITY beyond).  Calls share that array and each clears
 * what it needs: calls whose GPU work overlaps (other streams, other
 * threads) race.  Calls outside stream capture look the array's address up
 * on the current device; a call under capture reuses the last one found
 * there, so make the first call on each device before any stream capture
 * (B2D_ERR_STATE otherwise).  Returns once the work is queued; launch
 * failures of this call's own kernels give B2D_ERR_CUDA. */
typedef struct {
  float gravity_x, gravity_y;
  float bounds_x, bounds_y, bounds_w, bounds_h;
  float dt;
  uint32_t sub_steps;
  float particle_radius, grid_cell;
} b2d_noalloc_params;
int b2d_collide_substeps_noalloc(float* d_pos_xy, float* d_prev_xy, size_t n,
                                 const b2d_noalloc_params* params, void* cuda_stream);

/* ---- batch: many independent solvers stepped by one launch sequence ---- */
int b2d_batch_create(b2d_batch** out);
int b2d_batch_destroy(b2d_batch* b);       /* members return to their own engines */
int b2d_batch_add(b2d_batch* b, b2d_solver* s);
int b2d_batch_remove(b2d_batch* b, b2d_solver* s);
int b2d_batch_update(b2d_batch* b, float dt);  /* Solver::update on every member */
int b2d_batch_synchronize(b2d_batch* b);
int b2d_batch_set_stream(b2d_batch* b, void* cuda_stream);
int b2d_batch_set_profiling(b2d_batch* b, int on);
int b2d_batch_get_profile(b2d_batch* b, char* names, size_t names_cap, float* ms, size_t cap,
                          size_t* count);
int b2d_batch_get_launch_count(b2d_batch* b, uint32_t* out);
/* plain mode: each member world gets its own launches (no batching, no CUDA
 * graph) — the one-world-per-launch baseline the batched path is compared to */
int b2d_batch_set_plain(b2d_batch* b, int on);
/* executor tunables for every member (see b2d_set_tuning); re-plans members */
int b2d_batch_set_tuning(b2d_batch* b, const char* key, double value);

/* ---- serving: continuous batching of world-solve requests -------------- */
/* A request is a copy of a solver's world plus a number of Solver::update
 * calls (src/solver.rs:106-116).  A worker thread admits queued requests
 * first come first served while the device bytes of resident worlds stay
 * within the budget, steps every resident world once per tick in one launch
 * sequence, and retires finished requests.  A request taken from the queue
 * is planned on the host and installed on the device while the current
 * tick runs, and joins the next one (it stays B2D_SERVE_QUEUED until it is
 * installed).  Results are bit-identical to running the request alone. */
#define B2D_SERVE_QUEUED 0
#define B2D_SERVE_RUNNING 1
#define B2D_SERVE_DONE 2
#define B2D_SERVE_FAILED 3
#define B2D_SERVE_CANCELLED 4
typedef struct {
  uint64_t submitted, admitted, completed, failed, queued, active;
  uint64_t ticks, particle_substeps, resident_bytes;
  /* worker wall time, nanoseconds: admitting (planning and installing,
   * mostly while a tick runs), stepping (launch + wait, minus the admitting
   * done meanwhile), retiring (download + release) */
  uint64_t admit_ns, step_ns, retire_ns;
  uint64_t cancelled, resident_particles;
} b2d_server_stats;
int b2d_server_create(uint64_t budget_bytes, b2d_server** out);
int b2d_server_destroy(b2d_server* sv);
int b2d_server_start(b2d_server* sv);
int b2d_server_stop(b2d_server* sv);
/* B2D_ERR_BUDGET when the world alone exceeds the budget */
int b2d_server_submit(b2d_server* sv, b2d_solver* world, uint32_t steps, float dt,
                      uint64_t* id);
int b2d_server_poll(b2d_server* sv, uint64_t id, int* state);
/* drops a request: a queued one at once, a running one when the tick in
 * flight ends (its state becomes B2D_SERVE_CANCELLED and it is listed by
 * b2d_server_finished); B2D_ERR_STATE once it has finished */
int b2d_server_cancel(b2d_server* sv, uint64_t id);
/* admission also keeps the resident solver particles at or below n, so that
 * a tick (one update of every resident world) stays short under overload;
 * 0 = no limit (default); one request is always admitted onto an idle device */
int b2d_server_set_max_resident_particles(b2d_server* sv, uint64_t n);
/* fault injection (B2D_FAULT_*, see b2d_set_fault) on the server's engine,
 * applied before its next tick; B2D_FAULT_ALLOC fails the admission of the
 * next `value` requests to be installed, and only those */
int b2d_server_set_fault(b2d_server* sv, int kind, uint64_t value);
/* moves a finished request's world into dst (replacing its contents) and
 * releases the request; latency from submit to completion, queueing time */
int b2d_server_take(b2d_server* sv, uint64_t id, b2d_solver* dst, double* latency_s,
                    double* queue_s);
/* ids of requests finished (done or failed) since the last call, at most cap */
int b2d_server_finished(b2d_server* sv, uint64_t* ids, size_t cap, size_t* n);
int b2d_server_get_stats(b2d_server* sv, b2d_server_stats* out);

#ifdef __cplusplus
}
#endif
#endif /* BENDY2D_H */
