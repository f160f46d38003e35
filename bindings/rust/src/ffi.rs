//! Raw declarations of the C ABI in `include/bendy2d.h`, one per entry point,
//! in the header's order.  Every function returns a status code (`B2D_OK` =
//! 0); `b2d_last_error` gives the message of the calling thread's last
//! failure.  The safe types of this crate wrap these calls.
#![allow(non_camel_case_types)]

use std::os::raw::{c_char, c_double, c_int, c_void};

pub const B2D_OK: c_int = 0;
pub const B2D_ERR_NULL: c_int = 1;
pub const B2D_ERR_LINK_INDEX: c_int = 2;
pub const B2D_ERR_CIRCLE_LINK_INDEX: c_int = 3;
pub const B2D_ERR_POLY_LINK_INDEX: c_int = 4;
pub const B2D_ERR_ARG: c_int = 5;
pub const B2D_ERR_INDEX: c_int = 6;
pub const B2D_ERR_CUDA: c_int = 7;
pub const B2D_ERR_DEVICE: c_int = 8;
pub const B2D_ERR_BUDGET: c_int = 9;
pub const B2D_ERR_CAPACITY: c_int = 10;
pub const B2D_ERR_STATE: c_int = 11;

pub const B2D_MODE_REFERENCE: c_int = 0;
pub const B2D_MODE_FAST: c_int = 1;
pub const B2D_COLLIDE_PP: u32 = 1;
pub const B2D_COLLIDE_PC: u32 = 2;
pub const B2D_COLLIDE_PPOLY: u32 = 4;

pub const B2D_SERVE_QUEUED: c_int = 0;
pub const B2D_SERVE_RUNNING: c_int = 1;
pub const B2D_SERVE_DONE: c_int = 2;
pub const B2D_SERVE_FAILED: c_int = 3;
pub const B2D_SERVE_CANCELLED: c_int = 4;

pub const B2D_FAULT_WAIT_TIMEOUT: c_int = 1;
pub const B2D_FAULT_GRID_CAP: c_int = 2;
pub const B2D_FAULT_ALLOC: c_int = 3;

#[repr(C)]
#[derive(Debug, Clone, Copy, Default, PartialEq)]
pub struct b2d_vec2 {
    pub x: f32,
    pub y: f32,
}

#[repr(C)]
#[derive(Debug, Clone, Copy, Default, PartialEq)]
pub struct b2d_particle {
    pub pos: b2d_vec2,
    pub prev_pos: b2d_vec2,
    pub acc: b2d_vec2,
}

#[repr(C)]
#[derive(Debug, Clone, Copy, Default, PartialEq)]
pub struct b2d_link {
    pub particle_a: u64,
    pub particle_b: u64,
    pub target_distance: f32,
    pub stiffness: f32,
}

#[repr(C)]
#[derive(Debug, Clone, Copy, Default, PartialEq)]
pub struct b2d_circle {
    pub point: b2d_particle,
    pub radius: f32,
    pub is_static: u32,
}

#[repr(C)]
#[derive(Debug, Clone, Copy, Default, PartialEq)]
pub struct b2d_plan_stats {
    pub bodies: u32,
    pub group_bodies: u32,
    pub serial_bodies: u32,
    pub global_bodies: u32,
    pub levels: u64,
    pub ops: u64,
    pub colours: u32,
    pub device_bytes: u64,
    pub large_bodies: u32,
}

#[repr(C)]
#[derive(Debug, Clone, Copy, Default, PartialEq)]
pub struct b2d_noalloc_params {
    pub gravity_x: f32,
    pub gravity_y: f32,
    pub bounds_x: f32,
    pub bounds_y: f32,
    pub bounds_w: f32,
    pub bounds_h: f32,
    pub dt: f32,
    pub sub_steps: u32,
    pub particle_radius: f32,
    pub grid_cell: f32,
}

#[repr(C)]
#[derive(Debug, Clone, Copy, Default, PartialEq)]
pub struct b2d_server_stats {
    pub submitted: u64,
    pub admitted: u64,
    pub completed: u64,
    pub failed: u64,
    pub queued: u64,
    pub active: u64,
    pub ticks: u64,
    pub particle_substeps: u64,
    pub resident_bytes: u64,
    pub admit_ns: u64,
    pub step_ns: u64,
    pub retire_ns: u64,
    pub cancelled: u64,
    pub resident_particles: u64,
}

/// Opaque handles.
#[repr(C)]
pub struct b2d_solver {
    _private: [u8; 0],
}
#[repr(C)]
pub struct b2d_batch {
    _private: [u8; 0],
}
#[repr(C)]
pub struct b2d_server {
    _private: [u8; 0],
}

extern "C" {
    pub fn b2d_last_error() -> *const c_char;
    pub fn b2d_version() -> *const c_char;

    // Solver (src/solver.rs:19-189)
    pub fn b2d_solver_create(out: *mut *mut b2d_solver) -> c_int;
    pub fn b2d_solver_destroy(s: *mut b2d_solver) -> c_int;
    pub fn b2d_solver_clone(s: *mut b2d_solver, out: *mut *mut b2d_solver) -> c_int;

    pub fn b2d_set_gravity(s: *mut b2d_solver, x: f32, y: f32) -> c_int;
    pub fn b2d_get_gravity(s: *mut b2d_solver, out: *mut b2d_vec2) -> c_int;
    pub fn b2d_set_bounds(s: *mut b2d_solver, px: f32, py: f32, sx: f32, sy: f32) -> c_int;
    pub fn b2d_get_bounds(s: *mut b2d_solver, pos: *mut b2d_vec2, size: *mut b2d_vec2) -> c_int;
    pub fn b2d_set_bounds_active(s: *mut b2d_solver, active: c_int) -> c_int;
    pub fn b2d_get_bounds_active(s: *mut b2d_solver, out: *mut c_int) -> c_int;

    pub fn b2d_add_particle(s: *mut b2d_solver, x: f32, y: f32) -> c_int;
    pub fn b2d_add_circle(s: *mut b2d_solver, c: *const b2d_circle) -> c_int;
    pub fn b2d_add_polygon(
        s: *mut b2d_solver,
        n_vertices: usize,
        vertices: *const b2d_particle,
        n_links: usize,
        links: *const b2d_link,
        is_static: c_int,
        center: b2d_vec2,
        scale: f32,
    ) -> c_int;
    pub fn b2d_add_particle_link(s: *mut b2d_solver, a: u64, b: u64, target_distance: f32) -> c_int;
    pub fn b2d_add_circle_link(s: *mut b2d_solver, a: u64, b: u64, target_distance: f32) -> c_int;

    pub fn b2d_add_particle_prev(s: *mut b2d_solver, x: f32, y: f32, prev_x: f32, prev_y: f32) -> c_int;
    pub fn b2d_add_particles(s: *mut b2d_solver, n: usize, pos_xy: *const f32, prev_xy: *const f32) -> c_int;
    pub fn b2d_add_particle_links(
        s: *mut b2d_solver,
        n: usize,
        a: *const u64,
        b: *const u64,
        target_distance: *const f32,
        stiffness: *const f32,
    ) -> c_int;

    pub fn b2d_add_polygon_circle(
        s: *mut b2d_solver,
        radius: f32,
        pos: b2d_vec2,
        point_count: usize,
        is_static: c_int,
    ) -> c_int;
    pub fn b2d_add_polygon_points(s: *mut b2d_solver, n: usize, points: *const b2d_vec2, is_static: c_int) -> c_int;

    pub fn b2d_set_sub_steps(s: *mut b2d_solver, n: u32) -> c_int;
    pub fn b2d_get_sub_steps(s: *mut b2d_solver, out: *mut u32) -> c_int;
    pub fn b2d_set_link_iters(s: *mut b2d_solver, n: u32) -> c_int;
    pub fn b2d_set_mode(s: *mut b2d_solver, mode: c_int) -> c_int;
    pub fn b2d_set_collision(s: *mut b2d_solver, flags: u32, particle_radius: f32, grid_cell: f32) -> c_int;
    pub fn b2d_set_circle_static(s: *mut b2d_solver, index: usize, is_static: c_int) -> c_int;
    pub fn b2d_set_tuning(s: *mut b2d_solver, key: *const c_char, value: c_double) -> c_int;

    pub fn b2d_update(s: *mut b2d_solver, dt: f32) -> c_int;
    pub fn b2d_set_fault(s: *mut b2d_solver, kind: c_int, value: u64) -> c_int;

    pub fn b2d_get_particle_len(s: *mut b2d_solver, out: *mut usize) -> c_int;
    pub fn b2d_get_circles_len(s: *mut b2d_solver, out: *mut usize) -> c_int;
    pub fn b2d_get_polygons_len(s: *mut b2d_solver, out: *mut usize) -> c_int;
    pub fn b2d_get_particle_links_len(s: *mut b2d_solver, out: *mut usize) -> c_int;
    pub fn b2d_get_circle_links_len(s: *mut b2d_solver, out: *mut usize) -> c_int;
    pub fn b2d_get_particle_links(s: *mut b2d_solver, dst: *mut b2d_link, cap: usize) -> c_int;
    pub fn b2d_get_circle_links(s: *mut b2d_solver, dst: *mut b2d_link, cap: usize) -> c_int;
    pub fn b2d_get_particles(s: *mut b2d_solver, dst: *mut b2d_particle, cap: usize) -> c_int;
    pub fn b2d_get_circles(s: *mut b2d_solver, dst: *mut b2d_circle, cap: usize) -> c_int;
    pub fn b2d_get_particle(s: *mut b2d_solver, index: usize, out: *mut b2d_particle) -> c_int;
    pub fn b2d_get_circle(s: *mut b2d_solver, index: usize, out: *mut b2d_circle) -> c_int;
    pub fn b2d_get_polygon_info(
        s: *mut b2d_solver,
        index: usize,
        n_vertices: *mut usize,
        n_links: *mut usize,
        is_static: *mut c_int,
        center: *mut b2d_vec2,
        scale: *mut f32,
    ) -> c_int;
    pub fn b2d_get_polygon(
        s: *mut b2d_solver,
        index: usize,
        vertices: *mut b2d_particle,
        cap_vertices: usize,
        links: *mut b2d_link,
        cap_links: usize,
    ) -> c_int;

    pub fn b2d_read_state(s: *mut b2d_solver, pos_xy: *mut f32, prev_xy: *mut f32) -> c_int;
    pub fn b2d_write_state(s: *mut b2d_solver, pos_xy: *const f32, prev_xy: *const f32) -> c_int;

    pub fn b2d_set_stream(s: *mut b2d_solver, cuda_stream: *mut c_void) -> c_int;
    pub fn b2d_synchronize(s: *mut b2d_solver) -> c_int;
    pub fn b2d_set_graphs(s: *mut b2d_solver, on: c_int) -> c_int;
    pub fn b2d_set_profiling(s: *mut b2d_solver, on: c_int) -> c_int;
    pub fn b2d_get_profile(
        s: *mut b2d_solver,
        names: *mut c_char,
        names_cap: usize,
        ms: *mut f32,
        cap: usize,
        count: *mut usize,
    ) -> c_int;
    pub fn b2d_get_launch_count(s: *mut b2d_solver, out: *mut u32) -> c_int;

    pub fn b2d_state_bytes(s: *mut b2d_solver, out: *mut usize) -> c_int;
    pub fn b2d_state_upload_async(s: *mut b2d_solver, host_src: *const c_void) -> c_int;
    pub fn b2d_state_download_async(s: *mut b2d_solver, host_dst: *mut c_void) -> c_int;

    pub fn b2d_get_plan_stats(s: *mut b2d_solver, out: *mut b2d_plan_stats) -> c_int;
    pub fn b2d_get_link_order(s: *mut b2d_solver, order: *mut u64, cap: usize) -> c_int;

    pub fn b2d_collide_substeps_noalloc(
        d_pos_xy: *mut f32,
        d_prev_xy: *mut f32,
        n: usize,
        params: *const b2d_noalloc_params,
        cuda_stream: *mut c_void,
    ) -> c_int;

    // batch: many independent solvers stepped by one launch sequence
    pub fn b2d_batch_create(out: *mut *mut b2d_batch) -> c_int;
    pub fn b2d_batch_destroy(b: *mut b2d_batch) -> c_int;
    pub fn b2d_batch_add(b: *mut b2d_batch, s: *mut b2d_solver) -> c_int;
    pub fn b2d_batch_remove(b: *mut b2d_batch, s: *mut b2d_solver) -> c_int;
    pub fn b2d_batch_update(b: *mut b2d_batch, dt: f32) -> c_int;
    pub fn b2d_batch_synchronize(b: *mut b2d_batch) -> c_int;
    pub fn b2d_batch_set_stream(b: *mut b2d_batch, cuda_stream: *mut c_void) -> c_int;
    pub fn b2d_batch_set_profiling(b: *mut b2d_batch, on: c_int) -> c_int;
    pub fn b2d_batch_get_profile(
        b: *mut b2d_batch,
        names: *mut c_char,
        names_cap: usize,
        ms: *mut f32,
        cap: usize,
        count: *mut usize,
    ) -> c_int;
    pub fn b2d_batch_get_launch_count(b: *mut b2d_batch, out: *mut u32) -> c_int;
    pub fn b2d_batch_set_plain(b: *mut b2d_batch, on: c_int) -> c_int;
    pub fn b2d_batch_set_tuning(b: *mut b2d_batch, key: *const c_char, value: c_double) -> c_int;

    // serving: continuous batching of world-solve requests
    pub fn b2d_server_create(budget_bytes: u64, out: *mut *mut b2d_server) -> c_int;
    pub fn b2d_server_destroy(sv: *mut b2d_server) -> c_int;
    pub fn b2d_server_start(sv: *mut b2d_server) -> c_int;
    pub fn b2d_server_stop(sv: *mut b2d_server) -> c_int;
    pub fn b2d_server_submit(sv: *mut b2d_server, world: *mut b2d_solver, steps: u32, dt: f32, id: *mut u64) -> c_int;
    pub fn b2d_server_poll(sv: *mut b2d_server, id: u64, state: *mut c_int) -> c_int;
    pub fn b2d_server_cancel(sv: *mut b2d_server, id: u64) -> c_int;
    pub fn b2d_server_set_max_resident_particles(sv: *mut b2d_server, n: u64) -> c_int;
    pub fn b2d_server_set_fault(sv: *mut b2d_server, kind: c_int, value: u64) -> c_int;
    pub fn b2d_server_take(
        sv: *mut b2d_server,
        id: u64,
        dst: *mut b2d_solver,
        latency_s: *mut c_double,
        queue_s: *mut c_double,
    ) -> c_int;
    pub fn b2d_server_finished(sv: *mut b2d_server, ids: *mut u64, cap: usize, n: *mut usize) -> c_int;
    pub fn b2d_server_get_stats(sv: *mut b2d_server, out: *mut b2d_server_stats) -> c_int;
}
