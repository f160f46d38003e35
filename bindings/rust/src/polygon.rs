//! `Polygon`, src/polygon.rs:7-237.
use std::os::raw::c_int;

use nalgebra::Vector2;

use crate::common::line_intersection;
use crate::error::expect;
use crate::ffi;
use crate::link::ParticleLink;
use crate::particle::{vec_to_ffi, Particle};
use crate::solver::{read_polygon, Bounds};

/// A soft polygon: its vertex particles, the links that hold its shape, and
/// the centre used by the polygon-polygon contacts (`src/polygon.rs:7-14`).
#[derive(Debug, Clone)]
pub struct Polygon {
    pub particles: Vec<Particle>,
    pub particle_links: Vec<ParticleLink>,
    pub is_static: bool,
    pub center: Vector2<f32>,
    pub scale: f32,
}

/// A solver handle used only to run the library's polygon builders, which
/// are the same host code `Solver::add_polygon` meets inside the library.
struct Scratch(*mut ffi::b2d_solver);

impl Scratch {
    fn new() -> Self {
        let mut raw = std::ptr::null_mut();
        expect(unsafe { ffi::b2d_solver_create(&mut raw) });
        Scratch(raw)
    }
}

impl Drop for Scratch {
    fn drop(&mut self) {
        unsafe { ffi::b2d_solver_destroy(self.0) };
    }
}

impl Polygon {
    /// A regular polygon of `point_count` vertices on a circle, with
    /// perimeter links and the two chord families of `src/polygon.rs:17-82`.
    /// The reference accepts `point_count < 3` and panics at the first
    /// update; the library refuses it here, with a panic.
    pub fn circle(radius: f32, pos: Vector2<f32>, point_count: usize, is_static: bool) -> Self {
        let s = Scratch::new();
        expect(unsafe { ffi::b2d_add_polygon_circle(s.0, radius, vec_to_ffi(pos), point_count, is_static as c_int) });
        read_polygon(s.0, 0)
    }

    /// A polygon through `points` with perimeter links (`src/polygon.rs:84-123`).
    pub fn new(points: Vec<Vector2<f32>>, is_static: bool) -> Self {
        let s = Scratch::new();
        let pts: Vec<ffi::b2d_vec2> = points.iter().map(|p| vec_to_ffi(*p)).collect();
        expect(unsafe { ffi::b2d_add_polygon_points(s.0, pts.len(), pts.as_ptr(), is_static as c_int) });
        read_polygon(s.0, 0)
    }

    /// Centre update, then one Verlet step of every vertex, unless static
    /// (`src/polygon.rs:125-134`).
    pub fn update(&mut self, dt: f32) {
        if self.is_static {
            return;
        }
        self.calc_center();
        for p in &mut self.particles {
            p.update(dt);
        }
    }

    /// `Particle::solve_bounds` on every vertex (`src/polygon.rs:136-140`).
    pub fn solve_bounds(&mut self, bounds: Bounds) {
        for p in &mut self.particles {
            p.solve_bounds(bounds);
        }
    }

    /// Both directions of the edge-versus-vertex contact
    /// (`src/polygon.rs:142-145`).
    pub fn solve_polygon(&mut self, other: &mut Polygon) {
        self.solve_polygon_single(other);
        other.solve_polygon_single(self);
    }

    /// Every edge (i, i+1) of `self` against every vertex of `other`, as in
    /// `src/polygon.rs:147-162`: the edge's end points are copied when the
    /// edge starts and those copies are used for all of `other`'s vertices,
    /// while each hit writes both end points and the vertex.
    pub fn solve_polygon_single(&mut self, other: &mut Polygon) {
        let n = self.particles.len();
        for i in 0..n {
            let j = (i + 1) % n;
            let a = self.particles[i];
            let b = self.particles[j];
            let other_center = other.center;
            for q in &mut other.particles {
                if let Some((na, nb, nq)) = edge_contact(self.center, &a, &b, q, other_center) {
                    self.particles[i].pos = na;
                    self.particles[j].pos = nb;
                    q.pos = nq;
                }
            }
        }
    }

    /// Centre update, then every shape link in order (`src/polygon.rs:218-223`).
    pub fn solve_links(&mut self) {
        self.calc_center();
        for l in &mut self.particle_links {
            l.solve(&mut self.particles);
        }
    }

    /// `Particle::add_force_v2` on every vertex (`src/polygon.rs:225-229`).
    pub fn add_force_v2(&mut self, force: Vector2<f32>) {
        for p in &mut self.particles {
            p.add_force_v2(force);
        }
    }

    /// Mean of the vertex positions: summed from zero in vertex order, then
    /// divided by the count (`src/polygon.rs:231-237`).
    fn calc_center(&mut self) {
        let mut c = Vector2::new(0.0, 0.0);
        for p in &self.particles {
            c += p.pos;
        }
        c /= self.particles.len() as f32;
        self.center = c;
    }
}

/// The contact of vertex `q` (of a polygon with centre `other_center`) with
/// the edge a-b of a polygon with centre `center`, `src/polygon.rs:164-216`.
/// The segment from `q` to `other_center` must cross the edge.  Then the
/// edge moves two thirds of the vertex's depth along the edge's inward
/// normal, shared between a and b in proportion to the intersection's
/// distance from the other end, and the vertex moves to where a ray from it
/// against that normal (length 10000) crosses the old edge.  No crossing of
/// that ray: no contact.
fn edge_contact(
    center: Vector2<f32>,
    a: &Particle,
    b: &Particle,
    q: &Particle,
    other_center: Vector2<f32>,
) -> Option<(Vector2<f32>, Vector2<f32>, Vector2<f32>)> {
    let hit = line_intersection((a.pos, b.pos), (q.pos, other_center))?;
    let along = (b.pos - a.pos).normalize();
    let center_proj = (along.dot(&(center - hit)) / along.dot(&along)) * along;
    let inward = (center - (hit + center_proj)).normalize();
    let to_a = (hit - a.pos).magnitude();
    let to_b = (hit - b.pos).magnitude();
    let edge_len = to_a + to_b;
    let share_a = to_b / edge_len;
    let share_b = to_a / edge_len;
    let depth = hit - q.pos;
    let depth_on_normal = (inward.dot(&depth) / inward.dot(&inward)) * inward;
    let edge_move = depth_on_normal / 3.0 * 2.0;
    let new_a = a.pos - share_a * edge_move;
    let new_b = b.pos - share_b * edge_move;
    let new_q = line_intersection((a.pos, b.pos), (q.pos, q.pos - inward * 10000.0))?;
    Some((new_a, new_b, new_q))
}
