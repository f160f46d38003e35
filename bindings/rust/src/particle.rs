//! `Particle`, src/particle.rs:4-59.
use nalgebra::Vector2;

use crate::ffi;
use crate::solver::Bounds;

/// Verlet particle: position and previous position (public, as in the
/// reference) and an acceleration that only forces change (private, as in
/// the reference).
#[derive(Debug, Copy, Clone)]
pub struct Particle {
    pub pos: Vector2<f32>,
    pub prev_pos: Vector2<f32>,
    acc: Vector2<f32>,
}

/// One axis of `Particle::solve_bounds`: below `lo` or else above `hi`, the
/// particle is put on the bound and its Verlet velocity reflected.
fn reflect_axis(pos: &mut f32, prev: &mut f32, lo: f32, hi: f32) {
    if *pos < lo {
        let velocity = *prev - *pos;
        *prev = lo - velocity;
        *pos = lo;
    } else if *pos > hi {
        let velocity = *prev - *pos;
        *prev = hi - velocity;
        *pos = hi;
    }
}

impl Particle {
    /// At rest at `pos` (`src/particle.rs:12-18`).
    pub fn new(pos: Vector2<f32>) -> Self {
        Particle { pos, prev_pos: pos, acc: Vector2::zeros() }
    }

    /// One Verlet step, `src/particle.rs:20-25`: the new position is
    /// `(pos + velocity) + (acc * dt) * dt` in f32, and the acceleration is
    /// used up.
    pub fn update(&mut self, dt: f32) {
        let velocity = self.pos - self.prev_pos;
        let next = self.pos + velocity + self.acc * dt * dt;
        self.prev_pos = self.pos;
        self.pos = next;
        self.acc = Vector2::zeros();
    }

    /// Keeps the particle inside `bounds`, `src/particle.rs:27-46`.
    pub fn solve_bounds(&mut self, bounds: Bounds) {
        reflect_axis(&mut self.pos.x, &mut self.prev_pos.x, bounds.pos.x, bounds.pos.x + bounds.size.x);
        reflect_axis(&mut self.pos.y, &mut self.prev_pos.y, bounds.pos.y, bounds.pos.y + bounds.size.y);
    }

    /// `src/particle.rs:48-50`.
    pub fn add_force(&mut self, force_x: f32, force_y: f32) {
        self.acc += Vector2::new(force_x, force_y);
    }

    /// `src/particle.rs:52-54`.
    pub fn add_force_v2(&mut self, force: Vector2<f32>) {
        self.acc += force;
    }

    /// A force of magnitude `force` along the unit vector towards `point`
    /// (`src/particle.rs:56-59`).
    pub fn add_force_towards(&mut self, point: Vector2<f32>, force: f32) {
        let direction = (point - self.pos).normalize();
        self.acc += direction * force;
    }

    pub(crate) fn to_ffi(&self) -> ffi::b2d_particle {
        ffi::b2d_particle { pos: vec_to_ffi(self.pos), prev_pos: vec_to_ffi(self.prev_pos), acc: vec_to_ffi(self.acc) }
    }

    pub(crate) fn from_ffi(p: &ffi::b2d_particle) -> Self {
        Particle { pos: vec_from_ffi(p.pos), prev_pos: vec_from_ffi(p.prev_pos), acc: vec_from_ffi(p.acc) }
    }
}

pub(crate) fn vec_to_ffi(v: Vector2<f32>) -> ffi::b2d_vec2 {
    ffi::b2d_vec2 { x: v.x, y: v.y }
}

pub(crate) fn vec_from_ffi(v: ffi::b2d_vec2) -> Vector2<f32> {
    Vector2::new(v.x, v.y)
}
