//! `Circle`, src/circle.rs:4-45.
use crate::ffi;
use crate::particle::Particle;
use crate::solver::Bounds;

/// A rigid disc: a Verlet particle and a radius (`src/circle.rs:4-8`).
#[derive(Debug, Copy, Clone)]
pub struct Circle {
    pub point: Particle,
    pub radius: f32,
}

/// One axis of `Circle::solve_bounds`: the bounds shrunk by the radius, then
/// the particle rule (below `lo`, else above `hi`: put on the bound and
/// reflect the Verlet velocity).
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

impl Circle {
    /// Keeps the whole disc inside `bounds` (`src/circle.rs:11-30`).
    pub fn solve_bounds(&mut self, bounds: Bounds) {
        let r = self.radius;
        let p = &mut self.point;
        reflect_axis(&mut p.pos.x, &mut p.prev_pos.x, bounds.pos.x + r, bounds.pos.x + bounds.size.x - r);
        reflect_axis(&mut p.pos.y, &mut p.prev_pos.y, bounds.pos.y + r, bounds.pos.y + bounds.size.y - r);
    }

    /// Pushes two overlapping discs apart along the line between their
    /// centres, each by the other's share of the squared radii
    /// (`src/circle.rs:32-45`).
    pub fn solve_circle(&mut self, circle: &mut Circle) {
        let d = self.point.pos - circle.point.pos;
        let d2 = d.norm_squared();
        let reach = self.radius + circle.radius;
        if d2 < reach * reach {
            let n = d.normalize();
            let overlap = reach - d2.sqrt();
            let r_self2 = self.radius * self.radius;
            let r_other2 = circle.radius * circle.radius;
            let scale = 1.0 / (r_self2 + r_other2);
            self.point.pos += n * scale * overlap * r_other2;
            circle.point.pos -= n * scale * overlap * r_self2;
        }
    }

    pub(crate) fn to_ffi(&self) -> ffi::b2d_circle {
        ffi::b2d_circle { point: self.point.to_ffi(), radius: self.radius, is_static: 0 }
    }

    pub(crate) fn from_ffi(c: &ffi::b2d_circle) -> Self {
        Circle { point: Particle::from_ffi(&c.point), radius: c.radius }
    }
}
