//! `Link`, `ParticleLink`, `CircleLink`, src/link.rs:4-48.
use crate::circle::Circle;
use crate::ffi;
use crate::particle::Particle;

/// A distance constraint between elements `particle_a < particle_b`
/// (`src/link.rs:4-10`).  `Solver::update` panics when a link breaks
/// `particle_a < particle_b < len`, as the reference does.
#[derive(Debug, Copy, Clone)]
pub struct Link {
    pub particle_a: usize,
    pub particle_b: usize,
    pub target_distance: f32,
}

/// A link between two solver particles (`src/link.rs:12-15`).
#[derive(Debug, Copy, Clone)]
pub struct ParticleLink {
    pub link: Link,
}

/// A link between two circles (`src/link.rs:30-33`).
#[derive(Debug, Copy, Clone)]
pub struct CircleLink {
    pub link: Link,
}

/// The two elements of a link, mutably; panics unless `a < b < len`, the
/// condition under which the reference's `split_at_mut` indexing succeeds.
fn pair<T>(v: &mut [T], a: usize, b: usize) -> (&mut T, &mut T) {
    assert!(a < b && b < v.len(), "link ({}, {}) needs a < b < {}", a, b, v.len());
    let (lo, hi) = v.split_at_mut(b);
    (&mut lo[a], &mut hi[0])
}

impl ParticleLink {
    /// Moves both particles half of the length error each, along the unit
    /// vector between them (`src/link.rs:18-27`).
    pub fn solve(&mut self, particles: &mut Vec<Particle>) {
        let l = self.link;
        let (a, b) = pair(particles, l.particle_a, l.particle_b);
        let d = a.pos - b.pos;
        let dist = d.magnitude();
        let n = d.normalize();
        a.pos -= n * (dist - l.target_distance) * 0.5;
        b.pos += n * (dist - l.target_distance) * 0.5;
    }
}

impl CircleLink {
    /// Like `ParticleLink::solve`, with the correction split by the squared
    /// radii: each circle moves by the other's share (`src/link.rs:36-48`).
    pub fn solve(&mut self, circles: &mut Vec<Circle>) {
        let l = self.link;
        let (a, b) = pair(circles, l.particle_a, l.particle_b);
        let d = a.point.pos - b.point.pos;
        let dist = d.magnitude();
        let n = d.normalize();
        let ra2 = a.radius * a.radius;
        let rb2 = b.radius * b.radius;
        let scale = 1.0 / (ra2 + rb2);
        a.point.pos -= n * (dist - l.target_distance) * scale * rb2;
        b.point.pos += n * (dist - l.target_distance) * scale * ra2;
    }
}

impl Link {
    pub(crate) fn to_ffi(&self) -> ffi::b2d_link {
        ffi::b2d_link {
            particle_a: self.particle_a as u64,
            particle_b: self.particle_b as u64,
            target_distance: self.target_distance,
            stiffness: 1.0,
        }
    }

    pub(crate) fn from_ffi(l: &ffi::b2d_link) -> Self {
        Link { particle_a: l.particle_a as usize, particle_b: l.particle_b as usize, target_distance: l.target_distance }
    }
}
