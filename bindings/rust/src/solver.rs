//! `Solver` and `Bounds`, src/solver.rs:13-189, stepped on the GPU.
use std::ffi::CString;
use std::os::raw::{c_int, c_void};

use nalgebra::Vector2;

use crate::circle::Circle;
use crate::error::{check, expect, Error};
use crate::ffi;
use crate::link::{CircleLink, Link, ParticleLink};
use crate::particle::{vec_from_ffi, vec_to_ffi, Particle};
use crate::polygon::Polygon;

/// The box particles, circles and polygons stay in (`src/solver.rs:13-17`).
#[derive(Debug, Copy, Clone)]
pub struct Bounds {
    pub pos: Vector2<f32>,
    pub size: Vector2<f32>,
}

/// Link order of the GPU step (an extension; `Reference` is the default and
/// reproduces the reference bit for bit).
#[derive(Debug, Copy, Clone, PartialEq, Eq)]
pub enum Mode {
    /// The reference's sequential link order, replayed exactly.
    Reference,
    /// Links re-ordered by a colouring at build time: more parallel, same
    /// constraints, different rounding.
    Fast,
}

/// The world: particles, links, circles and polygons, with the public
/// fields of `src/solver.rs:19-31`.  The state lives on the GPU between
/// updates.  After every [`Solver::update`] the particles, circles and
/// polygons are read back into host copies, so the getters return
/// references as the reference's do; [`Solver::set_host_mirror`] turns that
/// read-back off for callers that use [`Solver::read_state`] or the getters
/// only after [`Solver::sync_host`].
pub struct Solver {
    pub gravity: Vector2<f32>,
    pub bounds: Bounds,
    pub bounds_active: bool,
    raw: *mut ffi::b2d_solver,
    particles: Vec<Particle>,
    particle_links: Vec<ParticleLink>,
    circles: Vec<Circle>,
    circle_links: Vec<CircleLink>,
    polygons: Vec<Polygon>,
    mirror: bool,
    // values last passed to the library
    sent_gravity: Vector2<f32>,
    sent_bounds: (Vector2<f32>, Vector2<f32>),
    sent_bounds_active: bool,
}

// A solver is plain data owned by one thread at a time, like the reference's
// (`update` takes `&mut self`); the library keeps no thread affinity.
unsafe impl Send for Solver {}

/// Reads polygon `index` of a solver handle back into the reference's type.
pub(crate) fn read_polygon(raw: *mut ffi::b2d_solver, index: usize) -> Polygon {
    let (mut nv, mut nl, mut is_static, mut center, mut scale) = (0usize, 0usize, 0 as c_int, ffi::b2d_vec2::default(), 0f32);
    expect(unsafe { ffi::b2d_get_polygon_info(raw, index, &mut nv, &mut nl, &mut is_static, &mut center, &mut scale) });
    let mut v = vec![ffi::b2d_particle::default(); nv];
    let mut l = vec![ffi::b2d_link::default(); nl];
    expect(unsafe { ffi::b2d_get_polygon(raw, index, v.as_mut_ptr(), nv, l.as_mut_ptr(), nl) });
    Polygon {
        particles: v.iter().map(Particle::from_ffi).collect(),
        particle_links: l.iter().map(|x| ParticleLink { link: Link::from_ffi(x) }).collect(),
        is_static: is_static != 0,
        center: vec_from_ffi(center),
        scale,
    }
}

impl Solver {
    /// The reference's defaults (`src/solver.rs:34-50`): gravity (0, 98.2),
    /// bounds at the origin of size 100 x 100, one sub-step.
    pub fn new() -> Self {
        let mut raw = std::ptr::null_mut();
        expect(unsafe { ffi::b2d_solver_create(&mut raw) });
        let mut g = ffi::b2d_vec2::default();
        let (mut bp, mut bs) = (ffi::b2d_vec2::default(), ffi::b2d_vec2::default());
        let mut active: c_int = 1;
        unsafe {
            expect(ffi::b2d_get_gravity(raw, &mut g));
            expect(ffi::b2d_get_bounds(raw, &mut bp, &mut bs));
            expect(ffi::b2d_get_bounds_active(raw, &mut active));
        }
        let bounds = Bounds { pos: vec_from_ffi(bp), size: vec_from_ffi(bs) };
        Solver {
            gravity: vec_from_ffi(g),
            bounds,
            bounds_active: active != 0,
            raw,
            particles: Vec::new(),
            particle_links: Vec::new(),
            circles: Vec::new(),
            circle_links: Vec::new(),
            polygons: Vec::new(),
            mirror: true,
            sent_gravity: vec_from_ffi(g),
            sent_bounds: (bounds.pos, bounds.size),
            sent_bounds_active: active != 0,
        }
    }

    /// `src/solver.rs:52-54`.
    pub fn add_particle(&mut self, pos: Vector2<f32>) {
        expect(unsafe { ffi::b2d_add_particle(self.raw, pos.x, pos.y) });
        self.particles.push(Particle::new(pos));
    }

    /// `src/solver.rs:55-57`.
    pub fn add_circle(&mut self, circle: Circle) {
        let c = circle.to_ffi();
        expect(unsafe { ffi::b2d_add_circle(self.raw, &c) });
        self.circles.push(circle);
    }

    /// `src/solver.rs:58-60`.
    pub fn add_polygon(&mut self, polygon: Polygon) {
        let v: Vec<ffi::b2d_particle> = polygon.particles.iter().map(|p| p.to_ffi()).collect();
        let l: Vec<ffi::b2d_link> = polygon.particle_links.iter().map(|x| x.link.to_ffi()).collect();
        expect(unsafe {
            ffi::b2d_add_polygon(
                self.raw,
                v.len(),
                v.as_ptr(),
                l.len(),
                l.as_ptr(),
                polygon.is_static as c_int,
                vec_to_ffi(polygon.center),
                polygon.scale,
            )
        });
        self.polygons.push(polygon);
    }

    /// `src/solver.rs:62-64`; the indices are checked at the next update.
    pub fn add_particle_link(&mut self, link: ParticleLink) {
        let l = link.link;
        expect(unsafe { ffi::b2d_add_particle_link(self.raw, l.particle_a as u64, l.particle_b as u64, l.target_distance) });
        self.particle_links.push(link);
    }

    /// `src/solver.rs:65-67`; the indices are checked at the next update.
    pub fn add_circle_link(&mut self, link: CircleLink) {
        let l = link.link;
        expect(unsafe { ffi::b2d_add_circle_link(self.raw, l.particle_a as u64, l.particle_b as u64, l.target_distance) });
        self.circle_links.push(link);
    }

    pub fn get_particle_len(&self) -> usize {
        self.particles.len()
    }
    pub fn get_circles_len(&self) -> usize {
        self.circles.len()
    }
    pub fn get_polygons_len(&self) -> usize {
        self.polygons.len()
    }
    pub fn get_particle_links(&self) -> &Vec<ParticleLink> {
        &self.particle_links
    }
    pub fn get_circle_links(&self) -> &Vec<CircleLink> {
        &self.circle_links
    }
    pub fn get_particles(&self) -> &Vec<Particle> {
        &self.particles
    }
    pub fn get_circles(&self) -> &Vec<Circle> {
        &self.circles
    }
    pub fn get_polygons(&self) -> &Vec<Polygon> {
        &self.polygons
    }
    pub fn get_particle(&self, index: usize) -> Option<&Particle> {
        self.particles.get(index)
    }
    pub fn get_circle(&self, index: usize) -> Option<&Circle> {
        self.circles.get(index)
    }
    pub fn get_polygon(&self, index: usize) -> Option<&Polygon> {
        self.polygons.get(index)
    }

    /// One `Solver::update` (`src/solver.rs:106-116`) on the GPU.  Panics
    /// where the reference panics: a particle, circle or polygon link that
    /// breaks `a < b < len` (`src/link.rs:19-21`, `:37-39`); and on a CUDA or
    /// device error, which has no counterpart there.
    pub fn update(&mut self, dt: f32) {
        if let Err(e) = self.try_update(dt) {
            panic!("{}", e);
        }
    }

    /// `update`, returning the library's status instead of panicking.
    pub fn try_update(&mut self, dt: f32) -> Result<(), Error> {
        self.send_fields()?;
        check(unsafe { ffi::b2d_update(self.raw, dt) })?;
        if self.mirror {
            self.sync_host()?;
        }
        Ok(())
    }

    /// Passes changed public fields to the library.
    pub(crate) fn send_fields(&mut self) -> Result<(), Error> {
        if self.gravity != self.sent_gravity {
            check(unsafe { ffi::b2d_set_gravity(self.raw, self.gravity.x, self.gravity.y) })?;
            self.sent_gravity = self.gravity;
        }
        if (self.bounds.pos, self.bounds.size) != self.sent_bounds {
            let b = self.bounds;
            check(unsafe { ffi::b2d_set_bounds(self.raw, b.pos.x, b.pos.y, b.size.x, b.size.y) })?;
            self.sent_bounds = (b.pos, b.size);
        }
        if self.bounds_active != self.sent_bounds_active {
            check(unsafe { ffi::b2d_set_bounds_active(self.raw, self.bounds_active as c_int) })?;
            self.sent_bounds_active = self.bounds_active;
        }
        Ok(())
    }

    /// Reads the particles, circles and polygons back from the GPU into the
    /// host copies the getters return.
    pub fn sync_host(&mut self) -> Result<(), Error> {
        let n = self.particles.len();
        let mut p = vec![ffi::b2d_particle::default(); n];
        check(unsafe { ffi::b2d_get_particles(self.raw, p.as_mut_ptr(), n) })?;
        self.particles = p.iter().map(Particle::from_ffi).collect();
        let nc = self.circles.len();
        let mut c = vec![ffi::b2d_circle::default(); nc];
        check(unsafe { ffi::b2d_get_circles(self.raw, c.as_mut_ptr(), nc) })?;
        self.circles = c.iter().map(Circle::from_ffi).collect();
        for i in 0..self.polygons.len() {
            self.polygons[i] = read_polygon(self.raw, i);
        }
        Ok(())
    }

    /// Whether `update` reads the state back for the getters (default on).
    pub fn set_host_mirror(&mut self, on: bool) {
        self.mirror = on;
    }

    // ---- extensions (absent or private in the reference) ------------------

    /// Sub-steps per update (the reference's private `sub_steps`, 1).
    pub fn set_sub_steps(&mut self, n: u32) {
        expect(unsafe { ffi::b2d_set_sub_steps(self.raw, n) });
    }
    /// Passes over the links per sub-step (1 reproduces the reference).
    pub fn set_link_iters(&mut self, n: u32) {
        expect(unsafe { ffi::b2d_set_link_iters(self.raw, n) });
    }
    pub fn set_mode(&mut self, mode: Mode) {
        let m = match mode {
            Mode::Reference => ffi::B2D_MODE_REFERENCE,
            Mode::Fast => ffi::B2D_MODE_FAST,
        };
        expect(unsafe { ffi::b2d_set_mode(self.raw, m) });
    }
    /// Particle collisions (`ffi::B2D_COLLIDE_*` flags) with particle radius
    /// and grid cell size; 0 reproduces the reference.
    pub fn set_collision(&mut self, flags: u32, particle_radius: f32, grid_cell: f32) {
        expect(unsafe { ffi::b2d_set_collision(self.raw, flags, particle_radius, grid_cell) });
    }
    /// A static circle is not integrated.
    pub fn set_circle_static(&mut self, index: usize, is_static: bool) -> Result<(), Error> {
        check(unsafe { ffi::b2d_set_circle_static(self.raw, index, is_static as c_int) })
    }
    /// Particle links with per-link stiffness (1 reproduces the reference).
    pub fn add_particle_links_stiff(&mut self, links: &[ParticleLink], stiffness: &[f32]) -> Result<(), Error> {
        assert_eq!(links.len(), stiffness.len());
        let a: Vec<u64> = links.iter().map(|l| l.link.particle_a as u64).collect();
        let b: Vec<u64> = links.iter().map(|l| l.link.particle_b as u64).collect();
        let t: Vec<f32> = links.iter().map(|l| l.link.target_distance).collect();
        check(unsafe { ffi::b2d_add_particle_links(self.raw, links.len(), a.as_ptr(), b.as_ptr(), t.as_ptr(), stiffness.as_ptr()) })?;
        self.particle_links.extend_from_slice(links);
        Ok(())
    }
    /// Particles with an initial previous position (a velocity), in bulk:
    /// `pos_xy` and `prev_xy` hold x, y pairs.
    pub fn add_particles(&mut self, pos_xy: &[f32], prev_xy: Option<&[f32]>) -> Result<(), Error> {
        assert!(pos_xy.len() % 2 == 0);
        let n = pos_xy.len() / 2;
        if let Some(q) = prev_xy {
            assert_eq!(q.len(), pos_xy.len());
        }
        let qp = prev_xy.map_or(std::ptr::null(), |q| q.as_ptr());
        check(unsafe { ffi::b2d_add_particles(self.raw, n, pos_xy.as_ptr(), qp) })?;
        for i in 0..n {
            let mut p = Particle::new(Vector2::new(pos_xy[2 * i], pos_xy[2 * i + 1]));
            if let Some(q) = prev_xy {
                p.prev_pos = Vector2::new(q[2 * i], q[2 * i + 1]);
            }
            self.particles.push(p);
        }
        Ok(())
    }
    /// Executor tunables (never change results); see `include/bendy2d.h`.
    pub fn set_tuning(&mut self, key: &str, value: f64) -> Result<(), Error> {
        let k = CString::new(key).expect("key without NUL");
        check(unsafe { ffi::b2d_set_tuning(self.raw, k.as_ptr(), value) })
    }
    /// Positions and previous positions (x, y pairs, insertion order) straight
    /// from the GPU into `pos_xy` / `prev_xy` (each 2 x particle count).
    pub fn read_state(&self, pos_xy: &mut [f32], prev_xy: &mut [f32]) -> Result<(), Error> {
        let n = 2 * self.particles.len();
        assert!(pos_xy.len() >= n && prev_xy.len() >= n);
        check(unsafe { ffi::b2d_read_state(self.raw, pos_xy.as_mut_ptr(), prev_xy.as_mut_ptr()) })
    }
    /// Replaces the GPU state of every particle.
    pub fn write_state(&mut self, pos_xy: &[f32], prev_xy: &[f32]) -> Result<(), Error> {
        let n = 2 * self.particles.len();
        assert!(pos_xy.len() >= n && prev_xy.len() >= n);
        check(unsafe { ffi::b2d_write_state(self.raw, pos_xy.as_ptr(), prev_xy.as_ptr()) })?;
        for i in 0..self.particles.len() {
            self.particles[i].pos = Vector2::new(pos_xy[2 * i], pos_xy[2 * i + 1]);
            self.particles[i].prev_pos = Vector2::new(prev_xy[2 * i], prev_xy[2 * i + 1]);
        }
        Ok(())
    }
    /// The CUDA stream updates are issued on (null: the library's own).
    ///
    /// # Safety
    /// `stream` must be a valid CUDA stream of the current device for as long
    /// as the solver uses it.
    pub unsafe fn set_stream(&mut self, stream: *mut c_void) -> Result<(), Error> {
        check(ffi::b2d_set_stream(self.raw, stream))
    }
    pub fn synchronize(&self) -> Result<(), Error> {
        check(unsafe { ffi::b2d_synchronize(self.raw) })
    }
    pub fn plan_stats(&self) -> Result<ffi::b2d_plan_stats, Error> {
        let mut s = ffi::b2d_plan_stats::default();
        check(unsafe { ffi::b2d_get_plan_stats(self.raw, &mut s) })?;
        Ok(s)
    }

    pub(crate) fn raw(&self) -> *mut ffi::b2d_solver {
        self.raw
    }

    pub(crate) fn mirror_on(&self) -> bool {
        self.mirror
    }

    /// Rebuilds every host copy from the library (after the world behind the
    /// handle was replaced, e.g. by a finished serving request).
    pub(crate) fn reload(&mut self) -> Result<(), Error> {
        let len = |f: unsafe extern "C" fn(*mut ffi::b2d_solver, *mut usize) -> c_int| -> Result<usize, Error> {
            let mut n = 0usize;
            check(unsafe { f(self.raw, &mut n) })?;
            Ok(n)
        };
        let (np, nc, ng) = (len(ffi::b2d_get_particle_len)?, len(ffi::b2d_get_circles_len)?, len(ffi::b2d_get_polygons_len)?);
        let (npl, ncl) = (len(ffi::b2d_get_particle_links_len)?, len(ffi::b2d_get_circle_links_len)?);
        let mut l = vec![ffi::b2d_link::default(); npl];
        check(unsafe { ffi::b2d_get_particle_links(self.raw, l.as_mut_ptr(), npl) })?;
        self.particle_links = l.iter().map(|x| ParticleLink { link: Link::from_ffi(x) }).collect();
        let mut l = vec![ffi::b2d_link::default(); ncl];
        check(unsafe { ffi::b2d_get_circle_links(self.raw, l.as_mut_ptr(), ncl) })?;
        self.circle_links = l.iter().map(|x| CircleLink { link: Link::from_ffi(x) }).collect();
        self.particles = vec![Particle::new(Vector2::zeros()); np];
        self.circles = vec![Circle { point: Particle::new(Vector2::zeros()), radius: 0.0 }; nc];
        self.polygons = (0..ng).map(|i| read_polygon(self.raw, i)).collect();
        self.sync_host()?;
        let mut g = ffi::b2d_vec2::default();
        let (mut bp, mut bs) = (ffi::b2d_vec2::default(), ffi::b2d_vec2::default());
        let mut active: c_int = 1;
        unsafe {
            check(ffi::b2d_get_gravity(self.raw, &mut g))?;
            check(ffi::b2d_get_bounds(self.raw, &mut bp, &mut bs))?;
            check(ffi::b2d_get_bounds_active(self.raw, &mut active))?;
        }
        self.gravity = vec_from_ffi(g);
        self.bounds = Bounds { pos: vec_from_ffi(bp), size: vec_from_ffi(bs) };
        self.bounds_active = active != 0;
        self.sent_gravity = self.gravity;
        self.sent_bounds = (self.bounds.pos, self.bounds.size);
        self.sent_bounds_active = self.bounds_active;
        Ok(())
    }
}

impl Default for Solver {
    fn default() -> Self {
        Solver::new()
    }
}

/// `#[derive(Clone)]` of the reference (`src/solver.rs:19`): an independent
/// world with the same state.
impl Clone for Solver {
    fn clone(&self) -> Self {
        let mut raw = std::ptr::null_mut();
        expect(unsafe { ffi::b2d_solver_clone(self.raw, &mut raw) });
        Solver {
            gravity: self.gravity,
            bounds: self.bounds,
            bounds_active: self.bounds_active,
            raw,
            particles: self.particles.clone(),
            particle_links: self.particle_links.clone(),
            circles: self.circles.clone(),
            circle_links: self.circle_links.clone(),
            polygons: self.polygons.clone(),
            mirror: self.mirror,
            sent_gravity: self.sent_gravity,
            sent_bounds: self.sent_bounds,
            sent_bounds_active: self.sent_bounds_active,
        }
    }
}

impl std::fmt::Debug for Solver {
    fn fmt(&self, f: &mut std::fmt::Formatter<'_>) -> std::fmt::Result {
        f.debug_struct("Solver")
            .field("gravity", &self.gravity)
            .field("bounds", &self.bounds)
            .field("bounds_active", &self.bounds_active)
            .field("particles", &self.particles.len())
            .field("particle_links", &self.particle_links.len())
            .field("circles", &self.circles.len())
            .field("circle_links", &self.circle_links.len())
            .field("polygons", &self.polygons.len())
            .finish()
    }
}

impl Drop for Solver {
    fn drop(&mut self) {
        unsafe { ffi::b2d_solver_destroy(self.raw) };
    }
}
