//! A 32 x 32 cloth of particles and links falling onto a static floor
//! polygon, stepped on the GPU exactly as bendy2d steps it on the CPU.
use bendy2d::link::{Link, ParticleLink};
use bendy2d::polygon::Polygon;
use bendy2d::solver::Solver;
use nalgebra::Vector2;

fn main() {
    let mut s = Solver::new();
    s.gravity = Vector2::new(0.0, -9.81);
    let n = 32;
    for y in 0..n {
        for x in 0..n {
            s.add_particle(Vector2::new(30.0 + x as f32, 60.0 + y as f32));
        }
    }
    let id = |x: usize, y: usize| y * n + x;
    for y in 0..n {
        for x in 0..n {
            if x + 1 < n {
                s.add_particle_link(ParticleLink { link: Link { particle_a: id(x, y), particle_b: id(x + 1, y), target_distance: 1.0 } });
            }
            if y + 1 < n {
                s.add_particle_link(ParticleLink { link: Link { particle_a: id(x, y), particle_b: id(x, y + 1), target_distance: 1.0 } });
            }
        }
    }
    let floor = vec![Vector2::new(0.0, 0.0), Vector2::new(100.0, 0.0), Vector2::new(100.0, 10.0), Vector2::new(0.0, 10.0)];
    s.add_polygon(Polygon::new(floor, true));
    for _ in 0..600 {
        s.update(1.0 / 60.0);
    }
    println!("particle 0 at {:?}", s.get_particle(0).unwrap().pos);
}
