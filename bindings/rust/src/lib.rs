//! bendy2d on a GB300 GPU.
//!
//! The same modules, types and methods as the bendy2d 0.0.1 crate
//! (`src/lib.rs:1-6`: `circle`, `common`, `link`, `particle`, `polygon`,
//! `solver`), so code written against bendy2d keeps compiling.  The state of
//! a [`solver::Solver`] lives on the GPU between updates and
//! [`solver::Solver::update`] runs there, through the C ABI of
//! libbendy2d_gb300 (`include/bendy2d.h`), with results bit-identical to the
//! reference's sequential step.  The per-object methods of the value types
//! (`Particle::update`, `Circle::solve_circle`, `ParticleLink::solve`, ...)
//! run on the host, as in the reference.
//!
//! Additions: [`batch::Batch`] (many solvers stepped by one launch sequence),
//! [`server::Server`] (continuous batching of solve requests), the raw
//! [`ffi`] declarations and the extension setters on `Solver`.
pub mod circle;
pub mod common;
pub mod link;
pub mod particle;
pub mod polygon;
pub mod solver;

pub mod batch;
pub mod error;
pub mod ffi;
pub mod server;
