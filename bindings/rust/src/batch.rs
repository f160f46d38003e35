//! Many independent solvers stepped together: one launch sequence (captured
//! in a CUDA graph) per update for every member world.  Results equal the
//! members' own updates.
use std::ffi::CString;
use std::os::raw::c_int;

use crate::error::{check, expect, Error};
use crate::ffi;
use crate::solver::Solver;

/// Owns its member solvers, so no member can be updated on its own while it
/// belongs to the batch.
pub struct Batch {
    raw: *mut ffi::b2d_batch,
    members: Vec<Solver>,
}

unsafe impl Send for Batch {}

impl Batch {
    pub fn new() -> Self {
        let mut raw = std::ptr::null_mut();
        expect(unsafe { ffi::b2d_batch_create(&mut raw) });
        Batch { raw, members: Vec::new() }
    }

    /// Adds a world; returns its index among the members.
    pub fn push(&mut self, solver: Solver) -> Result<usize, Error> {
        check(unsafe { ffi::b2d_batch_add(self.raw, solver.raw()) })?;
        self.members.push(solver);
        Ok(self.members.len() - 1)
    }

    /// Takes member `index` out of the batch (later members move down one).
    pub fn remove(&mut self, index: usize) -> Result<Solver, Error> {
        check(unsafe { ffi::b2d_batch_remove(self.raw, self.members[index].raw()) })?;
        Ok(self.members.remove(index))
    }

    pub fn members(&self) -> &[Solver] {
        &self.members
    }

    /// `Solver::update` on every member.
    pub fn update(&mut self, dt: f32) -> Result<(), Error> {
        for m in &mut self.members {
            m.send_fields()?;
        }
        check(unsafe { ffi::b2d_batch_update(self.raw, dt) })?;
        for m in &mut self.members {
            if m.mirror_on() {
                m.sync_host()?;
            }
        }
        Ok(())
    }

    pub fn synchronize(&self) -> Result<(), Error> {
        check(unsafe { ffi::b2d_batch_synchronize(self.raw) })
    }

    /// One world per launch and no graph: the baseline the batch beats.
    pub fn set_plain(&mut self, on: bool) -> Result<(), Error> {
        check(unsafe { ffi::b2d_batch_set_plain(self.raw, on as c_int) })
    }

    /// Executor tunables for every member (never change results).
    pub fn set_tuning(&mut self, key: &str, value: f64) -> Result<(), Error> {
        let k = CString::new(key).expect("key without NUL");
        check(unsafe { ffi::b2d_batch_set_tuning(self.raw, k.as_ptr(), value) })
    }

    /// Kernel launches per update.
    pub fn launch_count(&self) -> Result<u32, Error> {
        let mut n = 0u32;
        check(unsafe { ffi::b2d_batch_get_launch_count(self.raw, &mut n) })?;
        Ok(n)
    }
}

impl Default for Batch {
    fn default() -> Self {
        Batch::new()
    }
}

impl Drop for Batch {
    fn drop(&mut self) {
        // members return to their own engines, then drop with `members`
        unsafe { ffi::b2d_batch_destroy(self.raw) };
    }
}
