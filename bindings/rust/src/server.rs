//! Continuous batching of world-solve requests.  A request is a copy of a
//! solver's world plus a number of `Solver::update` calls; a worker thread
//! admits queued requests first come first served while the resident
//! worlds fit the device-memory budget, steps every resident world once per
//! tick in one launch sequence and retires finished requests.  Results are
//! bit-identical to running each request alone.
use std::os::raw::c_int;

use crate::error::{check, expect, Error};
use crate::ffi;
use crate::solver::Solver;

#[derive(Debug, Copy, Clone, PartialEq, Eq)]
pub enum RequestState {
    Queued,
    Running,
    Done,
    Failed,
    Cancelled,
}

/// Completion time of a taken request.
#[derive(Debug, Copy, Clone, PartialEq)]
pub struct Latency {
    /// submit to completion, seconds
    pub total_s: f64,
    /// time spent queued before admission, seconds
    pub queued_s: f64,
}

pub struct Server {
    raw: *mut ffi::b2d_server,
}

// the library synchronises every server call internally
unsafe impl Send for Server {}
unsafe impl Sync for Server {}

impl Server {
    /// A stopped server admitting worlds while their device bytes stay
    /// within `budget_bytes`.
    pub fn new(budget_bytes: u64) -> Self {
        let mut raw = std::ptr::null_mut();
        expect(unsafe { ffi::b2d_server_create(budget_bytes, &mut raw) });
        Server { raw }
    }

    pub fn start(&self) -> Result<(), Error> {
        check(unsafe { ffi::b2d_server_start(self.raw) })
    }

    pub fn stop(&self) -> Result<(), Error> {
        check(unsafe { ffi::b2d_server_stop(self.raw) })
    }

    /// Queues a copy of `world` for `steps` updates of `dt`.  A world that
    /// alone exceeds the budget is refused (`ffi::B2D_ERR_BUDGET`).
    pub fn submit(&self, world: &mut Solver, steps: u32, dt: f32) -> Result<u64, Error> {
        world.send_fields()?;
        let mut id = 0u64;
        check(unsafe { ffi::b2d_server_submit(self.raw, world.raw(), steps, dt, &mut id) })?;
        Ok(id)
    }

    pub fn poll(&self, id: u64) -> Result<RequestState, Error> {
        let mut st: c_int = 0;
        check(unsafe { ffi::b2d_server_poll(self.raw, id, &mut st) })?;
        Ok(match st {
            ffi::B2D_SERVE_QUEUED => RequestState::Queued,
            ffi::B2D_SERVE_RUNNING => RequestState::Running,
            ffi::B2D_SERVE_DONE => RequestState::Done,
            ffi::B2D_SERVE_CANCELLED => RequestState::Cancelled,
            _ => RequestState::Failed,
        })
    }

    /// Drops a request: a queued one at once, a running one when the tick in
    /// flight ends.  `ffi::B2D_ERR_STATE` once it has finished.
    pub fn cancel(&self, id: u64) -> Result<(), Error> {
        check(unsafe { ffi::b2d_server_cancel(self.raw, id) })
    }

    /// Admission also keeps the resident solver particles at or below `n`
    /// (0: no limit), so ticks stay short under overload.
    pub fn set_max_resident_particles(&self, n: u64) -> Result<(), Error> {
        check(unsafe { ffi::b2d_server_set_max_resident_particles(self.raw, n) })
    }

    /// Moves a finished request's world into `dst` (replacing its contents)
    /// and releases the request.
    pub fn take(&self, id: u64, dst: &mut Solver) -> Result<Latency, Error> {
        let (mut total, mut queued) = (0f64, 0f64);
        check(unsafe { ffi::b2d_server_take(self.raw, id, dst.raw(), &mut total, &mut queued) })?;
        dst.reload()?;
        Ok(Latency { total_s: total, queued_s: queued })
    }

    /// Requests finished (done, failed or cancelled) since the last call.
    pub fn finished(&self) -> Result<Vec<u64>, Error> {
        let mut out = Vec::new();
        let mut buf = [0u64; 256];
        loop {
            let mut n = 0usize;
            check(unsafe { ffi::b2d_server_finished(self.raw, buf.as_mut_ptr(), buf.len(), &mut n) })?;
            out.extend_from_slice(&buf[..n]);
            if n < buf.len() {
                return Ok(out);
            }
        }
    }

    pub fn stats(&self) -> Result<ffi::b2d_server_stats, Error> {
        let mut s = ffi::b2d_server_stats::default();
        check(unsafe { ffi::b2d_server_get_stats(self.raw, &mut s) })?;
        Ok(s)
    }
}

impl Drop for Server {
    fn drop(&mut self) {
        unsafe { ffi::b2d_server_destroy(self.raw) };
    }
}
