//! Status codes of the C ABI as a Rust error.
use std::ffi::CStr;
use std::fmt;
use std::os::raw::c_int;

use crate::ffi;

/// A failed C ABI call: its status code and the library's message.
#[derive(Debug, Clone, PartialEq, Eq)]
pub struct Error {
    pub code: c_int,
    pub message: String,
}

impl fmt::Display for Error {
    fn fmt(&self, f: &mut fmt::Formatter<'_>) -> fmt::Result {
        write!(f, "bendy2d-gb300 error {}: {}", self.code, self.message)
    }
}

impl std::error::Error for Error {}

/// `Ok(())` for `B2D_OK`, else the error with the calling thread's last
/// message.
pub fn check(code: c_int) -> Result<(), Error> {
    if code == ffi::B2D_OK {
        return Ok(());
    }
    let message = unsafe {
        let p = ffi::b2d_last_error();
        if p.is_null() { String::new() } else { CStr::from_ptr(p).to_string_lossy().into_owned() }
    };
    Err(Error { code, message })
}

/// `check` for calls whose reference counterpart cannot fail: a failure is
/// a panic with the library's message (the reference panics too, lazily,
/// inside `Solver::update`, `src/link.rs:19-21`).
pub(crate) fn expect(code: c_int) {
    if let Err(e) = check(code) {
        panic!("{}", e);
    }
}
