//! GB300 backend of qvnt (feature `gb300`): a register whose state vector lives only in GPU
//! memory, driven through the engine's C ABI (`ffi`).  Circuits are still built with qvnt's own
//! `op::` constructors, `.c()` and `.dgr()`; `GpuReg::apply` lowers the `MultiOp` / `SingleOp` to
//! the engine's gate records (`Lower`) and runs them on the device.  There is no CPU fallback:
//! user types that implement `Applicable` with their own Rust code do not implement `Lower` and
//! cannot be applied to a `GpuReg`.
pub mod ffi;
mod reg;

use std::ffi::CStr;

pub use reg::{GpuContext, GpuReg};

/// An operator the engine can run: writes its gate records in application order.
pub trait Lower {
    fn lower_into(&self, out: &mut Vec<ffi::qvnt_gate>);

    fn lower(&self) -> Vec<ffi::qvnt_gate> {
        let mut v = Vec::new();
        self.lower_into(&mut v);
        v
    }
}

/// A failed engine call: the `QVNT_ERR_*` status and the engine's message.
#[derive(Debug, Clone, PartialEq)]
pub struct GpuError {
    pub status: i32,
    pub message: String,
}

impl std::fmt::Display for GpuError {
    fn fmt(&self, f: &mut std::fmt::Formatter<'_>) -> std::fmt::Result {
        write!(f, "qvnt_gb300 status {}: {}", self.status, self.message)
    }
}

impl std::error::Error for GpuError {}

pub(crate) fn check(status: std::os::raw::c_int) -> Result<(), GpuError> {
    if status == ffi::QVNT_OK {
        return Ok(());
    }
    let message = unsafe {
        let p = ffi::qvnt_last_error();
        if p.is_null() {
            String::new()
        } else {
            CStr::from_ptr(p).to_string_lossy().into_owned()
        }
    };
    Err(GpuError { status, message })
}
