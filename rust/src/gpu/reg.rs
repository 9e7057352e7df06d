//! `GpuReg`: qvnt's `QReg` (src/register/quant.rs) with its state vector in GPU memory.  The same
//! public surface (`new`, `with_state`, `num`, `apply`, `measure_mask`, `measure`,
//! `get_probabilities`, `get_absolute`, `get_polar`, `reset`, `reset_by_mask`, `*` for the tensor
//! product, `Clone`); each call is one engine entry point.  Errors the engine reports (an invalid
//! mask, a CUDA failure) panic with its message, as qvnt's `expect`s do; the `try_` forms return
//! them instead.
use std::{ops::Mul, ptr, sync::Arc};

use rand::Rng;

use super::{check, ffi, GpuError, Lower};
use crate::{math::types::*, operator::Applicable, register::CReg};

/// One CUDA device (`qvnt_ctx`): stands in for qvnt's global Rayon pool (src/threads.rs).
pub struct GpuContext {
    h: *mut ffi::qvnt_ctx,
}

// The engine serialises the context's shared state (its plugin register) itself; registers own
// their CUDA streams.
unsafe impl Send for GpuContext {}
unsafe impl Sync for GpuContext {}

impl GpuContext {
    pub fn new(device: i32) -> Result<Arc<Self>, GpuError> {
        let mut h = ptr::null_mut();
        check(unsafe { ffi::qvnt_ctx_create(device, &mut h) })?;
        Ok(Arc::new(GpuContext { h }))
    }

    /// Engine of the registers this context makes and of `apply_host` (default: the f64 tensor-core
    /// engine `ffi::ENGINE_TENSOR64`; the one-pass-per-gate IEEE path is `ENGINE_PLAIN`).
    pub fn set_engine(&self, engine: i32) -> Result<(), GpuError> {
        check(unsafe { ffi::qvnt_ctx_set_engine(self.h, engine) })
    }

    /// `Applicable::apply(psi_i, psi_o)` (src/operator/applicable.rs) on host buffers: the state
    /// goes to the device, through the gates and back.
    pub fn apply_host<Op: Lower>(&self, op: &Op, psi_i: &[C], psi_o: &mut Vec<C>) -> Result<(), GpuError> {
        let gates = op.lower();
        psi_o.resize(psi_i.len(), C::new(0.0, 0.0));
        check(unsafe {
            ffi::qvnt_apply_host(
                self.h,
                gates.as_ptr(),
                gates.len(),
                psi_i.as_ptr() as *const f64,
                psi_o.as_mut_ptr() as *mut f64,
                psi_i.len() as u64,
            )
        })
    }
}

impl Drop for GpuContext {
    fn drop(&mut self) {
        unsafe { ffi::qvnt_ctx_destroy(self.h) };
    }
}

pub struct GpuReg {
    h: *mut ffi::qvnt_reg,
    q_num: N,
    ctx: Arc<GpuContext>,
}

unsafe impl Send for GpuReg {}

fn expect_ok(r: Result<(), GpuError>) {
    if let Err(e) = r {
        panic!("{}", e);
    }
}

impl GpuReg {
    /// `QReg::new(q_num)`: |0> on `max(2^q_num, 8)` amplitudes.
    pub fn new(ctx: &Arc<GpuContext>, q_num: N) -> Self {
        Self::with_state(ctx, q_num, 0)
    }

    /// `QReg::with_state(q_num, state)`: the basis state `state & (2^q_num - 1)`.
    pub fn with_state(ctx: &Arc<GpuContext>, q_num: N, state: N) -> Self {
        let mut h = ptr::null_mut();
        expect_ok(check(unsafe { ffi::qvnt_reg_create(ctx.h, q_num as u32, state as u64, &mut h) }));
        GpuReg { h, q_num, ctx: ctx.clone() }
    }

    pub fn num(&self) -> N {
        self.q_num
    }

    /// `QReg::apply(&op)`: runs the lowered gates on the device, in queue order.
    pub fn apply<Op: Applicable + Lower>(&mut self, op: &Op) {
        expect_ok(self.try_apply(op));
    }

    pub fn try_apply<Op: Lower>(&mut self, op: &Op) -> Result<(), GpuError> {
        let gates = op.lower();
        check(unsafe { ffi::qvnt_reg_apply(self.h, gates.as_ptr(), gates.len()) })
    }

    /// `QReg::measure_mask(mask)`: the uniform draw qvnt's `WeightedIndex` makes from
    /// `thread_rng` is drawn here and passed to the device; the state collapses unnormalised.
    pub fn measure_mask(&mut self, mask: N) -> CReg {
        let u01: f64 = rand::thread_rng().gen();
        self.measure_mask_with(mask, u01)
    }

    /// `measure_mask` with an injected draw in [0, 1).
    pub fn measure_mask_with(&mut self, mask: N, u01: f64) -> CReg {
        let mut v = 0u64;
        expect_ok(check(unsafe { ffi::qvnt_reg_measure_mask(self.h, mask as u64, u01, &mut v) }));
        CReg::with_state(self.q_num, v as N)
    }

    /// `QReg::measure()`: every qubit.
    pub fn measure(&mut self) -> CReg {
        let all = if self.q_num >= N::BITS as N { !0 } else { (1 << self.q_num) - 1 };
        self.measure_mask(all)
    }

    pub fn get_probabilities(&self) -> Vec<R> {
        let mut out = vec![0.0; 1usize << self.q_num];
        expect_ok(check(unsafe { ffi::qvnt_reg_get_probabilities(self.h, out.as_mut_ptr()) }));
        out
    }

    pub fn get_absolute(&self) -> R {
        let mut out = 0.0;
        expect_ok(check(unsafe { ffi::qvnt_reg_get_absolute(self.h, &mut out) }));
        out
    }

    pub fn get_polar(&self) -> Vec<(R, R)> {
        let mut flat = vec![0.0; 2usize << self.q_num];
        expect_ok(check(unsafe { ffi::qvnt_reg_get_polar(self.h, flat.as_mut_ptr()) }));
        flat.chunks_exact(2).map(|p| (p[0], p[1])).collect()
    }

    /// All `max(2^q_num, 8)` amplitudes, copied to the host.
    pub fn amplitudes(&self) -> Vec<C> {
        let mut len = 0u64;
        expect_ok(check(unsafe { ffi::qvnt_reg_len(self.h, &mut len) }));
        let mut out = vec![C::new(0.0, 0.0); len as usize];
        expect_ok(check(unsafe { ffi::qvnt_reg_get_amplitudes(self.h, out.as_mut_ptr() as *mut f64) }));
        out
    }

    /// `QReg::reset(state)`.
    pub fn reset(&mut self, state: N) {
        expect_ok(check(unsafe { ffi::qvnt_reg_reset(self.h, state as u64) }));
    }

    /// `QReg::reset_by_mask(mask)`: zero where `i & mask != 0`, then `normalize`.
    pub fn reset_by_mask(&mut self, mask: N) {
        expect_ok(check(unsafe { ffi::qvnt_reg_reset_by_mask(self.h, mask as u64) }));
    }

    /// Selects the engine of later `apply` calls (`ffi::ENGINE_*`).
    pub fn set_engine(&mut self, engine: i32) -> Result<(), GpuError> {
        check(unsafe { ffi::qvnt_reg_set_engine(self.h, engine) })
    }
}

impl Clone for GpuReg {
    fn clone(&self) -> Self {
        let mut h = ptr::null_mut();
        expect_ok(check(unsafe { ffi::qvnt_reg_clone(self.h, &mut h) }));
        GpuReg { h, q_num: self.q_num, ctx: self.ctx.clone() }
    }
}

/// Tensor product `QReg * QReg` (quant.rs): `self` on the low qubits, `other` on the high ones.
impl Mul for GpuReg {
    type Output = GpuReg;

    fn mul(self, other: Self) -> Self::Output {
        let mut h = ptr::null_mut();
        expect_ok(check(unsafe { ffi::qvnt_reg_tensor(self.h, other.h, &mut h) }));
        GpuReg { h, q_num: self.q_num + other.q_num, ctx: self.ctx.clone() }
    }
}

impl Drop for GpuReg {
    fn drop(&mut self) {
        unsafe { ffi::qvnt_reg_destroy(self.h) };
    }
}
