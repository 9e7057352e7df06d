//! `extern "C"` declarations of the GB300 engine (include/qvnt_gb300.h) used by the GPU-backed
//! register.  Every entry point returns a status: 0 = ok, otherwise a `QVNT_ERR_*` code with a
//! message in `qvnt_last_error()`.
#![allow(non_camel_case_types)]

use std::os::raw::{c_char, c_int, c_void};

/// One lowered `SingleOp` (`SingleOp { act, ctrl, func }`, src/operator/single/mod.rs): the atomic
/// op's kind and stored fields plus the control mask.  Fields a kind does not use stay zero.
#[repr(C)]
#[derive(Clone, Copy, Debug, PartialEq)]
pub struct qvnt_gate {
    pub kind: u32,
    pub dagger: u32,
    pub a_mask: u64,
    pub b_mask: u64,
    pub ctrl: u64,
    pub phase: [f64; 2],
    pub matrix: [f64; 32],
}

// The C layout: 304 bytes, phase at offset 32.
const _: () = assert!(std::mem::size_of::<qvnt_gate>() == 304);

impl qvnt_gate {
    pub const fn zeroed() -> Self {
        qvnt_gate { kind: 0, dagger: 0, a_mask: 0, b_mask: 0, ctrl: 0, phase: [0.0; 2], matrix: [0.0; 32] }
    }
}

/// `enum qvnt_gate_kind`: the order of `AtomicOpDispatch` (src/operator/atomic/dispatch.rs).
pub const KIND_ID: u32 = 0;
pub const KIND_X: u32 = 1;
pub const KIND_RX: u32 = 2;
pub const KIND_RXX: u32 = 3;
pub const KIND_Y: u32 = 4;
pub const KIND_RY: u32 = 5;
pub const KIND_RYY: u32 = 6;
pub const KIND_Z: u32 = 7;
pub const KIND_S: u32 = 8;
pub const KIND_T: u32 = 9;
pub const KIND_RZ: u32 = 10;
pub const KIND_RZZ: u32 = 11;
pub const KIND_U1: u32 = 12;
pub const KIND_U2: u32 = 13;
pub const KIND_H1: u32 = 14;
pub const KIND_H2: u32 = 15;
pub const KIND_SWAP: u32 = 16;
pub const KIND_ISWAP: u32 = 17;
pub const KIND_SQRT_SWAP: u32 = 18;
pub const KIND_SQRT_ISWAP: u32 = 19;

/// `enum qvnt_engine`.
pub const ENGINE_FUSED: c_int = 0;
pub const ENGINE_PLAIN: c_int = 1;
pub const ENGINE_PRECISION: c_int = 2;
pub const ENGINE_TENSOR64: c_int = 3;

pub const QVNT_OK: c_int = 0;

#[repr(C)]
pub struct qvnt_ctx {
    _private: [u8; 0],
}
#[repr(C)]
pub struct qvnt_reg {
    _private: [u8; 0],
}

extern "C" {
    pub fn qvnt_status_string(status: c_int) -> *const c_char;
    pub fn qvnt_last_error() -> *const c_char;
    pub fn qvnt_abi_version() -> u32;

    pub fn qvnt_ctx_create(device: c_int, out: *mut *mut qvnt_ctx) -> c_int;
    pub fn qvnt_ctx_destroy(ctx: *mut qvnt_ctx) -> c_int;
    pub fn qvnt_ctx_set_engine(ctx: *mut qvnt_ctx, engine: c_int) -> c_int;

    pub fn qvnt_reg_create(ctx: *mut qvnt_ctx, q_num: u32, state: u64, out: *mut *mut qvnt_reg) -> c_int;
    pub fn qvnt_reg_create_ex(ctx: *mut qvnt_ctx, q_num: u32, state: u64, engine: c_int, out: *mut *mut qvnt_reg)
        -> c_int;
    pub fn qvnt_reg_destroy(reg: *mut qvnt_reg) -> c_int;
    pub fn qvnt_reg_clone(reg: *const qvnt_reg, out: *mut *mut qvnt_reg) -> c_int;
    pub fn qvnt_reg_len(reg: *const qvnt_reg, len: *mut u64) -> c_int;
    pub fn qvnt_reg_set_engine(reg: *mut qvnt_reg, engine: c_int) -> c_int;
    pub fn qvnt_reg_apply(reg: *mut qvnt_reg, gates: *const qvnt_gate, count: usize) -> c_int;
    pub fn qvnt_reg_measure_mask(reg: *mut qvnt_reg, mask: u64, u01: f64, out: *mut u64) -> c_int;
    pub fn qvnt_reg_get_probabilities(reg: *mut qvnt_reg, out: *mut f64) -> c_int;
    pub fn qvnt_reg_get_absolute(reg: *mut qvnt_reg, out: *mut f64) -> c_int;
    pub fn qvnt_reg_get_polar(reg: *mut qvnt_reg, out: *mut f64) -> c_int;
    pub fn qvnt_reg_get_amplitudes(reg: *mut qvnt_reg, out: *mut f64) -> c_int;
    pub fn qvnt_reg_reset(reg: *mut qvnt_reg, state: u64) -> c_int;
    pub fn qvnt_reg_reset_by_mask(reg: *mut qvnt_reg, mask: u64) -> c_int;
    pub fn qvnt_reg_normalize(reg: *mut qvnt_reg) -> c_int;
    pub fn qvnt_reg_tensor(a: *const qvnt_reg, b: *const qvnt_reg, out: *mut *mut qvnt_reg) -> c_int;
    pub fn qvnt_reg_sync(reg: *mut qvnt_reg) -> c_int;
    pub fn qvnt_apply_host(
        ctx: *mut qvnt_ctx,
        gates: *const qvnt_gate,
        count: usize,
        psi_i: *const f64,
        psi_o: *mut f64,
        len: u64,
    ) -> c_int;
    pub fn qvnt_norm_sqr_noalloc(d_psi: *const f64, len: u64, d_out: *mut f64, stream: *mut c_void) -> c_int;
}
