//! `y::Op` lowered to the engine's `qvnt_gate` (its stored fields, src/operator/atomic/y.rs).
//! A child module of the op's own, so that it reads the op's private fields.
use super::Op;
use crate::gpu::ffi::{qvnt_gate, KIND_Y};

impl Op {
    pub(crate) fn gb300_lower(&self, g: &mut qvnt_gate) {
        g.kind = KIND_Y;
        // the stored power of i follows from the mask (y.rs `new`); the engine derives it again
        g.a_mask = self.a_mask as u64;
    }
}
