//! `h1::Op` lowered to the engine's `qvnt_gate` (its stored fields, src/operator/atomic/h1.rs).
//! A child module of the op's own, so that it reads the op's private fields.
use super::Op;
use crate::gpu::ffi::{qvnt_gate, KIND_H1};

impl Op {
    pub(crate) fn gb300_lower(&self, g: &mut qvnt_gate) {
        g.kind = KIND_H1;
        g.a_mask = self.a_mask as u64;
    }
}
