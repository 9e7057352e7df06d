//! `t::Op` lowered to the engine's `qvnt_gate` (its stored fields, src/operator/atomic/t.rs).
//! A child module of the op's own, so that it reads the op's private fields.
use super::Op;
use crate::gpu::ffi::{qvnt_gate, KIND_T};

impl Op {
    pub(crate) fn gb300_lower(&self, g: &mut qvnt_gate) {
        g.kind = KIND_T;
        g.a_mask = self.a_mask as u64;
        g.dagger = self.dagger as u32;
    }
}
