//! `rzz::Op` lowered to the engine's `qvnt_gate` (its stored fields, src/operator/atomic/rzz.rs).
//! A child module of the op's own, so that it reads the op's private fields.
use super::Op;
use crate::gpu::ffi::{qvnt_gate, KIND_RZZ};

impl Op {
    pub(crate) fn gb300_lower(&self, g: &mut qvnt_gate) {
        g.kind = KIND_RZZ;
        g.a_mask = self.ab_mask as u64;
        g.phase = [self.phase.re, self.phase.im];
    }
}
