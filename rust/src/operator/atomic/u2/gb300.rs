//! `u2::Op` lowered to the engine's `qvnt_gate` (its stored fields, src/operator/atomic/u2.rs).
//! A child module of the op's own, so that it reads the op's private fields.
use super::Op;
use crate::gpu::ffi::{qvnt_gate, KIND_U2};

impl Op {
    pub(crate) fn gb300_lower(&self, g: &mut qvnt_gate) {
        g.kind = KIND_U2;
        g.a_mask = self.a_mask as u64;
        g.b_mask = self.b_mask as u64;
        for (i, c) in self.matrix.iter().enumerate() {
            g.matrix[2 * i] = c.re;
            g.matrix[2 * i + 1] = c.im;
        }
    }
}
