//! `sqrt_i_swap::Op` lowered to the engine's `qvnt_gate` (its stored fields, src/operator/atomic/sqrt_i_swap.rs).
//! A child module of the op's own, so that it reads the op's private fields.
use super::Op;
use crate::gpu::ffi::{qvnt_gate, KIND_SQRT_ISWAP};

impl Op {
    pub(crate) fn gb300_lower(&self, g: &mut qvnt_gate) {
        g.kind = KIND_SQRT_ISWAP;
        g.a_mask = self.ab_mask as u64;
        g.dagger = self.dagger as u32;
    }
}
