//! `MultiOp` (a queue of `SingleOp`s, src/operator/multi/mod.rs) lowered in queue order: one
//! `qvnt_gate` per `SingleOp`, applied by the engine in that order (as `MultiOp::apply` does).
use super::MultiOp;
use crate::gpu::{ffi::qvnt_gate, Lower};

impl Lower for MultiOp {
    fn lower_into(&self, out: &mut Vec<qvnt_gate>) {
        out.reserve(self.0.len());
        for op in self.0.iter() {
            out.push(op.gb300_gate());
        }
    }
}
