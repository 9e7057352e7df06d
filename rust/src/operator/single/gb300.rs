//! `SingleOp { act, ctrl, func }` (src/operator/single/mod.rs) lowered to one `qvnt_gate`: the
//! atomic op's stored fields plus the control mask.  `act` is not carried: the engine recomputes
//! it from the kind and masks (`acts_on`), as `SingleOp::act_on` reads it from `func`.
use super::SingleOp;
use crate::gpu::{ffi::qvnt_gate, Lower};

impl SingleOp {
    pub(crate) fn gb300_gate(&self) -> qvnt_gate {
        let mut g = qvnt_gate::zeroed();
        self.func.gb300_lower(&mut g);
        g.ctrl = self.ctrl as u64;
        g
    }
}

impl Lower for SingleOp {
    fn lower_into(&self, out: &mut Vec<qvnt_gate>) {
        out.push(self.gb300_gate());
    }
}
