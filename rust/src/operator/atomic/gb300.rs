//! `AtomicOpDispatch` lowered variant by variant (src/operator/atomic/dispatch.rs: the engine's
//! kind numbers follow the same order).
use super::dispatch::AtomicOpDispatch;
use crate::gpu::ffi::qvnt_gate;

impl AtomicOpDispatch {
    pub(crate) fn gb300_lower(&self, g: &mut qvnt_gate) {
        match self {
            AtomicOpDispatch::Id(op) => op.gb300_lower(g),
            AtomicOpDispatch::X(op) => op.gb300_lower(g),
            AtomicOpDispatch::RX(op) => op.gb300_lower(g),
            AtomicOpDispatch::RXX(op) => op.gb300_lower(g),
            AtomicOpDispatch::Y(op) => op.gb300_lower(g),
            AtomicOpDispatch::RY(op) => op.gb300_lower(g),
            AtomicOpDispatch::RYY(op) => op.gb300_lower(g),
            AtomicOpDispatch::Z(op) => op.gb300_lower(g),
            AtomicOpDispatch::S(op) => op.gb300_lower(g),
            AtomicOpDispatch::T(op) => op.gb300_lower(g),
            AtomicOpDispatch::RZ(op) => op.gb300_lower(g),
            AtomicOpDispatch::RZZ(op) => op.gb300_lower(g),
            AtomicOpDispatch::U1(op) => op.gb300_lower(g),
            AtomicOpDispatch::U2(op) => op.gb300_lower(g),
            AtomicOpDispatch::H1(op) => op.gb300_lower(g),
            AtomicOpDispatch::H2(op) => op.gb300_lower(g),
            AtomicOpDispatch::Swap(op) => op.gb300_lower(g),
            AtomicOpDispatch::ISwap(op) => op.gb300_lower(g),
            AtomicOpDispatch::SqrtSwap(op) => op.gb300_lower(g),
            AtomicOpDispatch::SqrtISwap(op) => op.gb300_lower(g),
        }
    }
}
