"""Batching form: many independent registers run by one persistent launch (`qvnt_batch`).

Each register is `QReg::with_state(n_i, state_i)`, then `apply` of its own gate list, then (mask
non-zero) `measure_mask(mask_i)` with an injected draw -- what a caller would otherwise do with a
host loop over registers (src/register/quant.rs:113-150, :376-395, :490-501).  One `run()` replays a
CUDA graph: state reset, the persistent batch kernel (every circuit and every measurement), results
back.  The schedule's tile width and pass budget come from `autotune()` or `set_fusion()`.
"""
import ctypes

import numpy as np

from ._abi import QvntGate, check, lib
from .register import default_context


class Batch:
    def __init__(self, q_nums, states, gates, offsets, masks=None, ctx=None):
        """q_nums, states, masks: one entry per register; gates: a ctypes array of QvntGate;
        offsets: len(q_nums) + 1 gate offsets (register i owns gates[offsets[i]:offsets[i+1]])."""
        self.ctx = ctx or default_context()
        n = len(q_nums)
        self.q_nums = np.ascontiguousarray(q_nums, dtype=np.uint32)
        self.states = np.ascontiguousarray(states, dtype=np.uint64)
        self.offsets = np.ascontiguousarray(offsets, dtype=np.uint64)
        self.masks = np.ascontiguousarray(masks if masks is not None else np.zeros(n), dtype=np.uint64)
        assert self.offsets.size == n + 1
        P = ctypes.POINTER
        h = ctypes.c_void_p()
        check(lib().qvnt_batch_create(
            self.ctx.h, n, self.q_nums.ctypes.data_as(P(ctypes.c_uint32)),
            self.states.ctypes.data_as(P(ctypes.c_uint64)),
            ctypes.cast(gates, P(QvntGate)) if gates is not None else None,
            self.offsets.ctypes.data_as(P(ctypes.c_uint64)), self.masks.ctypes.data_as(P(ctypes.c_uint64)),
            ctypes.byref(h)))
        self.h = h
        self.count = n

    def run(self, u01=None):
        """One replay: returns the measured values (uint64 per register; 0 where the mask is 0)."""
        out = np.zeros(self.count, dtype=np.uint64)
        P = ctypes.POINTER
        u = None
        if u01 is not None:
            u = np.ascontiguousarray(u01, dtype=np.float64)
            assert u.size == self.count
        check(lib().qvnt_batch_run(self.h, u.ctypes.data_as(P(ctypes.c_double)) if u is not None else None,
                                   out.ctypes.data_as(P(ctypes.c_uint64))))
        return out

    def set_fusion(self, fusion_k, pass_budget=0):
        check(lib().qvnt_batch_set_fusion(self.h, fusion_k, pass_budget))

    def autotune(self, stride=8):
        k, b, ms = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_double()
        check(lib().qvnt_batch_autotune(self.h, stride, ctypes.byref(k), ctypes.byref(b), ctypes.byref(ms)))
        return k.value, b.value, ms.value

    def amplitudes(self, i):
        out = np.empty(1 << int(self.q_nums[i]), dtype=np.complex128)
        check(lib().qvnt_batch_get_amplitudes(self.h, i, out.ctypes.data))
        return out

    def info(self):
        it, ps, sb = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        k, b, ms = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_double()
        check(lib().qvnt_batch_info(self.h, ctypes.byref(it), ctypes.byref(ps), ctypes.byref(sb), ctypes.byref(k),
                                    ctypes.byref(b), ctypes.byref(ms)))
        return {"items": it.value, "passes": ps.value, "state_bytes": sb.value, "fusion_k": k.value,
                "pass_budget": b.value, "last_ms": ms.value}

    def close(self):
        if self.h:
            check(lib().qvnt_batch_destroy(self.h))
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
