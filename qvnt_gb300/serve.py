"""Serving form: a request loop with continuous admission over the register engine (`qvnt_server`).

A request is one register's life: `QReg::with_state(n, state)`, then its calls in order on the
resident state -- apply the next slice of its gate list, or measure_mask with an injected draw
(src/register/quant.rs:113-150, :376-395, :490-501).  The server runs `slots` requests at once, each
on its own CUDA stream, admits queued requests as slots and HBM budget free up, and records the
latency of every request from its arrival to its completion.
"""
import ctypes

import numpy as np

from . import _abi
from ._abi import QvntCall, QvntGate, ServerCounters, check, lib
from .register import default_context


class Server:
    def __init__(self, budget_bytes=150 * 10**9, slots=16, max_queue=4096, ctx=None):
        self.ctx = ctx or default_context()
        h = ctypes.c_void_p()
        check(lib().qvnt_server_create(self.ctx.h, int(budget_bytes), slots, max_queue, ctypes.byref(h)))
        self.h = h
        self._ncalls = {}

    def clock(self):
        t = ctypes.c_double()
        check(lib().qvnt_server_clock(self.h, ctypes.byref(t)))
        return t.value

    def submit(self, q_num, state, gates, calls, arrival=-1.0, keep_amplitudes=False, detached=False):
        """gates: ctypes QvntGate array or pointer (or None); calls: sequence of ("apply", count) /
        ("measure", mask, u01).  Returns the request id, or None when the queue is full (shed)."""
        arr = (QvntCall * max(len(calls), 1))()
        for i, c in enumerate(calls):
            if c[0] == "apply":
                arr[i].op, arr[i].gate_count = _abi.CALL_APPLY, int(c[1])
            else:
                arr[i].op, arr[i].mask, arr[i].u01 = _abi.CALL_MEASURE, int(c[1]), float(c[2])
        flags = (_abi.SUBMIT_KEEP_AMPLITUDES if keep_amplitudes else 0) | (_abi.SUBMIT_DETACHED if detached else 0)
        rid = ctypes.c_uint64()
        gp = ctypes.cast(gates, ctypes.POINTER(QvntGate)) if gates is not None else None
        st = lib().qvnt_server_submit(self.h, q_num, state, gp, arr, len(calls), float(arrival), flags,
                                      ctypes.byref(rid))
        if st == _abi.ERR_BUSY:
            return None
        check(st)
        if not detached:
            self._ncalls[rid.value] = (len(calls), q_num if keep_amplitudes else None)
        return rid.value

    def submit_request(self, data, arrival=-1.0):
        """Submits a request received as a binary wire stream (`qvnt_wire_encode_request`,
        `wire.encode_request`); returns what `submit` returns."""
        from .wire import decode_request
        r = decode_request(data)
        gates = _abi.gate_array(r["ops"].gates()) if len(r["ops"]) else None
        return self.submit(r["q_num"], r["state"], gates, r["calls"], arrival, r["keep_amplitudes"], r["detached"])

    def wait(self, rid, timeout=-1.0):
        """(measured values per call, final amplitudes or None, latency in seconds)."""
        ncalls, keep_n = self._ncalls.pop(rid)
        res = (ctypes.c_uint64 * max(ncalls, 1))()
        amps = None
        if keep_n is not None:
            amps = np.empty(max(1 << keep_n, 8), dtype=np.complex128)
        lat = ctypes.c_double()
        check(lib().qvnt_server_wait(self.h, rid, float(timeout), res, amps.ctypes.data if amps is not None else None,
                                     ctypes.byref(lat)))
        return [res[i] for i in range(ncalls)], amps, lat.value

    def stats(self):
        c = ServerCounters()
        check(lib().qvnt_server_stats(self.h, ctypes.byref(c)))
        return {name: getattr(c, name) for name, _ in ServerCounters._fields_}

    def _doubles(self, fn):
        n = ctypes.c_size_t()
        check(fn(self.h, None, 0, ctypes.byref(n)))
        out = np.zeros(n.value + 64, dtype=np.float64)
        check(fn(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), out.size, ctypes.byref(n)))
        return out[:min(n.value, out.size)]

    def latencies(self):
        return self._doubles(lib().qvnt_server_latencies)

    def queued_ages(self):
        return self._doubles(lib().qvnt_server_queued_ages)

    def close(self):
        if self.h:
            check(lib().qvnt_server_destroy(self.h))
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
