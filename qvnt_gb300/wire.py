"""Gate-list wire formats (host only): qvnt's operator names as text, and a lossless binary stream.

* ``ops_name(ops)`` / ``parse_ops(text)``: `MultiOp`'s ``{:?}`` text (src/operator/multi/mod.rs:90-94),
  e.g. ``"[C4_X123, RX1(1.23456)]"``.  What a qvnt program prints parses back to the gates qvnt's
  constructors build; the names omit the dagger of S, T, iSWAP, sqrt(SWAP) and sqrt(iSWAP), and a
  rotation's phase comes back as the phase of its printed angle.
* ``encode_gates`` / ``decode_gates`` and ``encode_request`` / ``decode_request``: the binary stream of
  ``qvnt_wire_*`` (versioned, CRC-32-checked, every gate field bit for bit), alone or as a whole
  serving request (the arguments of ``Server.submit``).

Malformed input raises QvntError (QVNT_ERR_BAD_ARG) with the library's message.
"""
import ctypes

from . import _abi
from ._abi import QvntCall, QvntGate, check, lib
from .operator import MultiOp, SingleOp


def _gate_array(ops):
    if ops is None:
        gates = []
    elif isinstance(ops, SingleOp):
        gates = [ops.g]
    elif isinstance(ops, MultiOp):
        gates = ops.gates()
    else:
        gates = [o.g if isinstance(o, SingleOp) else o for o in ops]
    arr = (QvntGate * max(len(gates), 1))()
    for i, g in enumerate(gates):
        ctypes.memmove(ctypes.byref(arr[i]), ctypes.byref(g), ctypes.sizeof(QvntGate))
    return arr, len(gates)


def _multi(arr, n):
    ops = []
    for i in range(n):
        g = QvntGate()
        ctypes.memmove(ctypes.byref(g), ctypes.byref(arr[i]), ctypes.sizeof(QvntGate))
        ops.append(SingleOp(g))
    return MultiOp(ops)


def ops_name(ops):
    """`format!("{:?}", multi_op)`: ``"[X1, C4_RZ2(0.5)]"``."""
    arr, n = _gate_array(ops)
    need = ctypes.c_size_t()
    check(lib().qvnt_ops_name(arr, n, None, 0, ctypes.byref(need)))
    buf = ctypes.create_string_buffer(need.value + 1)
    check(lib().qvnt_ops_name(arr, n, buf, need.value + 1, ctypes.byref(need)))
    return buf.value.decode()


def parse_ops(text):
    """The gates of a `MultiOp` ``{:?}`` list or of one `SingleOp` name, as a MultiOp."""
    raw = text.encode() if isinstance(text, str) else bytes(text)
    count = ctypes.c_size_t()
    check(lib().qvnt_ops_parse(raw, len(raw), None, 0, ctypes.byref(count)))
    arr = (QvntGate * max(count.value, 1))()
    check(lib().qvnt_ops_parse(raw, len(raw), arr, count.value, ctypes.byref(count)))
    return _multi(arr, count.value)


def _to_bytes(fn, *args):
    n = ctypes.c_size_t()
    check(fn(*args, None, 0, ctypes.byref(n)))
    buf = (ctypes.c_uint8 * n.value)()
    check(fn(*args, buf, n.value, ctypes.byref(n)))
    return bytes(buf)


def encode_gates(ops):
    """Binary stream of a gate list (MultiOp, SingleOp or QvntGate sequence)."""
    arr, n = _gate_array(ops)
    return _to_bytes(lib().qvnt_wire_encode_gates, arr, n)


def decode_gates(data):
    """MultiOp from encode_gates' stream."""
    data = bytes(data)
    src = (ctypes.c_uint8 * max(len(data), 1)).from_buffer_copy(data or b"\0")
    count = ctypes.c_size_t()
    check(lib().qvnt_wire_decode_gates(src, len(data), None, 0, ctypes.byref(count)))
    arr = (QvntGate * max(count.value, 1))()
    check(lib().qvnt_wire_decode_gates(src, len(data), arr, count.value, ctypes.byref(count)))
    return _multi(arr, count.value)


def _call_array(calls):
    arr = (QvntCall * max(len(calls), 1))()
    for i, c in enumerate(calls):
        if c[0] == "apply":
            arr[i].op, arr[i].gate_count = _abi.CALL_APPLY, int(c[1])
        elif c[0] == "measure":
            arr[i].op, arr[i].mask, arr[i].u01 = _abi.CALL_MEASURE, int(c[1]), float(c[2])
        else:
            raise ValueError("unknown call %r" % (c[0],))
    return arr


def encode_request(q_num, state, ops, calls, keep_amplitudes=False, detached=False):
    """Binary stream of one serving request; ``calls`` as for ``Server.submit``."""
    garr, ng = _gate_array(ops)
    carr = _call_array(calls)
    flags = (_abi.SUBMIT_KEEP_AMPLITUDES if keep_amplitudes else 0) | (_abi.SUBMIT_DETACHED if detached else 0)
    return _to_bytes(lib().qvnt_wire_encode_request, q_num, state, flags, garr, ng, carr, len(calls))


def decode_request(data):
    """dict(q_num, state, keep_amplitudes, detached, ops=MultiOp, calls=[("apply", n) | ("measure", mask, u01)])."""
    data = bytes(data)
    src = (ctypes.c_uint8 * max(len(data), 1)).from_buffer_copy(data or b"\0")
    q, s, fl = ctypes.c_uint32(), ctypes.c_uint64(), ctypes.c_int()
    ng, nc = ctypes.c_size_t(), ctypes.c_uint32()
    refs = (ctypes.byref(q), ctypes.byref(s), ctypes.byref(fl))
    check(lib().qvnt_wire_decode_request(src, len(data), *refs, None, 0, ctypes.byref(ng), None, 0, ctypes.byref(nc)))
    garr = (QvntGate * max(ng.value, 1))()
    carr = (QvntCall * max(nc.value, 1))()
    check(lib().qvnt_wire_decode_request(src, len(data), *refs, garr, ng.value, ctypes.byref(ng), carr, nc.value,
                                         ctypes.byref(nc)))
    calls = []
    for i in range(nc.value):
        c = carr[i]
        calls.append(("apply", c.gate_count) if c.op == _abi.CALL_APPLY else ("measure", c.mask, c.u01))
    return {"q_num": q.value, "state": s.value, "keep_amplitudes": bool(fl.value & _abi.SUBMIT_KEEP_AMPLITUDES),
            "detached": bool(fl.value & _abi.SUBMIT_DETACHED), "ops": _multi(garr, ng.value), "calls": calls}
