"""qvnt's operator API (`qvnt::operator`, imported as `op`), over the engine's C ABI.

Mirrors src/operator/mod.rs: every `op::` constructor returns a `MultiOp` (a queue of
`SingleOp`s, src/operator/multi/mod.rs:62-63); `*` concatenates, `.c(mask)` adds controls and
returns None when the mask overlaps (qvnt's `Option`), `.dgr()` inverts.  Where qvnt panics
(`expect("Mask should contain 1 bit!")`, src/operator/mod.rs:151-155) this raises ValueError.
The gate lists are built by the library's builders (qvnt_op_*, qvnt_gate_make).
"""
import ctypes
import math

from . import _abi
from ._abi import KIND, QvntGate, check, lib


class SingleOp:
    """One gate: `SingleOp { act, ctrl, func }` (src/operator/single/mod.rs:42-47)."""

    __slots__ = ("g",)

    def __init__(self, g):
        self.g = g

    @staticmethod
    def _make(kind, a_mask, b_mask=0, angle=0.0, matrix=None):
        g = QvntGate()
        m = None
        if matrix is not None:
            flat = []
            for z in matrix:
                z = complex(z)
                flat += [z.real, z.imag]
            m = (ctypes.c_double * len(flat))(*flat)
        st = lib().qvnt_gate_make(KIND[kind], a_mask, b_mask, float(angle), m, ctypes.byref(g))
        if st != _abi.OK:
            return None
        return SingleOp(g)

    def clone(self):
        g = QvntGate()
        ctypes.memmove(ctypes.byref(g), ctypes.byref(self.g), ctypes.sizeof(QvntGate))
        return SingleOp(g)

    def name(self):
        needed = ctypes.c_size_t()
        buf = ctypes.create_string_buffer(4096)
        check(lib().qvnt_gate_name(ctypes.byref(self.g), buf, 4096, ctypes.byref(needed)))
        return buf.value.decode()

    def __repr__(self):
        return self.name()

    def act_on(self):
        """`act | ctrl` (single/mod.rs:93-95)."""
        return lib().qvnt_gate_act_on(ctypes.byref(self.g))

    def dgr(self):
        s = self.clone()
        check(lib().qvnt_gate_dgr(ctypes.byref(s.g)))
        return s

    def c(self, c_mask):
        """Controlled copy, or None if c_mask overlaps act_on (single/mod.rs:106-116)."""
        s = self.clone()
        if lib().qvnt_gate_c(ctypes.byref(s.g), c_mask) != _abi.OK:
            return None
        return s

    def __eq__(self, other):
        return isinstance(other, SingleOp) and bytes(self.g) == bytes(other.g)

    def __mul__(self, other):
        return MultiOp([self]) * other

    def gates(self):
        return [self.g]

    def matrix(self, size):
        return MultiOp([self]).matrix(size)


class MultiOp:
    """Gate queue (src/operator/multi/mod.rs:62-191)."""

    __slots__ = ("ops",)

    def __init__(self, ops=None):
        self.ops = list(ops or [])

    @staticmethod
    def from_single(s):
        # `From<SingleOp>` drops Id (multi/mod.rs:135-146)
        if s is None:
            raise ValueError("invalid gate")
        return MultiOp([] if s.name() == "Id" else [s])

    def __len__(self):
        return len(self.ops)

    def __getitem__(self, i):
        return self.ops[i]

    def __iter__(self):
        return iter(self.ops)

    def __mul__(self, other):
        if isinstance(other, SingleOp):
            other = MultiOp.from_single(other)
        if not isinstance(other, MultiOp):
            return NotImplemented
        return MultiOp(self.ops + other.ops)

    def __imul__(self, other):
        return self * other

    def __eq__(self, other):
        return isinstance(other, MultiOp) and self.ops == other.ops

    def __repr__(self):
        return "[" + ", ".join(o.name() for o in self.ops) + "]"

    def ends_with(self, suffix):
        """multi/mod.rs:66-71"""
        return all(a == b for a, b in zip(reversed(self.ops), reversed(suffix.ops)))

    def act_on(self):
        r = 0
        for o in self.ops:
            r |= o.act_on()
        return r

    def dgr(self):
        """Reverse and dagger every gate (multi/mod.rs:120-123)."""
        return MultiOp([o.dgr() for o in reversed(self.ops)])

    def c(self, c_mask):
        """Control every gate; None if c_mask overlaps act_on (multi/mod.rs:125-132)."""
        if self.act_on() & c_mask:
            return None
        return MultiOp([o.c(c_mask) for o in self.ops])

    def gates(self):
        return [o.g for o in self.ops]

    def matrix(self, size):
        """`Applicable::matrix(size)` (src/operator/applicable.rs:17-46): applies the queue to every
        basis vector of a 2^size register on the GPU; returns rows of complex numbers."""
        from .register import QReg
        dim = 1 << size
        cols = []
        for c in range(dim):
            q = QReg.with_state(size, c)
            q.apply(self)
            cols.append(q.amplitudes()[:dim])
        return [[complex(cols[c][r]) for c in range(dim)] for r in range(dim)]


def plan_info(ops, q_num, fusion_k=0):
    """How the fused engine would run `ops` on a q_num-qubit register (host-side planning only):
    (passes, register stages, engine gates)."""
    gates = ops.gates()
    arr = _abi.gate_array(gates)
    p, s, e = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
    check(lib().qvnt_plan_info(arr, len(gates), q_num, fusion_k, ctypes.byref(p), ctypes.byref(s), ctypes.byref(e)))
    return p.value, s.value, e.value


def _list(builder, *args):
    count = ctypes.c_size_t()
    check(builder(*args, None, 0, ctypes.byref(count)))
    arr = (QvntGate * max(count.value, 1))()
    check(builder(*args, arr, count.value, ctypes.byref(count)))
    return MultiOp([SingleOp(arr[i]) for i in range(count.value)])


def _one(kind, a, b=0, angle=0.0, bits=None):
    s = SingleOp._make(kind, a, b, angle)
    if s is None:
        raise ValueError("Mask should contain %d bit!" % bits if bits else "invalid mask")
    return MultiOp.from_single(s)


# ---- constructors of src/operator/mod.rs ----------------------------------------------------
def id():  # noqa: A001  (qvnt's name)
    """`op::id()` (mod.rs:113-115): the empty queue."""
    return MultiOp()


def x(a_mask):
    return _one("X", a_mask)


def y(a_mask):
    return _one("Y", a_mask)


def z(a_mask):
    return _one("Z", a_mask)


def s(a_mask):
    return _one("S", a_mask)


def t(a_mask):
    return _one("T", a_mask)


def rx(phase, a_mask):
    return _one("RX", a_mask, angle=phase, bits=1)


def ry(phase, a_mask):
    return _one("RY", a_mask, angle=phase, bits=1)


def rz(phase, a_mask):
    return _one("RZ", a_mask, angle=phase, bits=1)


def rxx(phase, ab_mask):
    return _one("RXX", ab_mask, angle=phase, bits=2)


def ryy(phase, ab_mask):
    return _one("RYY", ab_mask, angle=phase, bits=2)


def rzz(phase, ab_mask):
    return _one("RZZ", ab_mask, angle=phase, bits=2)


def swap(ab_mask):
    return _one("SWAP", ab_mask, bits=2)


def sqrt_swap(ab_mask):
    return _one("SQRT_SWAP", ab_mask, bits=2)


def i_swap(ab_mask):
    return _one("ISWAP", ab_mask, bits=2)


def sqrt_i_swap(ab_mask):
    return _one("SQRT_ISWAP", ab_mask, bits=2)


def h(a_mask):
    """`op::h` (src/operator/multi/h.rs:14-45)."""
    return _list(lib().qvnt_op_h, a_mask)


def u1(lam, a_mask):
    """`op::u1` = rz (mod.rs:472-474)."""
    return rz(lam, a_mask)


def u2(phi, lam, a_mask):
    """`op::u2` = rz(lam) * ry(pi/2) * rz(phi) (mod.rs:480-482)."""
    if bin(a_mask).count("1") != 1:
        raise ValueError("Mask should contain 1 bit!")
    return _list(lib().qvnt_op_u2, float(phi), float(lam), a_mask)


def u3(the, phi, lam, a_mask):
    """`op::u3` = rz(lam) * ry(the) * rz(phi) (mod.rs:499-501)."""
    if bin(a_mask).count("1") != 1:
        raise ValueError("Mask should contain 1 bit!")
    return _list(lib().qvnt_op_u3, float(the), float(phi), float(lam), a_mask)


def qft(a_mask):
    """`op::qft` (src/operator/multi/qft.rs:4-33): no final swaps."""
    return _list(lib().qvnt_op_qft, a_mask)


def qft_swapped(a_mask):
    """`op::qft_swapped` (src/operator/multi/qft.rs:35-52)."""
    return _list(lib().qvnt_op_qft_swapped, a_mask)


# Crate-private atomic constructors (src/operator/single/pauli.rs:31-39): dense 2x2 / 4x4 gates.
def u1_matrix(a_mask, matrix):
    """`single::pauli::u1(a_mask, matrix)`: SingleOp or None (mask or unitarity check failed)."""
    return SingleOp._make("U1", a_mask, 0, 0.0, matrix)


def u2_matrix(a_mask, b_mask, matrix):
    """`single::pauli::u2(a_mask, b_mask, matrix)`: SingleOp or None."""
    return SingleOp._make("U2", a_mask, b_mask, 0.0, matrix)


PI = math.pi
