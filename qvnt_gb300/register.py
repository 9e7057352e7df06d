"""qvnt's registers (`QReg`, `CReg`, `VReg`, src/register/) over the engine's C ABI.

`QReg` owns a state vector that lives only in GPU memory (one `qvnt_reg` handle); `CReg` and `VReg`
are small host-side values, as in qvnt.  Measurement takes an optional uniform draw `u01` in [0, 1)
so that outcomes are reproducible; without it a draw comes from the operating system's entropy, as
qvnt's `thread_rng()` does (src/register/quant.rs:496-497).
"""
import ctypes
import random

import numpy as np

from . import _abi
from ._abi import QvntGate, check, gate_array, lib

_default_ctx = None
_rng = random.SystemRandom()


class Context:
    """One CUDA device (`qvnt_ctx`)."""

    def __init__(self, device=0):
        h = ctypes.c_void_p()
        check(lib().qvnt_ctx_create(device, ctypes.byref(h)))
        self.h = h
        self.device = device

    def mem_info(self):
        f, t = ctypes.c_uint64(), ctypes.c_uint64()
        check(lib().qvnt_ctx_mem_info(self.h, ctypes.byref(f), ctypes.byref(t)))
        return f.value, t.value

    def set_engine(self, engine):
        """Engine of the registers QReg makes on this context by default and of apply_host."""
        check(lib().qvnt_ctx_set_engine(self.h, engine))

    def apply_host(self, ops, psi_i, psi_o=None):
        """`Applicable::apply(psi_i, psi_o)` (src/operator/applicable.rs:5-6) on host buffers:
        psi_i / psi_o are complex128 arrays (len a power of two >= 8)."""
        psi_i = np.ascontiguousarray(psi_i, dtype=np.complex128)
        if psi_o is None:
            psi_o = np.empty_like(psi_i)
        gates = ops.gates()
        arr = gate_array(gates)
        check(lib().qvnt_apply_host(self.h, arr, len(gates), psi_i.ctypes.data, psi_o.ctypes.data, psi_i.size))
        return psi_o

    def close(self):
        if self.h:
            check(lib().qvnt_ctx_destroy(self.h))
            self.h = None


def default_context():
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


class CReg:
    """Classical register (src/register/class.rs:50-126)."""

    def __init__(self, q_num=0, value=0):
        self.q_num = q_num
        self.q_mask = ((1 << q_num) - 1) & 0xFFFFFFFFFFFFFFFF
        self.value = value

    @staticmethod
    def new(q_num):
        return CReg(q_num, 0)

    @staticmethod
    def with_state(q_num, state):
        return CReg(q_num, state)

    def num(self):
        return self.q_num

    def get(self):
        return self.value

    def set(self, bit, mask):
        self.value = (self.value | mask) if bit else (self.value & ~mask)

    def xor(self, bit, mask):
        if bit:
            self.value ^= mask

    def reset(self, i_state):
        self.value = i_state & self.q_mask

    def get_by_mask(self, mask):
        """Compresses the masked bits (class.rs:115-125)."""
        r, k = 0, 0
        for bit in bits_iter(mask & self.q_mask):
            if self.value & bit:
                r |= 1 << k
            k += 1
        return r

    def __mul__(self, other):
        return CReg(self.q_num + other.q_num, self.value | (other.value << self.q_num))

    def __eq__(self, other):
        return isinstance(other, CReg) and (self.q_num, self.value) == (other.q_num, other.value)

    def __repr__(self):
        s = ""
        for bit in bits_iter(self.q_mask):
            s = ("1" if bit & self.value else "0") + s
        return "(" + s + ")"


def bits_iter(bits):
    """Set bits of a mask as powers of two, LSB first (src/math/bits_iter.rs:12-27)."""
    pos = 1
    while pos <= bits:
        if pos & bits:
            yield pos
        pos <<= 1


class VReg:
    """Qubit alias -> mask helper (src/register/virtl.rs:84-157)."""

    def __init__(self, masks):
        self.masks = list(masks)

    @staticmethod
    def new(num):
        return VReg.new_with_mask((1 << num) - 1)

    @staticmethod
    def new_with_mask(mask):
        return VReg(bits_iter(mask))

    def __getitem__(self, key):
        if isinstance(key, int):
            return self.masks[key]
        if isinstance(key, slice) and key == slice(None):
            return self._fold(lambda i: True)
        if callable(key):
            return self._fold(key)
        return self._fold(lambda i: i in list(key))

    def _fold(self, f):
        acc = 0
        for i, m in enumerate(self.masks):
            if f(i):
                acc |= m
        return acc

    def __repr__(self):
        return "[" + ", ".join("%032x" % m for m in self.masks) + "]"


class QReg:
    """Quantum register (src/register/quant.rs:102-505) with its state in GPU memory."""

    def __init__(self, q_num, state=0, ctx=None, engine=None):
        self.ctx = ctx or default_context()
        h = ctypes.c_void_p()
        if engine is None:
            check(lib().qvnt_reg_create(self.ctx.h, q_num, state, ctypes.byref(h)))
        else:
            check(lib().qvnt_reg_create_ex(self.ctx.h, q_num, state, engine, ctypes.byref(h)))
        self.h = h
        self.q_num = q_num

    @classmethod
    def _wrap(cls, h, q_num, ctx):
        r = cls.__new__(cls)
        r.ctx, r.h, r.q_num = ctx, h, q_num
        return r

    @staticmethod
    def new(q_num, ctx=None):
        return QReg(q_num, 0, ctx)

    @staticmethod
    def with_state(q_num, state, ctx=None):
        return QReg(q_num, state, ctx)

    def __del__(self):
        h = getattr(self, "h", None)
        if h and _abi._lib is not None:
            _abi._lib.qvnt_reg_destroy(h)
            self.h = None

    def close(self):
        self.__del__()

    def clone(self):
        h = ctypes.c_void_p()
        check(lib().qvnt_reg_clone(self.h, ctypes.byref(h)))
        return QReg._wrap(h, self.q_num, self.ctx)

    def num(self):
        return self.q_num

    def len(self):
        n = ctypes.c_uint64()
        check(lib().qvnt_reg_len(self.h, ctypes.byref(n)))
        return n.value

    def num_threads(self, n):
        """qvnt picks a Rayon thread count here (quant.rs:185-200); the GPU engine has none to pick."""
        return self if n >= 1 else None

    def set_engine(self, engine):
        check(lib().qvnt_reg_set_engine(self.h, engine))
        return self

    def set_fusion_width(self, k):
        check(lib().qvnt_reg_set_fusion_width(self.h, k))
        return self

    def apply(self, op):
        gates = op.gates()
        if not gates:
            return
        arr = gate_array(gates)
        check(lib().qvnt_reg_apply(self.h, arr, len(gates)))

    def apply_gates(self, arr, count):
        """Applies a prebuilt ctypes QvntGate array (no Python-side copies)."""
        check(lib().qvnt_reg_apply(self.h, arr, count))

    def measure_mask(self, mask, u01=None, renormalise=False):
        if u01 is None:
            u01 = _rng.random()
        out = ctypes.c_uint64()
        check(lib().qvnt_reg_measure_mask_ex(self.h, mask, float(u01), 1 if renormalise else 0, ctypes.byref(out)))
        return CReg.with_state(self.q_num, out.value)

    def measure(self, u01=None):
        return self.measure_mask((1 << self.q_num) - 1, u01)

    def get_probabilities(self):
        out = np.empty(1 << self.q_num, dtype=np.float64)
        check(lib().qvnt_reg_get_probabilities(self.h, out.ctypes.data))
        return out

    def get_absolute(self):
        v = ctypes.c_double()
        check(lib().qvnt_reg_get_absolute(self.h, ctypes.byref(v)))
        return v.value

    def get_polar(self):
        out = np.empty((1 << self.q_num, 2), dtype=np.float64)
        check(lib().qvnt_reg_get_polar(self.h, out.ctypes.data))
        return out

    def sample_all(self, count, normals=None, seed=None):
        """`Reg::sample_all(count)` (quant.rs:513-594): histogram of `count` measurements without
        collapse.  `normals`: 2^n standard normal draws (qvnt's thread_rng draws); without them the
        device draws from `seed` (random when None)."""
        out = np.zeros(1 << self.q_num, dtype=np.uint64)
        z = None
        if normals is not None:
            z = np.ascontiguousarray(normals, dtype=np.float64)
            assert z.size == out.size
        if seed is None:
            seed = _rng.getrandbits(64)
        check(lib().qvnt_reg_sample_all(self.h, count, seed, z.ctypes.data if z is not None else None,
                                        out.ctypes.data))
        return out

    @staticmethod
    def combine_with_unitary(a, b, c):
        """`Reg::combine_with_unitary((a, b), c)` (quant.rs:273-308); c: 2x2 complex, row-major."""
        m = (ctypes.c_double * 8)(*[v for z in c for v in (complex(z).real, complex(z).imag)])
        h = ctypes.c_void_p()
        check(lib().qvnt_reg_combine_with_unitary(a.h, b.h, m, ctypes.byref(h)))
        return QReg._wrap(h, a.q_num + 1, a.ctx)

    def linear_composition(self, other, c0, c1):
        """`Reg::linear_composition(psi, (c0, c1))` (quant.rs:311-328): self = self c0 + other c1."""
        m = (ctypes.c_double * 4)(complex(c0).real, complex(c0).imag, complex(c1).real, complex(c1).imag)
        check(lib().qvnt_reg_linear_composition(self.h, other.h, m))
        return self

    def overlap(self, other):
        """(fidelity |<self|other>|^2 / (<self|self> <other|other>), max |self_i - other_i|), in FP64."""
        f, m = ctypes.c_double(), ctypes.c_double()
        check(lib().qvnt_reg_overlap(self.h, other.h, ctypes.byref(f), ctypes.byref(m)))
        return f.value, m.value

    def amplitudes(self):
        """All max(2^n, 8) amplitudes (qvnt's `psi` field) as complex128."""
        out = np.empty(self.len(), dtype=np.complex128)
        check(lib().qvnt_reg_get_amplitudes(self.h, out.ctypes.data))
        return out

    def amplitudes_range(self, first, count):
        """Amplitudes [first, first + count) as complex128."""
        out = np.empty(count, dtype=np.complex128)
        check(lib().qvnt_reg_get_amplitudes_range(self.h, first, count, out.ctypes.data))
        return out

    def set_amplitudes(self, psi):
        psi = np.ascontiguousarray(psi, dtype=np.complex128)
        if psi.size != self.len():
            raise ValueError("expected %d amplitudes" % self.len())
        check(lib().qvnt_reg_set_amplitudes(self.h, psi.ctypes.data))

    def reset(self, state=0):
        check(lib().qvnt_reg_reset(self.h, state))

    def reset_by_mask(self, mask):
        check(lib().qvnt_reg_reset_by_mask(self.h, mask))

    def normalize(self):
        check(lib().qvnt_reg_normalize(self.h))
        return self

    def sync(self):
        check(lib().qvnt_reg_sync(self.h))

    def stream(self):
        """The register's cudaStream_t as an integer handle."""
        s = ctypes.c_void_p()
        check(lib().qvnt_reg_get_stream(self.h, ctypes.byref(s)))
        return s.value or 0

    def get_vreg(self):
        return VReg.new_with_mask((1 << self.q_num) - 1)

    def get_vreg_by(self, mask):
        if mask & ~((1 << self.q_num) - 1):
            return None
        return VReg.new_with_mask(mask)

    def __mul__(self, other):
        """Tensor product (quant.rs:330-371): self on the low qubits."""
        h = ctypes.c_void_p()
        check(lib().qvnt_reg_tensor(self.h, other.h, ctypes.byref(h)))
        return QReg._wrap(h, self.q_num + other.q_num, self.ctx)

    def stats(self):
        a, b = ctypes.c_uint64(), ctypes.c_uint64()
        check(lib().qvnt_reg_stats(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def kernel_timing(self, enable=-1):
        ms, n = ctypes.c_double(), ctypes.c_uint64()
        check(lib().qvnt_reg_kernel_timing(self.h, enable, ctypes.byref(ms), ctypes.byref(n)))
        return ms.value, n.value

    def __repr__(self):
        amps = self.amplitudes()
        n = min(len(amps), 8, 1 << self.q_num)
        return "QReg {" + ", ".join("%d: %r" % (i, amps[i]) for i in range(n)) + (" .." if (1 << self.q_num) > 8 else "") + "}"
