"""ctypes binding of the CPU oracle (oracle/qvnt_oracle.c): TEST INFRASTRUCTURE ONLY.

The oracle restates qvnt 0.4.4's arithmetic; the tests, the smoke check and the CPU-baseline leg of
the benchmark use it as the checker.  Built by oracle/Makefile into oracle/_build/.
"""
import ctypes
import os
import subprocess

import numpy as np

from qvnt_gb300._abi import KIND, QvntGate

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
LIB = os.path.join(ORACLE_DIR, "_build", "libqvnt_oracle.so")

_lib = None
P = ctypes.POINTER
c_u32, c_u64, c_int, c_double, c_size, c_void = (ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int, ctypes.c_double,
                                                 ctypes.c_size_t, ctypes.c_void_p)

_PROTOS = {
    "oracle_acts_on": (c_u64, [P(QvntGate)]),
    "oracle_for_each": (None, [P(QvntGate), c_void, c_void, c_u64, c_int]),
    "oracle_apply": (None, [P(QvntGate), c_size, c_void, c_void, c_u64, c_int]),
    "oracle_reg_len": (c_u64, [c_u32]),
    "oracle_reg_init": (None, [c_u32, c_u64, c_void]),
    "oracle_get_absolute": (c_double, [c_void, c_u64]),
    "oracle_get_probabilities": (None, [c_void, c_u64, c_u32, c_void]),
    "oracle_weighted_index": (c_u64, [c_void, c_u64, c_double]),
    "oracle_collapse_mask": (None, [c_void, c_u64, c_u64, c_u64]),
    "oracle_measure_mask": (c_u64, [c_void, c_u64, c_u32, c_u64, c_double, P(c_u64)]),
    "oracle_reset": (None, [c_void, c_u64, c_u32, c_u64]),
    "oracle_normalize": (None, [c_void, c_u64, c_u32]),
    "oracle_reset_by_mask": (None, [c_void, c_u64, c_u32, c_u64]),
    "oracle_get_polar": (None, [c_void, c_u32, c_void]),
    "oracle_tensor": (None, [c_void, c_u32, c_void, c_u32, c_void]),
    "oracle_sample_all": (c_int, [c_void, c_u64, c_u32, c_u64, c_void, c_void]),
    "oracle_combine_with_unitary": (None, [c_void, c_void, c_u32, P(c_double), c_void]),
    "oracle_linear_composition": (None, [c_void, c_void, c_u64, P(c_double)]),
    "oracle_gate_make": (c_int, [c_u32, c_u64, c_u64, c_double, P(c_double), P(QvntGate)]),
    "oracle_is_unitary_m1": (c_int, [P(c_double)]),
    "oracle_is_unitary_m2": (c_int, [P(c_double)]),
    "oracle_gate_dgr": (None, [P(QvntGate)]),
    "oracle_gate_c": (c_int, [P(QvntGate), c_u64]),
    "oracle_op_h": (c_size, [c_u64, P(QvntGate)]),
    "oracle_op_qft": (c_size, [c_u64, P(QvntGate)]),
    "oracle_op_qft_swapped": (c_size, [c_u64, P(QvntGate)]),
    "oracle_op_u3": (c_size, [c_double, c_double, c_double, c_u64, P(QvntGate)]),
    "oracle_ops_dgr": (None, [P(QvntGate), c_size]),
    "oracle_matrix": (None, [P(QvntGate), c_size, c_u32, c_void]),
    "oracle_max_threads": (c_int, []),
}


def build():
    subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        for name, (res, args) in _PROTOS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def arr(gates):
    a = (QvntGate * max(len(gates), 1))()
    for i, g in enumerate(gates):
        a[i] = g
    return a


def make(kind, a=0, b=0, angle=0.0, matrix=None):
    g = QvntGate()
    m = None
    if matrix is not None:
        m = (ctypes.c_double * len(matrix))(*matrix)
    st = lib().oracle_gate_make(KIND[kind], a, b, float(angle), m, ctypes.byref(g))
    return g if st == 0 else None


def dgr(g):
    h = QvntGate.from_buffer_copy(g)
    lib().oracle_gate_dgr(ctypes.byref(h))
    return h


def c(g, mask):
    h = QvntGate.from_buffer_copy(g)
    return h if lib().oracle_gate_c(ctypes.byref(h), mask) == 0 else None


def _lst(fn, *args):
    n = fn(*args, None)
    a = (QvntGate * max(n, 1))()
    fn(*args, a)
    return [QvntGate.from_buffer_copy(a[i]) for i in range(n)]


def op_h(mask):
    return _lst(lib().oracle_op_h, mask)


def op_qft(mask):
    return _lst(lib().oracle_op_qft, mask)


def op_qft_swapped(mask):
    return _lst(lib().oracle_op_qft_swapped, mask)


def op_u3(the, phi, lam, mask):
    return _lst(lib().oracle_op_u3, float(the), float(phi), float(lam), mask)


def reg_len(n):
    return lib().oracle_reg_len(n)


def new_state(n, state=0):
    psi = np.zeros(reg_len(n), dtype=np.complex128)
    lib().oracle_reg_init(n, state, psi.ctypes.data)
    return psi


def apply(gates, psi, nthreads=None):
    """MultiOp::apply on a complex128 buffer, in place (one out-of-place pass per gate)."""
    nthreads = nthreads or lib().oracle_max_threads()
    scratch = np.empty_like(psi)
    a = arr(gates)
    lib().oracle_apply(a, len(gates), psi.ctypes.data, scratch.ctypes.data, psi.size, nthreads)
    return psi


def matrix(gates, size):
    out = np.empty((1 << size, 1 << size), dtype=np.complex128)
    lib().oracle_matrix(arr(gates), len(gates), size, out.ctypes.data)
    return out


def get_absolute(psi):
    return lib().oracle_get_absolute(psi.ctypes.data, psi.size)


def get_probabilities(psi, n):
    out = np.empty(1 << n, dtype=np.float64)
    lib().oracle_get_probabilities(psi.ctypes.data, psi.size, n, out.ctypes.data)
    return out


def weighted_index(w, u01):
    w = np.ascontiguousarray(w, dtype=np.float64)
    return lib().oracle_weighted_index(w.ctypes.data, w.size, float(u01))


def measure_mask(psi, n, mask, u01):
    """Returns (CReg value, chosen index); collapses psi in place."""
    idx = ctypes.c_uint64()
    v = lib().oracle_measure_mask(psi.ctypes.data, psi.size, n, mask, float(u01), ctypes.byref(idx))
    return v, idx.value


def normalize(psi, n):
    lib().oracle_normalize(psi.ctypes.data, psi.size, n)
    return psi


def reset_by_mask(psi, n, mask):
    lib().oracle_reset_by_mask(psi.ctypes.data, psi.size, n, mask)
    return psi


def get_polar(psi, n):
    out = np.empty((1 << n, 2), dtype=np.float64)
    lib().oracle_get_polar(psi.ctypes.data, n, out.ctypes.data)
    return out


def tensor(a, na, b, nb):
    out = np.empty(reg_len(na + nb), dtype=np.complex128)
    lib().oracle_tensor(a.ctypes.data, na, b.ctypes.data, nb, out.ctypes.data)
    return out


def sample_all(psi, n, count, z):
    """Histogram of `count` (2^n entries) given the standard-normal draws z; None where qvnt panics."""
    out = np.zeros(1 << n, dtype=np.uint64)
    z = np.ascontiguousarray(z, dtype=np.float64)
    st = lib().oracle_sample_all(psi.ctypes.data, psi.size, n, count, z.ctypes.data, out.ctypes.data)
    return None if st else out


def combine_with_unitary(a, b, n, c):
    out = np.empty(reg_len(n + 1), dtype=np.complex128)
    m = (ctypes.c_double * 8)(*[v for z in c for v in (complex(z).real, complex(z).imag)])
    lib().oracle_combine_with_unitary(a.ctypes.data, b.ctypes.data, n, m, out.ctypes.data)
    return out


def linear_composition(psi, other, c0, c1):
    m = (ctypes.c_double * 4)(complex(c0).real, complex(c0).imag, complex(c1).real, complex(c1).imag)
    lib().oracle_linear_composition(psi.ctypes.data, other.ctypes.data, psi.size, m)
    return psi


def max_threads():
    return lib().oracle_max_threads()


# ---- workloads built by the oracle's own builders ---------------------------------------------
# The seeded circuits of qvnt_gb300.circuits, drawn from the same SplitMix64 stream but built with
# the oracle's restatement of qvnt's constructors (oracle_gate_make, oracle_op_h/u3/qft,
# oracle_gate_c).  The CPU baseline and the reference arm of the benchmark use these, so that no
# code of the engine library runs on their path; a CPU test checks that both builders give the
# same gate list byte for byte.
_M64 = (1 << 64) - 1
TWO_PI = 2.0 * 3.141592653589793


class SplitMix64:
    def __init__(self, seed):
        self.state = seed & _M64

    def next_u64(self):
        self.state = (self.state + 0x9E3779B97F4A7C15) & _M64
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _M64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _M64
        return z ^ (z >> 31)

    def uniform(self):
        return (self.next_u64() >> 11) * (1.0 / 9007199254740992.0)

    def below(self, n):
        return self.next_u64() % n


def random_layers_gates(n, depth, rng):
    """Per layer: one of {h, s, t, u3} on every qubit, 15 two-qubit gates from {rxx, ryy, rzz, swap,
    i_swap, sqrt_i_swap} on random distinct pairs, 3 Toffolis x(t).c(c1 | c2)."""
    out = []
    for _ in range(depth):
        for q in range(n):
            kind = rng.below(4)
            m = 1 << q
            if kind == 0:
                out += op_h(m)
            elif kind == 1:
                out.append(make("S", m))
            elif kind == 2:
                out.append(make("T", m))
            else:
                th, ph, la = TWO_PI * rng.uniform(), TWO_PI * rng.uniform(), TWO_PI * rng.uniform()
                out += op_u3(th, ph, la, m)
        for _ in range(15):
            a = rng.below(n)
            b = rng.below(n - 1)
            if b >= a:
                b += 1
            ab = (1 << a) | (1 << b)
            kind = rng.below(6)
            if kind < 3:
                out.append(make(("RXX", "RYY", "RZZ")[kind], ab, angle=TWO_PI * rng.uniform()))
            else:
                out.append(make(("SWAP", "ISWAP", "SQRT_ISWAP")[kind - 3], ab))
        for _ in range(3):
            t = rng.below(n)
            c1 = rng.below(n - 1)
            if c1 >= t:
                c1 += 1
            c2 = rng.below(n)
            while c2 == t or c2 == c1:
                c2 = rng.below(n)
            out.append(c(make("X", 1 << t), (1 << c1) | (1 << c2)))
    return out


def random_circuit_gates(n=30, depth=40, seed=2, with_qft=True):
    """The random circuit: random layers, then op::qft over all n qubits."""
    out = random_layers_gates(n, depth, SplitMix64(seed))
    if with_qft:
        out += op_qft((1 << n) - 1)
    return out


def plain_circuit_gates(n=20, layers=20, seed=1):
    """op::h(all), then per layer rx, ry, rz on every qubit and nearest-neighbour CNOTs at an
    alternating offset, then op::qft(all)."""
    rng = SplitMix64(seed)
    out = op_h((1 << n) - 1)
    for layer in range(layers):
        for q in range(n):
            out.append(make("RX", 1 << q, angle=TWO_PI * rng.uniform()))
            out.append(make("RY", 1 << q, angle=TWO_PI * rng.uniform()))
            out.append(make("RZ", 1 << q, angle=TWO_PI * rng.uniform()))
        for i in range(layer % 2, n - 1, 2):
            out.append(c(make("X", 1 << (i + 1)), 1 << i))
    return out + op_qft((1 << n) - 1)


def gate_class(g):
    """Stratum of a gate of these workloads, for sampled timings: 'qft' (controlled RZ), 'toffoli'
    (X with controls), 'two' (two-qubit kinds), 'one' (the rest)."""
    k = g.kind
    if g.ctrl and k == KIND["RZ"]:
        return "qft"
    if g.ctrl:
        return "toffoli"
    if k in (KIND["RXX"], KIND["RYY"], KIND["RZZ"], KIND["SWAP"], KIND["ISWAP"], KIND["SQRT_ISWAP"],
             KIND["SQRT_SWAP"], KIND["H2"], KIND["U2"]):
        return "two"
    return "one"
