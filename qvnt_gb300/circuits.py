"""Seeded synthetic circuits: the workloads the engine is measured and checked on.

There is no public circuit suite behind these; each generator draws from a SplitMix64 stream so
that the GPU run, the CPU oracle and the CPU baseline see the same gate list.

  plain_circuit(n=20, layers=20)   op::h(all), then per layer rx, ry, rz on every qubit with angles
                                   in [0, 2pi) and nearest-neighbour CNOTs x(1<<(i+1)).c(1<<i) at an
                                   alternating even/odd offset; then op::qft(all).  (~1,610 gates at
                                   n = 20.)
  random_circuit(n=30, depth=40)   per layer one gate from {h, s, t, u3(th, phi, lam)} on every
                                   qubit, 15 two-qubit gates from {rxx, ryy, rzz, swap, i_swap,
                                   sqrt_i_swap} on random distinct pairs, 3 Toffolis
                                   x(t).c(c1 | c2); then op::qft(all).  (~2,985 gates at n = 30.)
  batch_workload(count=4096)       registers with n uniform in [8, 20], with_state(n, random basis
                                   index), each its own random layers with depth uniform in
                                   [10, 60], then measure_mask(all).
"""
import ctypes
import math

import numpy as np

from . import operator as op
from ._abi import QvntGate, check, lib
from .operator import MultiOp

_MASK64 = (1 << 64) - 1
TWO_PI = 2.0 * math.pi


class SplitMix64:
    def __init__(self, seed):
        self.state = seed & _MASK64

    def next_u64(self):
        self.state = (self.state + 0x9E3779B97F4A7C15) & _MASK64
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _MASK64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _MASK64
        return z ^ (z >> 31)

    def uniform(self):
        """Uniform double in [0, 1) with 53 random bits."""
        return (self.next_u64() >> 11) * (1.0 / 9007199254740992.0)

    def below(self, n):
        return self.next_u64() % n


def plain_circuit(n=20, layers=20, seed=1):
    rng = SplitMix64(seed)
    all_mask = (1 << n) - 1
    ops = [op.h(all_mask)]
    for layer in range(layers):
        for q in range(n):
            ops.append(op.rx(TWO_PI * rng.uniform(), 1 << q))
            ops.append(op.ry(TWO_PI * rng.uniform(), 1 << q))
            ops.append(op.rz(TWO_PI * rng.uniform(), 1 << q))
        for i in range(layer % 2, n - 1, 2):
            ops.append(op.x(1 << (i + 1)).c(1 << i))
    ops.append(op.qft(all_mask))
    return _concat(ops)


def random_layers(n, depth, rng):
    ops = []
    for _ in range(depth):
        for q in range(n):
            kind = rng.below(4)
            if kind == 0:
                ops.append(op.h(1 << q))
            elif kind == 1:
                ops.append(op.s(1 << q))
            elif kind == 2:
                ops.append(op.t(1 << q))
            else:
                th, ph, la = TWO_PI * rng.uniform(), TWO_PI * rng.uniform(), TWO_PI * rng.uniform()
                ops.append(op.u3(th, ph, la, 1 << q))
        for _ in range(15):
            a = rng.below(n)
            b = rng.below(n - 1)
            if b >= a:
                b += 1
            ab = (1 << a) | (1 << b)
            kind = rng.below(6)
            if kind < 3:
                ops.append((op.rxx, op.ryy, op.rzz)[kind](TWO_PI * rng.uniform(), ab))
            else:
                ops.append((op.swap, op.i_swap, op.sqrt_i_swap)[kind - 3](ab))
        for _ in range(3):
            t = rng.below(n)
            c1 = rng.below(n - 1)
            if c1 >= t:
                c1 += 1
            c2 = rng.below(n)
            while c2 == t or c2 == c1:
                c2 = rng.below(n)
            ops.append(op.x(1 << t).c((1 << c1) | (1 << c2)))
    return ops


def random_circuit(n=30, depth=40, seed=2, with_qft=True):
    rng = SplitMix64(seed)
    ops = random_layers(n, depth, rng)
    if with_qft:
        ops.append(op.qft((1 << n) - 1))
    return _concat(ops)


def random_layers_gates(n, depth, rng):
    """`random_layers(n, depth, rng)` drawn by the library's C twin of the generator
    (qvnt_workload_random_layers: same draws, same gates), as a ctypes QvntGate array; advances
    `rng` exactly as random_layers does."""
    arr, count = _c_layers(n, depth, rng)
    return arr, count


def _c_layers(n, depth, rng, into=None, at=0):
    st = ctypes.c_uint64(rng.state)
    cnt = ctypes.c_size_t()
    check(lib().qvnt_workload_random_layers(n, depth, ctypes.byref(st), None, 0, ctypes.byref(cnt)))
    count = cnt.value
    st = ctypes.c_uint64(rng.state)
    if into is None:
        into = (QvntGate * max(count, 1))()
        at = 0
    dst = ctypes.cast(ctypes.byref(into, at * ctypes.sizeof(QvntGate)), ctypes.POINTER(QvntGate))
    check(lib().qvnt_workload_random_layers(n, depth, ctypes.byref(st), dst, count, ctypes.byref(cnt)))
    rng.state = st.value
    return into, count


class BatchWorkload:
    """Registers for the batching form: q_nums, initial basis states, concatenated gate lists with
    offsets, measure masks."""

    def __init__(self, q_nums, states, depths, gates, offsets, masks):
        self.q_nums, self.states, self.depths = q_nums, states, depths
        self.gates, self.offsets, self.masks = gates, offsets, masks

    @property
    def count(self):
        return len(self.q_nums)

    @property
    def total_gates(self):
        return int(self.offsets[-1])

    def gates_of(self, i):
        """(ctypes pointer, count) of register i's gate list."""
        a, b = int(self.offsets[i]), int(self.offsets[i + 1])
        return ctypes.cast(ctypes.byref(self.gates, a * ctypes.sizeof(QvntGate)), ctypes.POINTER(QvntGate)), b - a


def batch_workload(count=4096, seed=4, q_range=(8, 20), depth_range=(10, 60), measure=True):
    """The batching workload: `count` registers, qubit counts uniform in q_range, each
    `with_state(n, uniform basis index)` and its own circuit of random layers (the gate mix of
    random_circuit) with depth uniform in depth_range, then measure_mask of all qubits."""
    rng = SplitMix64(seed)
    q_nums = np.zeros(count, dtype=np.uint32)
    states = np.zeros(count, dtype=np.uint64)
    depths = np.zeros(count, dtype=np.uint32)
    seeds = np.zeros(count, dtype=np.uint64)
    for i in range(count):
        n = q_range[0] + rng.below(q_range[1] - q_range[0] + 1)
        q_nums[i] = n
        states[i] = rng.below(1 << n)
        depths[i] = depth_range[0] + rng.below(depth_range[1] - depth_range[0] + 1)
        seeds[i] = rng.next_u64()
    counts = np.zeros(count, dtype=np.uint64)
    for i in range(count):
        st = ctypes.c_uint64(int(seeds[i]))
        cnt = ctypes.c_size_t()
        check(lib().qvnt_workload_random_layers(int(q_nums[i]), int(depths[i]), ctypes.byref(st), None, 0,
                                                ctypes.byref(cnt)))
        counts[i] = cnt.value
    offsets = np.zeros(count + 1, dtype=np.uint64)
    offsets[1:] = np.cumsum(counts)
    gates = (QvntGate * max(int(offsets[-1]), 1))()
    for i in range(count):
        _c_layers(int(q_nums[i]), int(depths[i]), SplitMix64(int(seeds[i])), gates, int(offsets[i]))
    masks = np.array([(1 << int(n)) - 1 if measure else 0 for n in q_nums], dtype=np.uint64)
    return BatchWorkload(q_nums, states, depths, gates, offsets, masks)


class ServeRequest:
    """One served request: arrival time (s), register size and basis state, and its calls: rounds
    of (apply `depths[i]` random layers, measure_mask(masks[i]) with draw u01s[i])."""

    __slots__ = ("arrival", "n", "state", "depths", "masks", "u01s", "seed")

    def __init__(self, arrival, n, state, depths, masks, u01s, seed):
        self.arrival, self.n, self.state = arrival, n, state
        self.depths, self.masks, self.u01s, self.seed = depths, masks, u01s, seed

    def build(self):
        """(gate array, calls) for Server.submit."""
        rng = SplitMix64(self.seed)
        counts = []
        for d in self.depths:
            st = ctypes.c_uint64(rng.state)
            cnt = ctypes.c_size_t()
            check(lib().qvnt_workload_random_layers(self.n, d, ctypes.byref(st), None, 0, ctypes.byref(cnt)))
            counts.append(cnt.value)
            rng.state = st.value
        gates = (QvntGate * max(sum(counts), 1))()
        rng = SplitMix64(self.seed)
        at = 0
        calls = []
        for d, c, m, u in zip(self.depths, counts, self.masks, self.u01s):
            _c_layers(self.n, d, rng, gates, at)
            at += c
            calls.append(("apply", c))
            calls.append(("measure", m, u))
        return gates, calls


def serve_requests(rate=2000.0, duration=60.0, seed=5, q_range=(10, 28), depth_range=(5, 100)):
    """The serving workload: Poisson arrivals at `rate` per second over `duration` seconds; qubit
    count log-uniform in q_range, depth uniform in depth_range split over 1-3 rounds of apply then
    measure_mask (of 1-3 random qubits).  Yields ServeRequest in arrival order."""
    rng = SplitMix64(seed)
    t = 0.0
    lo, hi = math.log(q_range[0]), math.log(q_range[1] + 1)
    while True:
        t += -math.log(1.0 - rng.uniform()) / rate
        if t >= duration:
            return
        n = min(q_range[1], int(math.exp(lo + (hi - lo) * rng.uniform())))
        state = rng.below(1 << n)
        depth = depth_range[0] + rng.below(depth_range[1] - depth_range[0] + 1)
        rounds = min(depth, 1 + rng.below(3))
        cuts = sorted(rng.below(depth - 1) + 1 for _ in range(rounds - 1)) if rounds > 1 else []
        bounds = [0] + cuts + [depth]
        depths = [bounds[i + 1] - bounds[i] for i in range(rounds)]
        depths = [d for d in depths if d > 0] or [depth]
        masks, u01s = [], []
        for _ in depths:
            m = 0
            for _ in range(1 + rng.below(3)):
                m |= 1 << rng.below(n)
            masks.append(m)
            u01s.append(rng.uniform())
        yield ServeRequest(t, n, state, depths, masks, u01s, rng.next_u64())


def inverse(circuit):
    """The true inverse of a circuit.  qvnt's `.dgr()` maps a rotation R(theta) to -R(theta)
    (its stored phase is negated, src/operator/atomic/rx.rs:42-47), so it is not an inverse for
    rotations; here rotations are inverted by conjugating the stored phase instead."""
    out = []
    for s in reversed(circuit.ops):
        g = s.clone()
        if g.g.kind in (2, 3, 5, 6, 10, 11):  # RX RXX RY RYY RZ RZZ
            g.g.phase[1] = -g.g.phase[1]
        else:
            g = g.dgr()
        out.append(g)
    return MultiOp(out)


def _concat(ops):
    r = MultiOp()
    for o in ops:
        r = r * o
    return r
