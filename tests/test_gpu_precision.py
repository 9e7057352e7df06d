"""Precision engine on the GPU: complex<f32> states, dense 5-qubit blocks on the tcgen05 tensor
cores (TF32 hi/lo split, FP32 accumulation), FP64 norms and measurement.

Tolerance: fidelity defect 1 - |<plain|precision>|^2 <= 1e-5 against the plain f64 engine (bit-exact
with the oracle), and max-abs amplitude error <= 1e-5."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DEFECT = 1e-5
MAXABS = 1e-5


def _mixed_circuit(n, count, seed):
    """Every gate kind with supports (targets and controls) of at most five qubits."""
    from qvnt_gb300 import operator as op
    from qvnt_gb300.circuits import SplitMix64
    from qvnt_gb300.operator import MultiOp, SingleOp

    rng = SplitMix64(seed)

    def bits(k):
        qs = []
        while len(qs) < k:
            b = rng.below(n)
            if b not in qs:
                qs.append(b)
        return qs

    ops = []
    while len(ops) < count:
        kind = rng.below(20)
        qs = bits(5)
        ctrl = (1 << qs[4]) if rng.below(3) == 0 else 0
        s = None
        if kind in (1, 4, 7, 8, 9):
            m = (1 << qs[0]) | ((1 << qs[1]) if rng.below(2) else 0) | ((1 << qs[2]) if rng.below(2) else 0)
            s = SingleOp._make(["ID", "X", "", "", "Y", "", "", "Z", "S", "T"][kind], m)
        elif kind in (2, 5, 10, 14):
            s = SingleOp._make({2: "RX", 5: "RY", 10: "RZ", 14: "H1"}[kind], 1 << qs[0], 0, 6.283 * rng.uniform())
        elif kind in (3, 6, 11, 16, 17, 18, 19):
            name = {3: "RXX", 6: "RYY", 11: "RZZ", 16: "SWAP", 17: "ISWAP", 18: "SQRT_SWAP", 19: "SQRT_ISWAP"}[kind]
            s = SingleOp._make(name, (1 << qs[0]) | (1 << qs[1]), 0, 6.283 * rng.uniform())
        elif kind == 12:
            th, ph = rng.uniform() * 3, rng.uniform() * 6
            m = [math.cos(th), -np.exp(1j * ph) * math.sin(th), math.sin(th), np.exp(1j * ph) * math.cos(th)]
            s = op.u1_matrix(1 << qs[0], m)
        elif kind == 13:
            hh = 1 / math.sqrt(2)
            m = [hh, hh, 0, 0, hh, -hh, 0, 0, 0, 0, 1j * hh, 1j * hh, 0, 0, hh, -hh]
            s = op.u2_matrix(1 << qs[0], 1 << qs[1], m)
        elif kind == 15:
            s = SingleOp._make("H2", 1 << qs[0], 1 << qs[1])
        if s is None:
            continue
        if ctrl and rng.below(2):
            s = s.c(ctrl)
        if s is not None:
            ops.append(s)
    if rng.below(2) == 0:
        pass
    return MultiOp(ops)


def _pair(n, circuit, state=0):
    from qvnt_gb300 import ENGINE_PLAIN, ENGINE_PRECISION, QReg

    ref = QReg(n, state, engine=ENGINE_PLAIN)
    ref.apply(circuit)
    q = QReg(n, state, engine=ENGINE_PRECISION)
    q.apply(circuit)
    return ref, q


@pytest.mark.parametrize("n,depth", [(12, 3), (14, 6), (17, 4)])
def test_precision_random_layers(n, depth):
    from qvnt_gb300.circuits import random_circuit

    c = random_circuit(n, depth, seed=40 + n)  # layers and qft
    ref, q = _pair(n, c)
    fid, mx = q.overlap(ref)
    assert 1.0 - fid <= DEFECT, (n, fid)
    assert mx <= MAXABS, (n, mx)
    assert abs(q.get_absolute() - 1.0) <= 1e-6


def test_precision_every_gate_kind():
    c = _mixed_circuit(13, 300, seed=9)
    ref, q = _pair(13, c, state=77)
    fid, mx = q.overlap(ref)
    assert 1.0 - fid <= DEFECT, fid
    assert mx <= MAXABS, mx
    # the amplitudes themselves
    a, b = q.amplitudes(), ref.amplitudes()
    assert np.max(np.abs(a - b)) <= MAXABS


def test_precision_measure_and_unnormalised_state():
    from qvnt_gb300.circuits import random_circuit

    c = random_circuit(13, 4, seed=5)
    ref, q = _pair(13, c)
    for u in (0.1, 0.37, 0.8):
        r1 = ref.clone()
        r2 = q.clone()
        assert r1.measure_mask(0b101101, u01=u).get() == r2.measure_mask(0b101101, u01=u).get()
    # measure_mask leaves the state unnormalised; a later apply keeps that norm (qvnt semantics)
    v = q.measure_mask(0b11, u01=0.6).get()
    assert ref.measure_mask(0b11, u01=0.6).get() == v
    before = q.get_absolute()
    q.apply(c)
    ref.apply(c)
    assert abs(q.get_absolute() - before) <= 1e-6 * before
    fid, mx = q.overlap(ref)
    assert 1.0 - fid <= DEFECT and mx <= MAXABS


def test_precision_engine_switch_round_trip():
    from qvnt_gb300 import ENGINE_FUSED, ENGINE_PRECISION, QReg
    from qvnt_gb300.circuits import random_circuit

    c = random_circuit(12, 3, seed=8)
    q = QReg(12, 5, engine=ENGINE_FUSED)
    q.apply(c)
    keep = q.amplitudes()
    q.set_engine(ENGINE_PRECISION)
    assert np.max(np.abs(q.amplitudes() - keep)) <= 1e-7
    q.set_engine(ENGINE_FUSED)
    assert np.max(np.abs(q.amplitudes() - keep)) <= 1e-7


def test_precision_rejects_small_and_wide():
    from qvnt_gb300 import ENGINE_PRECISION, QReg
    from qvnt_gb300 import operator as op
    from qvnt_gb300._abi import QvntError

    q = QReg(8, 0, engine=ENGINE_PRECISION)
    with pytest.raises(QvntError):
        q.apply(op.h(1))  # below 12 qubits
    q = QReg(12, 0, engine=ENGINE_PRECISION)
    with pytest.raises(QvntError):
        q.apply(op.x(1).c(0b111110))  # six qubits in one gate
