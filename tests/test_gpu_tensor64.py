"""The TENSOR64 engine (dense 5-qubit blocks on the tensor cores, 53-bit operands split into exact
fp16 digit products, IEEE f64 storage) against the CPU oracle (qvnt's MultiOp::apply,
src/operator/multi/mod.rs:97-114, and AtomicOp::for_each, src/operator/atomic/dispatch.rs:32-67).

Bar: within 1e-12 max-abs and within REL of the largest amplitude (a bound set from the measured
error of the engine: one rounding of each block's inputs to 53 bits and one rounding to f64 per
block).  Registers below 12 qubits run on the plain kernels and stay bit-identical.
"""
import numpy as np
import pytest

import oracle_ref as orc
from qvnt_gb300 import ENGINE_PLAIN, ENGINE_TENSOR64, QReg, op
from qvnt_gb300.circuits import plain_circuit, random_circuit
from test_gpu_parity import all_kinds_circuit

pytestmark = pytest.mark.gpu

TOL = 1e-12
REL = 2e-13


def run(n, state, circ, engine=ENGINE_TENSOR64):
    q = QReg.with_state(n, state)
    q.set_engine(engine)
    q.apply(circ)
    return q


def oracle(n, state, circ):
    psi = orc.new_state(n, state)
    orc.apply(circ.gates(), psi)
    return psi


def close(got, want):
    d = float(np.max(np.abs(got - want)))
    scale = float(np.max(np.abs(want)))
    return d, d / scale


@pytest.mark.parametrize("n", [12, 13, 14, 17])
def test_random_all_kinds_vs_oracle(n):
    """Every gate kind, multi-bit masks, controls (gates wider than five qubits run as plain passes)."""
    circ = all_kinds_circuit(n, 300, seed=500 + n, ctrl_prob=0.4)
    want = oracle(n, 12345 % (1 << n), circ)
    got = run(n, 12345 % (1 << n), circ).amplitudes()
    d, rel = close(got, want)
    print("tensor64 all kinds n=%d: max-abs %.3e rel %.3e" % (n, d, rel))
    assert d <= TOL and rel <= REL


@pytest.mark.parametrize("n", [3, 7, 11])
def test_small_registers_plain_exact(n):
    circ = all_kinds_circuit(n, 100, seed=n)
    assert np.array_equal(run(n, 1, circ).amplitudes(), oracle(n, 1, circ))


def test_config1_20q():
    """Config 1 (QReg::new(20), h(all), 20 rx/ry/rz + CNOT layers, qft) against the oracle, then
    measure_mask(0xFFFFF) with injected draws."""
    circ = plain_circuit(20, 20, seed=1)
    want = oracle(20, 0, circ)
    q = run(20, 0, circ)
    got = q.amplitudes()
    d, rel = close(got, want)
    print("tensor64 config 1: max-abs %.3e rel %.3e" % (d, rel))
    assert d <= TOL and rel <= REL
    for u in (0.0, 0.123456789, 0.5, 0.987654321):
        r = q.clone()
        v = r.measure_mask(0xFFFFF, u).get()
        ov, _ = orc.measure_mask(want.copy(), 20, 0xFFFFF, u)
        if v != ov:
            cum = np.cumsum(orc.get_probabilities(want, 20))
            assert abs(cum[min(v, ov)] - u * cum[-1]) < 1e-12 or abs(cum[max(v, ov) - 1] - u * cum[-1]) < 1e-12
        r.close()


def test_sparse_and_scaled_states():
    """Rows of zeros, a basis state, and a state scaled far from norm 1 (the row exponents carry it)."""
    n = 14
    circ = random_circuit(n, 3, seed=9)
    for state in (0, 5, (1 << n) - 1):
        got = run(n, state, circ).amplitudes()
        d, rel = close(got, oracle(n, state, circ))
        assert d <= TOL and rel <= REL
    rng = np.random.default_rng(3)
    psi = (rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)) * 1e-100
    psi[rng.integers(0, 1 << n, 64)] = 0.0
    q = QReg.new(n)
    q.set_engine(ENGINE_TENSOR64)
    q.set_amplitudes(psi)
    q.apply(circ)
    want = psi.copy()
    orc.apply(circ.gates(), want)
    d, rel = close(q.amplitudes(), want)
    assert rel <= REL


def test_split_calls_and_plain_switch():
    """Applying a circuit in pieces, switching to the plain engine in between (same storage)."""
    n = 15
    circ = random_circuit(n, 6, seed=21)
    ops = circ.ops
    half = len(ops) // 2
    from qvnt_gb300.operator import MultiOp
    q = QReg.new(n)
    q.set_engine(ENGINE_TENSOR64)
    q.apply(MultiOp(ops[:half]))
    q.set_engine(ENGINE_PLAIN)
    q.apply(MultiOp(ops[half:half + 10]))
    q.set_engine(ENGINE_TENSOR64)
    q.apply(MultiOp(ops[half + 10:]))
    d, rel = close(q.amplitudes(), oracle(n, 0, circ))
    assert d <= TOL and rel <= REL


def test_apply_host_on_tensor64():
    from qvnt_gb300 import Context
    ctx = Context(0)
    ctx.set_engine(ENGINE_TENSOR64)
    n = 16
    circ = random_circuit(n, 4, seed=4) * op.h(0b1011)
    psi = orc.new_state(n, 7)
    out = ctx.apply_host(circ, psi)
    d, rel = close(out, oracle(n, 7, circ))
    assert d <= TOL and rel <= REL
    ctx.close()
