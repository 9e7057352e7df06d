"""The dense-block planner of the TENSOR64 and precision engines, checked on the CPU: the blocks it
returns (qvnt_dense_plan_blocks: supports and 32 x 32 unitaries, in order), applied to a random state
with numpy, equal the oracle's gate-by-gate f64 result (qvnt's MultiOp::apply,
src/operator/multi/mod.rs:97-114) within 1e-13 of the largest amplitude.  This pins the planner's
reordering (gates commute past skipped ones only when their supports are disjoint or both are
diagonal) and its matrix products without a GPU."""
import ctypes

import numpy as np
import pytest

import oracle_ref as orc
from qvnt_gb300 import op
from qvnt_gb300._abi import QvntGate, lib
from qvnt_gb300.circuits import plain_circuit, random_circuit


def plan(gates, n):
    arr = (QvntGate * len(gates))(*gates)
    nb = ctypes.c_size_t()
    assert lib().qvnt_dense_plan_blocks(arr, len(gates), n, None, None, 0, ctypes.byref(nb)) == 0
    sups = (ctypes.c_uint64 * nb.value)()
    mats = (ctypes.c_double * (2048 * nb.value))()
    assert lib().qvnt_dense_plan_blocks(arr, len(gates), n, sups, mats, nb.value, ctypes.byref(nb)) == 0
    u = np.frombuffer(mats, dtype=np.float64).view(np.complex128).reshape(nb.value, 32, 32)
    return list(sups), u


def apply_blocks(psi, sups, mats, n):
    psi = psi.copy()
    for sup, u in zip(sups, mats):
        qs = [q for q in range(n) if (sup >> q) & 1]
        assert len(qs) == 5
        spread = np.array([sum(((c >> j) & 1) << q for j, q in enumerate(qs)) for c in range(32)], dtype=np.int64)
        rest = np.array([i for i in range(1 << n) if not i & sup], dtype=np.int64)
        idx = rest[:, None] | spread[None, :]
        psi[idx] = psi[idx] @ u.T
    return psi


@pytest.mark.parametrize("name, n", [("random", 12), ("random", 13), ("plain", 12)])
def test_blocks_reproduce_the_circuit(name, n):
    circ = random_circuit(n, 6, seed=40 + n) if name == "random" else plain_circuit(n, 4, seed=n)
    circ = circ * op.x(0b1011) * op.s(0b110000) * op.h(0b111)  # multi-bit gates, split into factors
    gates = circ.gates()
    sups, mats = plan(gates, n)
    assert len(sups) < len(gates)
    eye = np.eye(32)
    for u in mats:
        assert np.max(np.abs(u @ u.conj().T - eye)) < 1e-13
    rng = np.random.default_rng(n)
    psi = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    psi /= np.linalg.norm(psi)
    want = psi.copy()
    orc.apply(gates, want)
    got = apply_blocks(psi, sups, mats, n)
    assert np.max(np.abs(got - want)) <= 1e-13 * np.max(np.abs(want))


def test_wide_gate_is_rejected():
    gates = (op.x(1).c(0b111110)).gates()  # 6 qubits with its controls
    arr = (QvntGate * len(gates))(*gates)
    nb = ctypes.c_size_t()
    assert lib().qvnt_dense_plan_blocks(arr, len(gates), 8, None, None, 0, ctypes.byref(nb)) != 0
