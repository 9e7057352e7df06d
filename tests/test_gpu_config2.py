"""Config 2 pinned against the oracle at its own depth: the seeded random circuit (depth 40 of
{h, s, t, u3} layers, 15 two-qubit gates and 3 Toffolis per layer, then op::qft over all qubits) at
26 qubits, compared with the oracle's result committed in tests/golden/config2_26q.npz (written by
tests/golden/make_config2.py; the oracle runs qvnt's MultiOp::apply, src/operator/multi/mod.rs:97-114,
one gather pass per gate as in src/operator/atomic/dispatch.rs:32-67).

Bars: the PLAIN engine is bit-identical (sampled amplitudes, chunk norms, the sum of all amplitudes,
the measured index for every draw).  The TENSOR64 engine (the headline f64 engine) is within 1e-12
max-abs and within REL_T64 of the largest sampled amplitude.  The FUSED (double-float) engine is
within 1e-12 max-abs and, relative to the largest sampled amplitude, within REL_FUSED.  Both
relative bounds are set from the measured errors, so that a regression of a few bits shows up.
"""
import hashlib
import os

import numpy as np
import pytest

from qvnt_gb300 import ENGINE_FUSED, ENGINE_PLAIN, ENGINE_TENSOR64, QReg
from qvnt_gb300.circuits import random_circuit

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "config2_26q.npz")
ABS_TOL = 1e-12
REL_FUSED = 1e-12  # measured 2.05e-13 at 26 qubits (2,633 gates)
REL_T64 = 2e-13  # measured 1.16e-13 at 26 qubits (288-block plan)


@pytest.fixture(scope="module")
def fixture():
    f = np.load(FIXTURE)
    return {k: f[k] for k in f.files}


@pytest.fixture(scope="module")
def circuit(fixture):
    n, depth, seed = int(fixture["qubits"]), int(fixture["depth"]), int(fixture["seed"])
    circ = random_circuit(n, depth, seed=seed)
    gates = circ.gates()
    assert len(gates) == int(fixture["gate_count"])
    assert hashlib.sha256(b"".join(bytes(g) for g in gates)).hexdigest() == str(fixture["gates_sha256"])
    return circ


def run(fixture, circuit, engine):
    n = int(fixture["qubits"])
    q = QReg.new(n)
    q.set_engine(engine)
    q.apply(circuit)
    return q


def errors(psi, fixture):
    idx = fixture["idx"].astype(np.int64)
    d = np.abs(psi[idx] - fixture["amp"])
    return float(d.max()), float(d.max() / np.abs(fixture["amp"]).max())


def check_measure(q, fixture, exact):
    n = int(fixture["qubits"])
    mask = (1 << n) - 1
    for u, want in zip(fixture["draws"], fixture["chosen"]):
        r = q.clone()
        got = r.measure_mask(mask, float(u)).get()
        r.close()
        if exact:
            assert got == int(want), (u, got, int(want))
        elif got != int(want):
            # a different index only where the draw sits on a cumulative-probability boundary
            p = q.get_probabilities()
            cum = np.cumsum(p)
            lo, hi = sorted((got, int(want)))
            assert abs(cum[hi - 1] - float(u) * cum[-1]) < 1e-12, (u, got, int(want))


def test_plain_engine_bit_identical(fixture, circuit):
    q = run(fixture, circuit, ENGINE_PLAIN)
    psi = q.amplitudes()
    idx = fixture["idx"].astype(np.int64)
    assert np.array_equal(psi[idx], fixture["amp"])
    n = int(fixture["qubits"])
    chunks = (np.abs(psi[: 1 << n].reshape(256, -1)) ** 2).sum(axis=1)
    assert np.array_equal(chunks, fixture["chunk_norms"])
    assert psi.sum() == complex(fixture["psi_sum"])
    # get_absolute sums in chunks; the oracle's left-to-right loop over 2^26 terms carries ~1e-13 of
    # its own rounding, so the check is against the chunk norms' pairwise total
    assert abs(q.get_absolute() - float(fixture["chunk_norms"].sum())) <= 1e-14
    assert abs(q.get_absolute() - float(fixture["norm"])) <= 1e-12
    check_measure(q, fixture, exact=True)
    q.close()


def test_fused_engine_within_tolerance(fixture, circuit):
    q = run(fixture, circuit, ENGINE_FUSED)
    psi = q.amplitudes()
    mx, rel = errors(psi, fixture)
    print("fused config 2 at %d qubits: max-abs %.3e, relative to max |psi| %.3e" % (int(fixture["qubits"]), mx, rel))
    assert mx <= ABS_TOL and rel <= REL_FUSED
    n = int(fixture["qubits"])
    chunks = (np.abs(psi[: 1 << n].reshape(256, -1)) ** 2).sum(axis=1)
    assert np.max(np.abs(chunks - fixture["chunk_norms"])) <= 1e-13
    # double-float rounding drifts the norm (measured 1.5e-13 here)
    assert abs(q.get_absolute() - float(fixture["chunk_norms"].sum())) <= 1e-12
    check_measure(q, fixture, exact=False)
    q.close()


def test_tensor64_engine_within_tolerance(fixture, circuit):
    q = run(fixture, circuit, ENGINE_TENSOR64)
    psi = q.amplitudes()
    mx, rel = errors(psi, fixture)
    print("tensor64 config 2 at %d qubits: max-abs %.3e, relative to max |psi| %.3e" % (int(fixture["qubits"]), mx, rel))
    assert mx <= ABS_TOL and rel <= REL_T64
    n = int(fixture["qubits"])
    chunks = (np.abs(psi[: 1 << n].reshape(256, -1)) ** 2).sum(axis=1)
    assert np.max(np.abs(chunks - fixture["chunk_norms"])) <= 1e-13
    assert abs(q.get_absolute() - float(fixture["chunk_norms"].sum())) <= 1e-13
    check_measure(q, fixture, exact=False)
    q.close()
