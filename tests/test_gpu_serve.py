"""Serving form on the GPU: continuous admission with requests overlapping on the device.

Each request's measured values and final amplitudes are the same alone (one slot, one request at a
time) and in the mix (many slots, all submitted at once); the single-register engine driven directly
gives the same.  Admission keeps the running states inside the HBM budget."""
import itertools

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _requests(count, seed, q_range, depth_range):
    from qvnt_gb300.circuits import serve_requests

    return list(itertools.islice(serve_requests(rate=1000.0, duration=1e9, seed=seed, q_range=q_range,
                                                depth_range=depth_range), count))


def _run(server, reqs, keep=True):
    ids = []
    for r in reqs:
        gates, calls = r.build()
        ids.append(server.submit(r.n, r.state, gates, calls, keep_amplitudes=keep))
    return [server.wait(i, timeout=120.0) for i in ids]


def test_serve_alone_equals_mix():
    from qvnt_gb300.serve import Server

    reqs = _requests(14, 3, (10, 17), (2, 8))
    alone = []
    s1 = Server(budget_bytes=2 << 30, slots=1)
    for r in reqs:
        alone.extend(_run(s1, [r]))
    s1.close()
    s8 = Server(budget_bytes=2 << 30, slots=8)
    mix = _run(s8, reqs)
    st = s8.stats()
    s8.close()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    for (ra, aa, _), (rm, am, _) in zip(alone, mix):
        assert ra == rm
        assert np.max(np.abs(aa - am)) <= TOL


def test_serve_matches_register_engine():
    import ctypes

    from qvnt_gb300 import QReg
    from qvnt_gb300._abi import QvntGate
    from qvnt_gb300.serve import Server

    reqs = _requests(4, 8, (10, 14), (3, 6))
    s = Server(budget_bytes=1 << 30, slots=4)
    got = _run(s, reqs)
    s.close()
    for r, (res, amps, lat) in zip(reqs, got):
        gates, calls = r.build()
        q = QReg.with_state(r.n, r.state)
        at, want = 0, []
        for c in calls:
            if c[0] == "apply":
                ptr = ctypes.cast(ctypes.byref(gates, at * ctypes.sizeof(QvntGate)), ctypes.POINTER(QvntGate))
                q.apply_gates(ptr, c[1])
                at += c[1]
                want.append(0)
            else:
                want.append(q.measure_mask(c[1], u01=c[2]).get())
        assert res == want
        assert np.max(np.abs(amps - q.amplitudes())) <= TOL
        assert lat > 0


def test_serve_admission_respects_budget():
    from qvnt_gb300.serve import Server

    reqs = _requests(10, 11, (20, 20), (2, 3))
    budget = 3 * ((1 << 20) * 16 + (1 << 20)) + (1 << 20)  # three 20-qubit states
    s = Server(budget_bytes=budget, slots=8)
    ids = []
    for r in reqs:
        gates, calls = r.build()
        ids.append(s.submit(r.n, r.state, gates, calls))
    for i in ids:
        s.wait(i, timeout=120.0)
    st = s.stats()
    s.close()
    assert st["completed"] == len(reqs)
    assert 1 <= st["peak_running"] <= 3
    assert st["bytes_active"] == 0


def test_serve_sheds_and_rejects():
    from qvnt_gb300._abi import QvntError
    from qvnt_gb300.serve import Server

    reqs = _requests(40, 13, (18, 20), (20, 30))
    built = [r.build() for r in reqs]
    s = Server(budget_bytes=1 << 30, slots=1, max_queue=2)
    ids = [s.submit(r.n, r.state, g, c, detached=True) for r, (g, c) in zip(reqs, built)]
    assert any(i is None for i in ids)  # the queue of two filled up: requests were shed
    st = s.stats()
    assert st["shed"] == sum(1 for i in ids if i is None)
    with pytest.raises(QvntError):
        s.submit(10, 1 << 10, None, [])  # basis state outside the register
    with pytest.raises(QvntError):
        s.submit(10, 0, None, [("measure", 1 << 12, 0.5)])  # mask outside the register
    s.close()


def test_serve_wire_request_vs_oracle():
    """A serving request received as a binary QVNW stream (gate records and calls, CRC-checked) is
    decoded by Server.submit_request, run on the device, and matches the oracle driving qvnt's
    QReg::with_state / apply / measure_mask (src/register/quant.rs:129-150, :376-395, :490-501) with
    the same gates and draws: identical measured values, final amplitudes within 1e-12."""
    import oracle_ref as orc
    from qvnt_gb300 import op
    from qvnt_gb300.circuits import random_circuit
    from qvnt_gb300.serve import Server
    from qvnt_gb300.wire import decode_request, encode_request

    n, state = 12, 0b101100111010
    ops = random_circuit(n, 3, seed=41, with_qft=False) * op.qft(0b111111) * op.h(0b1010).c(0b100000000)
    cut = len(ops) // 2
    calls = [("apply", cut), ("measure", 0b11, 0.61), ("apply", len(ops) - cut), ("measure", 0b1100000, 0.27)]
    data = encode_request(n, state, ops, calls, keep_amplitudes=True)
    assert decode_request(data)["calls"] == calls
    s = Server(budget_bytes=1 << 30, slots=2)
    rid = s.submit_request(data)
    measured, amps, _ = s.wait(rid, timeout=60.0)
    s.close()
    gates = ops.gates()
    psi = orc.new_state(n, state)
    want, at = [], 0
    for c in calls:
        if c[0] == "apply":
            orc.apply(gates[at:at + c[1]], psi)
            at += c[1]
            want.append(0)
        else:
            v, _ = orc.measure_mask(psi, n, c[1], c[2])
            want.append(v)
    assert [int(m) for m in measured] == want
    assert np.max(np.abs(amps - psi)) <= TOL
