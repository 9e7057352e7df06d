"""GPU parity: the engine's kernels against the CPU oracle, through the C ABI.

Bar: the PLAIN engine (one pass per SingleOp, qvnt's operand order, no FMA contraction) is
bit-identical to the oracle; the FUSED engine agrees within 1e-12 max-abs on every amplitude
(the f64 tolerance this engine is built to) and within REL of the largest amplitude, a bound set
from its measured error so that a loss of a few bits fails.  Measured indices are identical given the same draw,
except where the draw falls within 1e-12 of a cumulative-probability boundary.
"""
import math

import numpy as np
import pytest

import oracle_ref as orc
from qvnt_gb300 import ENGINE_FUSED, ENGINE_PLAIN, MaskError, QReg, op
from qvnt_gb300.circuits import SplitMix64, inverse, plain_circuit, random_circuit
from qvnt_gb300.operator import MultiOp, SingleOp

pytestmark = pytest.mark.gpu

TOL = 1e-12
REL = 5e-13  # measured up to 1.3e-13 on these circuits
ENGINES = [ENGINE_PLAIN, ENGINE_FUSED]


def assert_close(got, want):
    """max|got - want| <= TOL and <= REL * max|want|."""
    d = float(np.max(np.abs(got - want)))
    scale = float(np.max(np.abs(want)))
    print("fused vs oracle: max-abs %.3e, relative %.3e" % (d, d / scale if scale else d))
    assert d <= TOL and d <= REL * scale, (d, d / scale if scale else d)


def run_gpu(n, state, circuit, engine, k=None):
    q = QReg.with_state(n, state)
    q.set_engine(engine)
    if k:
        q.set_fusion_width(k)
    q.apply(circuit)
    return q


def run_oracle(n, state, circuit):
    psi = orc.new_state(n, state)
    orc.apply(circuit.gates(), psi)
    return psi


def cplx(m):
    return np.array([[complex(z[0], z[1]) for z in row] for row in m])


def all_kinds_circuit(n, count, seed, ctrl_prob=0.3):
    """Random gates of all 20 kinds with random multi-bit masks and controls."""
    rng = SplitMix64(seed)
    ops = []

    def bits(k):
        assert k <= n, "circuit needs %d distinct qubits of %d" % (k, n)
        qs = []
        while len(qs) < k:
            b = rng.below(n)
            if b not in qs:
                qs.append(b)
        return qs

    while len(ops) < count:
        kind = rng.below(20)
        s = None
        if kind in (1, 4, 7, 8, 9):  # X Y Z S T: any mask
            m = rng.next_u64() & ((1 << n) - 1)
            s = SingleOp._make(["ID", "X", "", "", "Y", "", "", "Z", "S", "T"][kind], m)
        elif kind in (2, 5, 10, 14):
            a, = bits(1)
            s = SingleOp._make({2: "RX", 5: "RY", 10: "RZ", 14: "H1"}[kind], 1 << a, 0, 6.283 * rng.uniform())
        elif kind in (3, 6, 11, 16, 17, 18, 19):
            a, b = bits(2)
            name = {3: "RXX", 6: "RYY", 11: "RZZ", 16: "SWAP", 17: "ISWAP", 18: "SQRT_SWAP", 19: "SQRT_ISWAP"}[kind]
            s = SingleOp._make(name, (1 << a) | (1 << b), 0, 6.283 * rng.uniform())
        elif kind == 12:
            a, = bits(1)
            th, ph = rng.uniform() * 3, rng.uniform() * 6
            m = [math.cos(th), -np.exp(1j * ph) * math.sin(th), math.sin(th), np.exp(1j * ph) * math.cos(th)]
            s = op.u1_matrix(1 << a, m)
        elif kind == 13:
            a, b = bits(2)
            hh = 1 / math.sqrt(2)
            m = [hh, hh, 0, 0, hh, -hh, 0, 0, 0, 0, 1j * hh, 1j * hh, 0, 0, hh, -hh]
            s = op.u2_matrix(1 << a, 1 << b, m)
        elif kind == 15:
            a, b = bits(2)
            s = SingleOp._make("H2", 1 << a, 1 << b)
        else:
            continue
        if s is None:
            continue
        if rng.below(4) == 0:
            s = s.dgr()
        if rng.uniform() < ctrl_prob:
            free = [b for b in range(n) if not (s.act_on() >> b) & 1]
            if free:
                c = 1 << free[rng.below(len(free))]
                if rng.below(3) == 0 and len(free) > 1:
                    c |= 1 << free[rng.below(len(free))]
                cs = s.c(c)
                if cs is not None:
                    s = cs
        ops.append(s)
    return MultiOp(ops)


@pytest.mark.parametrize("engine", ENGINES)
def test_matrix_repr_on_gpu(golden, engine):
    for case in golden["matrix_cases"]:
        ops = []
        for spec in case["gates"]:
            m = spec["matrix"]
            s = SingleOp._make(spec["kind"], spec["a"], spec["b"], spec["angle"],
                               None if m is None else [complex(m[2 * i], m[2 * i + 1]) for i in range(len(m) // 2)])
            if spec["dgr"]:
                s = s.dgr()
            ops.append(s)
        size = case["size"]
        dim = 1 << size
        got = np.zeros((dim, dim), dtype=np.complex128)
        for c in range(dim):
            q = QReg.with_state(size, c)
            q.set_engine(engine)
            q.apply(MultiOp(ops))
            got[:, c] = q.amplitudes()[:dim]
        want = cplx(case["matrix"])
        if engine == ENGINE_PLAIN:
            assert np.array_equal(got, want), case["cite"]
        else:
            assert_close(got, want)


@pytest.mark.parametrize("engine", ENGINES)
def test_quantum_reg_vector(golden, engine):
    case = golden["register_cases"][0]
    q = QReg.with_state(case["q_num"], case["state"])
    q.set_engine(engine)
    ops = op.h(0b1111) * op.h(0b0011).c(0b1000) * op.swap(0b1001).c(0b0010)
    assert repr(ops) == case["names"]
    q.apply(ops)
    want = np.array([complex(a, b) for a, b in case["psi"]])
    got = q.amplitudes()
    if engine == ENGINE_PLAIN:
        assert np.array_equal(got, want)
    else:
        assert_close(got, want)
    mask = case["measure_mask"]
    for u in (0.0, 0.3, 0.77, 0.999):
        r = q.clone()
        assert r.measure_mask(mask, u).get() & ~mask == 0


@pytest.mark.parametrize("n", [1, 2, 3, 5, 9, 12])
@pytest.mark.parametrize("engine", ENGINES)
def test_random_all_kinds(n, engine):
    # registers below 3 qubits keep 8 amplitudes (quant.rs:15): their gates may use the padding bits
    circ = all_kinds_circuit(max(n, 3), 150, seed=100 + n)
    state = 0x0B4B4B4B & ((1 << n) - 1)
    want = run_oracle(n, state, circ)
    got = run_gpu(n, state, circ, engine).amplitudes()
    if engine == ENGINE_PLAIN:
        assert np.array_equal(got, want)
    else:
        assert_close(got, want)


@pytest.mark.parametrize("k", [6, 8, 10, 13])
def test_fused_widths(k):
    n = 14
    circ = all_kinds_circuit(n, 400, seed=77, ctrl_prob=0.5)
    want = run_oracle(n, 12345, circ)
    got = run_gpu(n, 12345, circ, ENGINE_FUSED, k=k).amplitudes()
    assert_close(got, want)


@pytest.mark.parametrize("engine", ENGINES)
def test_plain_circuit_20q(engine):
    """Config 1: QReg::new(20), h(all), 20 layers of rx/ry/rz + NN CNOTs, qft(all); before measuring."""
    circ = plain_circuit(20, 20, seed=1)
    want = run_oracle(20, 0, circ)
    q = run_gpu(20, 0, circ, engine)
    got = q.amplitudes()
    if engine == ENGINE_PLAIN:
        assert np.array_equal(got, want)
    else:
        assert_close(got, want)
    # measure_mask(0xFFFFF) with injected draws, against the oracle on the same state
    for u in (0.0, 0.123456789, 0.5, 0.987654321):
        r = q.clone()
        v = r.measure_mask(0xFFFFF, u).get()
        p = want.copy()
        ov, oidx = orc.measure_mask(p, 20, 0xFFFFF, u)
        if v != ov:
            probs = orc.get_probabilities(want, 20)
            cum = np.cumsum(probs)
            chosen = u * cum[-1]
            assert min(abs(cum[min(v, ov)] - chosen), abs(cum[max(v, ov) - 1] - chosen)) < 1e-12
        else:
            got_c = r.amplitudes()
            assert np.max(np.abs(got_c - p)) <= (0 if engine == ENGINE_PLAIN else TOL)


def test_random_circuit_22q_plain_vs_oracle():
    """Config-2 gate mix (h, s, t, u3, rxx/ryy/rzz, swap/i_swap/sqrt_i_swap, Toffoli, qft) at 22 qubits."""
    circ = random_circuit(22, 8, seed=3)
    want = run_oracle(22, 0, circ)
    got = run_gpu(22, 0, circ, ENGINE_PLAIN).amplitudes()
    assert np.array_equal(got, want)
    got_f = run_gpu(22, 0, circ, ENGINE_FUSED).amplitudes()
    assert_close(got_f, want)


def test_register_passes_vs_oracle():
    n = 13
    circ = all_kinds_circuit(n, 200, seed=5)
    q = run_gpu(n, 77, circ, ENGINE_PLAIN)
    psi = run_oracle(n, 77, circ)
    assert np.array_equal(q.get_probabilities(), orc.get_probabilities(psi, n)) or \
        np.max(np.abs(q.get_probabilities() - orc.get_probabilities(psi, n))) <= 1e-15
    assert abs(q.get_absolute() - orc.get_absolute(psi)) <= 1e-13
    pol = q.get_polar()
    opol = orc.get_polar(psi, n)
    assert np.max(np.abs(pol[:, 0] - opol[:, 0])) <= 1e-15
    big = opol[:, 0] > 1e-12
    d = np.abs(np.angle(np.exp(1j * (pol[big, 1] - opol[big, 1]))))
    assert np.max(d) <= 1e-12
    # reset_by_mask (zero + normalize) and normalize thresholds
    r = q.clone()
    r.reset_by_mask(0b101)
    p2 = orc.reset_by_mask(psi.copy(), n, 0b101)
    assert np.max(np.abs(r.amplitudes() - p2)) <= 1e-15
    r.reset_by_mask((1 << n) - 1)
    assert np.array_equal(r.amplitudes(), orc.new_state(n, 0))
    r = q.clone()
    r.reset(5)
    assert np.array_equal(r.amplitudes(), orc.new_state(n, 5))


def test_tensor_vs_oracle(golden):
    for case in golden["tensor_cases"]:
        a, b = case["a"], case["b"]
        qa = QReg.with_state(a["q_num"], a["state"])
        qa.apply(op.h(a["h"]))
        qb = QReg.with_state(b["q_num"], b["state"])
        qb.apply(op.h(b["h"]))
        t = qa * qb
        assert np.all(np.abs(t.get_probabilities() - np.array(case["prob"])) < case["eps"])
    for na, nb in ((3, 4), (1, 2), (5, 6)):
        # registers below 3 qubits hold 8 amplitudes: their gates may use the padding bits
        ca = all_kinds_circuit(max(na, 3), 30, seed=na)
        cb = all_kinds_circuit(max(nb, 3), 30, seed=nb + 50)
        qa, qb = run_gpu(na, 1, ca, ENGINE_PLAIN), run_gpu(nb, 2, cb, ENGINE_PLAIN)
        pa, pb = run_oracle(na, 1, ca), run_oracle(nb, 2, cb)
        assert np.array_equal((qa * qb).amplitudes(), orc.tensor(pa, na, pb, nb))


def test_measure_many_draws_vs_oracle():
    n = 11
    circ = all_kinds_circuit(n, 120, seed=9)
    base = run_gpu(n, 0, circ, ENGINE_PLAIN)
    psi = run_oracle(n, 0, circ)
    rng = SplitMix64(4)
    for _ in range(40):
        u = rng.uniform()
        mask = rng.next_u64() & ((1 << n) - 1) or 1
        r = base.clone()
        v = r.measure_mask(mask, u).get()
        p = psi.copy()
        ov, oidx = orc.measure_mask(p, n, mask, u)
        assert v == ov
        assert np.array_equal(r.amplitudes(), p)  # collapse leaves the state unnormalised, as qvnt
    # mask outside the register measures nothing (quant.rs:491-494)
    r = base.clone()
    assert r.measure_mask(1 << 20, 0.5).get() == 0
    assert np.array_equal(r.amplitudes(), base.amplitudes())


def test_measure_renormalise_option():
    q = QReg.new(6)
    q.apply(op.h(0b111111))
    q.measure_mask(0b11, 0.4, renormalise=True)
    assert abs(q.get_absolute() - 1.0) < 1e-14


def test_errors_leave_state_unchanged():
    q = QReg.new(5)
    q.apply(op.h(0b11111))
    before = q.amplitudes()
    with pytest.raises(MaskError):
        q.apply(op.x(1 << 5))  # beyond the register: qvnt panics on psi[idx ^ mask]
    bad = op.rx(1.0, 1).ops[0].clone()
    bad.g.ctrl = 1  # ctrl overlapping act
    with pytest.raises(MaskError):
        q.apply(op.h(1) * bad)
    assert np.array_equal(q.amplitudes(), before)
    with pytest.raises(Exception):
        q.measure_mask(1, 1.5)


def test_u2_controlled_on_b_quirk():
    # u2 `acts_on` returns only a_mask (u2.rs:70-72), so qvnt lets a control share b's qubit
    hh = 1 / math.sqrt(2)
    m = [hh, hh, 0, 0, hh, -hh, 0, 0, 0, 0, hh, hh, 0, 0, hh, -hh]
    s = op.u2_matrix(0b01, 0b10, m)
    cs = s.c(0b10)
    assert cs is not None
    circ = op.h(0b111) * MultiOp([cs]) * op.rx(0.3, 0b100)
    for engine in ENGINES:
        got = run_gpu(3, 0, circ, engine).amplitudes()
        want = run_oracle(3, 0, circ)
        assert np.max(np.abs(got - want)) <= (0 if engine == ENGINE_PLAIN else TOL)


def test_small_register_padding():
    # QReg::new(1) keeps 8 amplitudes; x on a padding bit moves amplitude there (quant.rs:113-150)
    for engine in ENGINES:
        q = QReg.new(1)
        q.set_engine(engine)
        q.apply(op.x(0b100))
        a = q.amplitudes()
        assert a.size == 8 and a[4] == 1.0
        assert np.array_equal(q.get_probabilities(), np.zeros(2))


def test_apply_host_plugin_matches_register():
    n = 12
    circ = all_kinds_circuit(n, 100, seed=31)
    psi_i = orc.new_state(n, 3)
    from qvnt_gb300 import default_context
    out = default_context().apply_host(circ, psi_i)
    want = run_oracle(n, 3, circ)
    assert_close(out, want)


def test_full_size_round_trip_30q():
    """Config 2 at full size (30 qubits, depth 40 + qft): the circuit followed by its inverse returns
    |0> and keeps the norm -- size-independent properties of a correct unitary pass sequence."""
    circ = random_circuit(30, 40, seed=2)
    q = QReg.new(30)
    q.apply(circ)
    assert abs(q.get_absolute() - 1.0) < 1e-11
    q.apply(inverse(circ))
    a0 = q.amplitudes_range(0, 1)[0]
    assert abs(a0 - 1.0) < 1e-10
    assert abs(q.get_absolute() - 1.0) < 1e-11


def test_double_float_storage_conversion_exact():
    """The device's f64 <-> double-float conversion (bit operations) equals the IEEE conversions:
    hi = float(x), lo = float(x - hi), back = hi + lo, for ordinary values, ties, zeros, float
    subnormals and values beyond the float range."""
    rng = np.random.default_rng(12)
    n = 12
    x = rng.normal(size=2 << n) * np.exp(rng.uniform(-80, 80, size=2 << n))
    f = rng.normal(size=64).astype(np.float32).astype(np.float64)
    ulp = np.spacing(f.astype(np.float32)).astype(np.float64)
    special = np.concatenate([f + ulp / 2, f - ulp / 2, f + ulp * 1.5, [0.0, -0.0, 1e-40, -3e-39, 1e-320, 3.5e38,
                                                                      -1e39, 1.0, -1.0, 2.0 ** -126, 2.0 ** -149]])
    x[:special.size] = special
    q = QReg.new(n)
    q.set_engine(ENGINE_FUSED)
    q.set_amplitudes(x.view(np.complex128))
    got = q.amplitudes().view(np.float64)
    with np.errstate(over="ignore", invalid="ignore"):
        hi = x.astype(np.float32)
        lo = (x - hi.astype(np.float64)).astype(np.float32)
        want = hi.astype(np.float64) + lo.astype(np.float64)
    fin = np.isfinite(want)
    assert np.array_equal(got[fin], want[fin])
