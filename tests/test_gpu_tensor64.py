"""The TENSOR64 engine (dense 5-qubit blocks on the tensor cores, 53-bit operands split into exact
fp16 digit products, IEEE f64 storage) against the CPU oracle (qvnt's MultiOp::apply,
src/operator/multi/mod.rs:97-114, and AtomicOp::for_each, src/operator/atomic/dispatch.rs:32-67).

Bar: within 1e-12 max-abs and within REL of the largest amplitude (a bound set from the measured
error of the engine: one rounding of each block's inputs to 53 bits and one rounding to f64 per
block).  Registers below 12 qubits run on the plain kernels and stay bit-identical.
"""
import math

import numpy as np
import pytest

import oracle_ref as orc
from qvnt_gb300 import ENGINE_PLAIN, ENGINE_TENSOR64, KINDS, QReg, op
from qvnt_gb300.circuits import plain_circuit, random_circuit
from test_gpu_parity import all_kinds_circuit

pytestmark = pytest.mark.gpu

TOL = 1e-12
REL = 2e-13
REL_HP = 1e-15  # against the high-precision reference


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


# ---- a high-precision reference: the circuit's own gate records (the coefficient doubles the engine and
# qvnt use) applied with 320-bit fixed-point arithmetic, so that its own rounding (2^-320) is nil
_HP = 320


def _hp(v):
    """A double as an integer at scale 2^-320 (exact for |v| >= 2^-267)."""
    m, e = math.frexp(v)
    mi = int(m * (1 << 53))
    sh = e - 53 + _HP
    return mi << sh if sh >= 0 else mi >> -sh


def _hp_state(psi):
    return [_hp(float(z.real)) for z in psi], [_hp(float(z.imag)) for z in psi]


def _hp_apply(gates, re, im, n):
    """qvnt's atomic formulas (src/operator/atomic/{x,z,s,t,rx,ry,rz,h1}.rs, controls as in
    dispatch.rs:32-67) for the kinds the precision circuit uses, without rounding."""
    frac = _hp(0.70710678118654752440084436210484903)  # the double qvnt's h1.rs and t.rs use
    mul = lambda a, c: (a * c) >> _HP  # noqa: E731
    for g in gates:
        kind, a, ctrl = KINDS[g.kind], int(g.a_mask), int(g.ctrl)
        cr, ci = _hp(g.phase[0]), _hp(g.phase[1])
        nr, ni = list(re), list(im)
        for idx in range(1 << n):
            if idx & ctrl != ctrl:
                continue
            p0r, p0i = re[idx], im[idx]
            p1r, p1i = re[idx ^ a], im[idx ^ a]
            if kind == "X":
                r, i = p1r, p1i
            elif kind == "Z":
                r, i = (-p0r, -p0i) if bin(idx & a).count("1") & 1 else (p0r, p0i)
            elif kind in ("S", "T"):
                count = bin(idx & a).count("1")
                q = count if kind == "S" else count >> 1
                r, i = p0r, p0i
                if q & 2:
                    r, i = -r, -i
                if q & 1:
                    r, i = -i, r
                if kind == "T" and count & 1:
                    r, i = mul(r, frac) - mul(i, frac), mul(r, frac) + mul(i, frac)
            elif kind == "RX":
                r, i = mul(p0r, cr) + mul(p1i, ci), mul(p0i, cr) - mul(p1r, ci)
            elif kind == "RY":
                pi = ci if idx & a else -ci
                r, i = mul(p0r, cr) + mul(p1r, pi), mul(p0i, cr) + mul(p1i, pi)
            elif kind == "RZ":
                pi = ci if idx & a else -ci
                r, i = mul(cr, p0r) - mul(pi, p0i), mul(cr, p0i) + mul(pi, p0r)
            elif kind == "H1":
                if idx & a:
                    p0r, p0i = -p0r, -p0i
                r, i = mul(p0r + p1r, frac), mul(p0i + p1i, frac)
            else:
                raise AssertionError(kind)
            nr[idx], ni[idx] = r, i
        re, im = nr, ni
    return re, im


def _hp_error(got, ref):
    """max |got - ref| / max |ref|, the differences taken exactly."""
    re, im = ref
    d = max(math.hypot(_hp(float(z.real)) - x, _hp(float(z.imag)) - y) for z, x, y in zip(got, re, im))
    m = max(math.hypot(x, y) for x, y in zip(re, im))
    return d / m


def _precision_circuit(n, count, seed):
    rng = np.random.default_rng(seed)
    circ = op.id()
    for _ in range(count):
        q = int(rng.integers(n))
        kind = rng.choice(["rx", "ry", "rz", "h", "t", "s", "cx", "cz", "ccx"])
        if kind in ("rx", "ry", "rz"):
            g = getattr(op, kind)(float(rng.uniform(-np.pi, np.pi)), 1 << q)
        elif kind in ("h", "t", "s"):
            g = getattr(op, kind)(1 << q)
        else:
            others = [int(v) for v in rng.choice([v for v in range(n) if v != q], 2, replace=False)]
            ctrl = (1 << others[0]) | ((1 << others[1]) if kind == "ccx" else 0)
            g = (op.z if kind == "cz" else op.x)(1 << q).c(ctrl)
        circ = circ * g
    return circ


@pytest.mark.parametrize("n", [12, 13])
def test_precision_against_high_precision_reference(n):
    """The engine against the same gate records applied without rounding (320-bit fixed point), beside
    qvnt's own f64 loop (the oracle: one rounding per product and sum, gate by gate): the engine's
    error, relative to the largest amplitude, stays within REL_HP and within twice the f64 loop's."""
    rng = np.random.default_rng(n)
    psi = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    psi /= np.linalg.norm(psi)
    circ = _precision_circuit(n, 40, seed=n)
    ref = _hp_apply(circ.gates(), *_hp_state(psi), n)
    want = psi.copy()
    orc.apply(circ.gates(), want)
    q = QReg.new(n)
    q.set_engine(ENGINE_TENSOR64)
    q.set_amplitudes(psi)
    q.apply(circ)
    got = q.amplitudes()
    e_t64, e_f64 = _hp_error(got, ref), _hp_error(want, ref)
    print("n=%d: tensor64 %.3e, f64 gate by gate %.3e (relative to max |psi|)" % (n, e_t64, e_f64))
    assert e_t64 <= REL_HP and e_t64 <= 2.0 * e_f64


def test_nonfinite_block_runs_on_plain_kernels():
    """A block whose matrix is not finite (a rotation by NaN) is not split into digits: the run of gates
    it belongs to goes to the plain kernels, so the result equals the PLAIN engine's bit for bit (NaNs
    in the same places)."""
    n = 13
    circ = random_circuit(n, 2, seed=31) * op.rx(float("nan"), 1 << 4) * op.h(0b101)
    a = run(n, 3, circ).amplitudes()
    b = run(n, 3, circ, ENGINE_PLAIN).amplitudes()
    assert np.array_equal(np.isnan(a), np.isnan(b))
    ok = ~np.isnan(a)
    assert np.array_equal(a[ok], b[ok])
