"""Register-wide operations beside the gate path on the GPU, against the oracle: sample_all
(quant.rs:513-594, with injected normal draws), combine_with_unitary (quant.rs:273-308) and
linear_composition (quant.rs:311-328).  Plain engine bit-exact, fused engine within 1e-12."""
import numpy as np
import pytest

import oracle_ref as orc

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _state(n, seed, engine):
    from qvnt_gb300 import QReg
    from qvnt_gb300.circuits import random_circuit

    c = random_circuit(n, 3, seed=seed)
    q = QReg.with_state(n, seed % (1 << n))
    q.set_engine(engine)
    q.apply(c)
    psi = orc.new_state(n, seed % (1 << n))
    orc.apply(c.gates(), psi)
    return q, psi


@pytest.mark.parametrize("n", [3, 8, 12])
def test_sample_all_vs_oracle(n):
    from qvnt_gb300 import ENGINE_FUSED, ENGINE_PLAIN

    for engine in (ENGINE_PLAIN, ENGINE_FUSED):
        q, psi = _state(n, 20 + n, engine)
        for count, zs in ((1000, 0.5), (1_000_000, 1.0), (17, 30.0)):
            z = np.random.default_rng(count).normal(size=1 << n) * zs
            got = q.sample_all(count, normals=z)
            want = orc.sample_all(psi, n, count, z)
            assert int(got.sum()) == count
            if engine == ENGINE_PLAIN:
                assert np.array_equal(got, want)
            else:  # double-float probabilities: a count may differ at a rounding tie only
                assert np.sum(got != want) <= 1


def test_sample_all_device_draws():
    from qvnt_gb300 import ENGINE_FUSED

    q, psi = _state(10, 5, ENGINE_FUSED)
    p = orc.get_probabilities(psi, 10)
    count = 10_000_000
    h = q.sample_all(count, seed=1234)
    assert int(h.sum()) == count
    assert np.array_equal(h, q.sample_all(count, seed=1234))  # seeded draws repeat
    # counts follow count * p within a few standard deviations
    sd = np.sqrt(count * p * (1 - p)) + 1
    assert np.max(np.abs(h - count * p) / sd) < 8


def test_sample_all_rejects_padded_registers():
    from qvnt_gb300 import QReg
    from qvnt_gb300._abi import QvntError

    with pytest.raises(QvntError):
        QReg.new(2).sample_all(10, seed=1)


def test_combine_and_linear_composition_vs_oracle():
    from qvnt_gb300 import ENGINE_FUSED, ENGINE_PLAIN, QReg
    from qvnt_gb300._abi import QvntError

    h = 2 ** -0.5
    c = [h, 1j * h, 1j * h, h]
    for engine in (ENGINE_PLAIN, ENGINE_FUSED):
        for n in (3, 6, 11):
            qa, pa = _state(n, 31 + n, engine)
            qb, pb = _state(n, 47 + n, engine)
            out = QReg.combine_with_unitary(qa, qb, c)
            want = orc.combine_with_unitary(pa, pb, n, c)
            got = out.amplitudes()
            if engine == ENGINE_PLAIN:
                assert np.array_equal(got, want)
            else:
                assert np.max(np.abs(got - want)) <= TOL
            qa.linear_composition(qb, 0.6 + 0.2j, -0.3j)
            want_l = orc.linear_composition(pa.copy(), pb, 0.6 + 0.2j, -0.3j)
            if engine == ENGINE_PLAIN:
                assert np.array_equal(qa.amplitudes(), want_l)
            else:
                assert np.max(np.abs(qa.amplitudes() - want_l)) <= TOL
    qa, _ = _state(5, 1, ENGINE_PLAIN)
    qb, _ = _state(6, 2, ENGINE_PLAIN)
    with pytest.raises(QvntError):
        QReg.combine_with_unitary(qa, qb, c)  # different sizes: qvnt returns None
    with pytest.raises(QvntError):
        qa.linear_composition(qb, 1, 0)  # different lengths: qvnt's assert_eq panics
    with pytest.raises(QvntError):
        QReg.combine_with_unitary(qa, qa, [1, 1, 0, 1])  # not unitary
