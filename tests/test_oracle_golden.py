"""Pins the CPU oracle to the known answers of qvnt's own unit tests (tests/golden/)."""
import numpy as np
import pytest

import oracle_ref as orc


def build_gate(spec):
    g = orc.make(spec["kind"], spec["a"], spec["b"], spec["angle"], spec["matrix"])
    assert g is not None, spec
    if spec["dgr"]:
        g = orc.dgr(g)
    if spec["ctrl"]:
        g = orc.c(g, spec["ctrl"])
    return g


def cplx(m):
    return np.array([[complex(z[0], z[1]) for z in row] for row in m])


def test_matrix_repr_exact(golden):
    # every atomic `matrix_repr` test: qvnt compares with assert_eq! (exact f64 equality)
    for case in golden["matrix_cases"]:
        gates = [build_gate(s) for s in case["gates"]]
        got = orc.matrix(gates, case["size"])
        want = cplx(case["matrix"])
        assert np.array_equal(got, want), case["cite"]


def test_invalid_masks_rejected(golden):
    for case in golden["invalid_cases"]:
        s = case["gate"]
        assert orc.make(s["kind"], s["a"], s["b"], s["angle"], s["matrix"]) is None, case["cite"]
    for case in golden["non_unitary_cases"]:
        s = case["gate"]
        assert orc.make(s["kind"], s["a"], s["b"], s["angle"], s["matrix"]) is None, case["cite"]


def program_gates(program):
    gates = []
    for name, mask, ctrl in program:
        if name == "h":
            gs = orc.op_h(mask)
        elif name == "swap":
            gs = [orc.make("SWAP", mask)]
        else:
            raise KeyError(name)
        if ctrl:
            gs = [orc.c(g, ctrl) for g in gs]
        gates += gs
    return gates


def test_quantum_reg_vector(golden):
    # quant.rs:642-677: exact 16-amplitude vector after h * C8_h * C2_swap
    for case in golden["register_cases"]:
        psi = orc.new_state(case["q_num"], case["state"])
        gates = program_gates(case["program"])
        assert len(gates) == 4
        orc.apply(gates, psi, nthreads=1)
        want = np.array([complex(a, b) for a, b in case["psi"]])
        assert np.array_equal(psi[: len(want)], want), case["cite"]
        for u in np.linspace(0.0, 0.999, 17):
            p = psi.copy()
            v, _ = orc.measure_mask(p, case["q_num"], case["measure_mask"], u)
            assert v & ~case["measure_mask"] == 0


def test_tensor_probabilities(golden):
    for case in golden["tensor_cases"]:
        a, b = case["a"], case["b"]
        pa = orc.new_state(a["q_num"], a["state"])
        orc.apply(orc.op_h(a["h"]), pa, 1)
        pb = orc.new_state(b["q_num"], b["state"])
        orc.apply(orc.op_h(b["h"]), pb, 1)
        t = orc.tensor(pa, a["q_num"], pb, b["q_num"])
        prob = orc.get_probabilities(t, a["q_num"] + b["q_num"])
        assert np.all(np.abs(prob - np.array(case["prob"])) < case["eps"]), case["cite"]
    for case in golden["prob_cases"]:
        p = orc.new_state(case["q_num"], case["state"])
        orc.apply(orc.op_h(case["h"]), p, 1)
        prob = orc.get_probabilities(p, case["q_num"])
        assert np.all(np.abs(prob - np.array(case["prob"])) < case["eps"]), case["cite"]


def test_ctrl_overlap(golden):
    for case in golden["ctrl_cases"]:
        s = case["gate"]
        g = orc.make(s["kind"], s["a"], s["b"], s["angle"])
        assert orc.c(g, case["reject"]) is None
        assert orc.c(g, case["accept"]) is not None


def test_weighted_index_rule():
    # rand 0.8.5 WeightedIndex: first index whose inclusive cumulative weight exceeds u * total
    w = np.array([0.0, 0.25, 0.0, 0.5, 0.25])
    assert orc.weighted_index(w, 0.0) == 1
    assert orc.weighted_index(w, 0.2499) == 1
    assert orc.weighted_index(w, 0.25) == 3
    assert orc.weighted_index(w, 0.7499) == 3
    assert orc.weighted_index(w, 0.75) == 4
    assert orc.weighted_index(w, 0.9999) == 4


def test_rotation_dgr_quirk():
    # qvnt's rotation .dgr() negates the stored phase: R(theta).dgr() == -R(theta) (rx.rs:42-47)
    for kind, size, mask in (("RX", 1, 1), ("RY", 1, 1), ("RZ", 1, 1), ("RXX", 2, 3), ("RYY", 2, 3), ("RZZ", 2, 3)):
        g = orc.make(kind, mask, angle=0.7)
        m = orc.matrix([g], size)
        md = orc.matrix([orc.dgr(g)], size)
        assert np.array_equal(md, -m), kind


def test_h_and_qft_structure():
    # h.rs: pairs of set bits become H2 (higher bit first), an odd bit H1
    hs = orc.op_h(0b1111)
    assert [(g.kind, g.a_mask, g.b_mask) for g in hs] == [(15, 0b10, 0b01), (15, 0b1000, 0b100)]
    hs = orc.op_h(0b10101)
    assert [(g.kind, g.a_mask, g.b_mask) for g in hs] == [(15, 0b100, 0b1), (14, 0b10000, 0)]
    q = orc.op_qft(0xFFFFF)
    assert len(q) == 20 + 190
    q30 = orc.op_qft((1 << 30) - 1)
    assert len(q30) == 30 + 435
    assert len(orc.op_qft_swapped(0xFF)) == 8 + 28 + 4


def test_oracle_threads_agree():
    # for_each (serial) and for_each_par (OpenMP) give identical amplitudes
    from qvnt_gb300.circuits import SplitMix64
    rng = SplitMix64(7)
    n = 10
    gates = []
    for _ in range(60):
        q = rng.below(n)
        gates.append(orc.make("RX", 1 << q, angle=rng.uniform() * 6.28))
        gates += orc.op_h(1 << rng.below(n))
        a, b = rng.below(n), rng.below(n)
        if a != b:
            gates.append(orc.make("RZZ", (1 << a) | (1 << b), angle=1.0))
    p1 = orc.apply(gates, orc.new_state(n, 5), nthreads=1)
    p8 = orc.apply(gates, orc.new_state(n, 5), nthreads=4)
    assert np.array_equal(p1, p8)


def test_normalize_thresholds():
    psi = orc.new_state(3, 0)
    psi[:] = 0.0
    orc.normalize(psi, 3)
    assert psi[0] == 1.0 and np.count_nonzero(psi) == 1  # norm <= 1e-15 resets to |0>
    # `1. - norm <= 1e-9` (quant.rs:402) is one-sided: a norm above 1 is left as it is
    psi = np.full(8, 0.5 + 0j)
    orc.normalize(psi, 3)
    assert np.sum(np.abs(psi) ** 2) == 2.0
    psi = np.full(8, 0.25 + 0j)
    orc.normalize(psi, 3)
    assert np.isclose(np.sum(np.abs(psi) ** 2), 1.0)


def test_oracle_sample_all_invariants():
    """sample_all keeps the total at `count` for deficits and excesses, and panics (None) below 3
    qubits as qvnt does."""
    import numpy as np

    import oracle_ref as orc

    n = 5
    rng = np.random.default_rng(1)
    psi = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    psi /= np.linalg.norm(psi)
    for count in (1, 7, 1000, 123457):
        for seed in range(4):
            z = np.random.default_rng(seed).normal(size=1 << n) * (10.0 if seed == 3 else 1.0)
            out = orc.sample_all(psi.astype(np.complex128), n, count, z)
            assert int(out.sum()) == count
    assert orc.sample_all(orc.new_state(2, 0), 2, 10, np.zeros(4)) is None


def test_oracle_linear_and_combine():
    import numpy as np

    import oracle_ref as orc

    rng = np.random.default_rng(3)
    a = rng.normal(size=16) + 1j * rng.normal(size=16)
    b = rng.normal(size=16) + 1j * rng.normal(size=16)
    lin = orc.linear_composition(a.copy(), b, 0.3 - 0.1j, 1.2j)
    assert np.allclose(lin, a * (0.3 - 0.1j) + b * 1.2j, atol=1e-15)
    h = 2 ** -0.5
    c = [h, h, h, -h]
    out = orc.combine_with_unitary(a, b, 4, c)
    assert np.allclose(out[:16], h * a + h * b) and np.allclose(out[16:], h * a - h * b)
