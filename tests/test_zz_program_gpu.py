"""The QASM runner on the GPU: qvnt_program_run (`Sym::finish`, src/qasm/sym.rs:40-74) on a device
register against the restatement over the oracle, on the seeded random programs of the CPU tests.
Plain engine: measured values and classical bits identical; amplitudes within 1e-12 (reset_by_mask
renormalises with a device sum, within 1e-15 of the oracle's per call).  Collected after the other
GPU tests."""
import numpy as np
import pytest

from test_program_cpu import random_program, sym_finish_ref

pytestmark = pytest.mark.gpu

TOL = 1e-12


@pytest.mark.parametrize("measure_op", ["set", "xor"])
def test_program_run_vs_oracle(measure_op):
    from qvnt_gb300 import ENGINE_PLAIN, QReg
    from qvnt_gb300.circuits import SplitMix64
    from qvnt_gb300.qasm import run_program

    for seed in range(1, 25):
        n = 3 + seed % 6
        c_num = 1 + seed % 5
        p, nmeas = random_program(n, c_num, 12 + seed % 9, seed)
        rng = SplitMix64(seed + 99)
        draws = [rng.uniform() for _ in range(nmeas)]
        state = rng.next_u64() & ((1 << n) - 1)
        creg = rng.next_u64() & ((1 << c_num) - 1)
        q = QReg.with_state(n, state)
        q.set_engine(ENGINE_PLAIN)
        c, used = run_program(q, p, c_num, creg, draws, measure_op)
        want, wc, wd = sym_finish_ref(n, c_num, p, state, creg, draws, measure_op)
        assert used == wd == nmeas
        assert c == wc, seed
        assert np.max(np.abs(q.amplitudes() - want)) <= TOL, seed


def test_sym_teleport_on_gpu():
    from qvnt_gb300 import ENGINE_PLAIN, op
    from qvnt_gb300.qasm import Program, Sym

    import oracle_ref as orc

    prep = op.ry(1.1, 0b001) * op.rz(0.7, 0b001)
    p = (Program().apply(prep).apply(op.h(0b010)).apply(op.x(0b100).c(0b010))
         .apply(op.x(0b010).c(0b001)).apply(op.h(0b001)).measure(0b011, 0b011)
         .if_branch(0b10, 1, op.x(0b100)).if_branch(0b01, 1, op.z(0b100)))
    ref = orc.new_state(1, 0)
    orc.apply(prep.gates(), ref)
    want = ref[:2] / np.linalg.norm(ref[:2])
    sym = Sym(p, 3, 2, engine=ENGINE_PLAIN)
    outcomes = set()
    for u in np.linspace(0.01, 0.99, 25):
        sym.reset()
        sym.finish([u])
        c = sym.get_class().get()
        outcomes.add(c)
        amps = sym.amplitudes()[[c, c | 0b100]]
        amps = amps / np.linalg.norm(amps)
        assert abs(abs(np.vdot(want, amps)) - 1.0) <= 1e-12
    assert outcomes == {0, 1, 2, 3}
    # Sym::measure outside the program (sym.rs:76-87): qubit 2 into classical bit 1
    sym.reset()
    sym.measure(0b100, 0b10, 0.5)
    assert sym.get_class().get() == 0


def test_qasm_program_on_gpu():
    """An OpenQASM program through the front end (`Int`) and `Sym::new(int)` on the device."""
    from qvnt_gb300 import ENGINE_PLAIN
    from qvnt_gb300.circuits import SplitMix64
    from qvnt_gb300.qasm import Int, sym_from_int

    src = """OPENQASM 2.0;
    qreg q[4]; creg c[2]; creg d[2];
    gate prep(a, b) x { ry(a) x; rz(b/2) x; }
    prep(1.1, 0.7) q[0]; h q[1]; cx q[1], q[2]; cx q[0], q[1]; h q[0];
    measure q[0] -> c[0]; measure q[1] -> c[1];
    if (c==2) x q[2]; if (c==1) z q[2]; if (c==3) y q[2];
    h q[3]; measure q[2] -> d[0];
    reset q[3];"""
    i = Int.from_source(src)
    sym = sym_from_int(i, engine=ENGINE_PLAIN)
    for seed in range(8):
        rng = SplitMix64(seed)
        draws = [rng.uniform() for _ in range(i.q_ops.measure_count())]
        sym.reset()
        sym.finish(draws)
        want, wc, _ = sym_finish_ref(4, 4, i.q_ops, 0, 0, draws, "set")
        assert sym.get_class().get() == wc
        assert np.max(np.abs(sym.amplitudes() - want)) <= TOL
