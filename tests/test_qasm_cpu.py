"""CPU tests of the OpenQASM front end (`Ast`, `Int`; src/qasm/ast/mod.rs, src/qasm/int/).

Pinned on qvnt's own unit tests (restated as known answers): expression evaluation (parse.rs:44-62),
the AST of a small source and the parser's errors (ast/mod.rs:52-131), register masks and every
interpreter error case (int/mod.rs:414-640).  The lowering of qvnt's `operation_tree` source is
derived by hand from the interpreter's rules.  Programs then run through the runner loop over the
oracle (the harness of test_program_cpu.py); qvnt's 17 example programs are read from the qvnt
checkout directory that QVNT_QASM_EXAMPLES names (skipped when it is unset) and must all run, as qvnt's `run_qasm` test requires (qasm/mod.rs:15-39).
"""
import math
import os

import numpy as np
import pytest

import oracle_ref as orc
from qvnt_gb300.circuits import SplitMix64
from qvnt_gb300.qasm import NOP, Ast, Int, QasmError, eval_expr
from test_program_cpu import harness, run_harness, sym_finish_ref  # noqa: F401  (fixture)

EXAMPLES = ["adder", "bigadder", "Deutsch_Algorithm", "inverseqft1", "inverseqft2", "ipea_3_pi_8", "qe_qft_3",
            "qe_qft_4", "qe_qft_5", "qec", "qft", "qpt", "rb", "teleport", "teleportv2", "W-state", "W3test"]
# Directory of qvnt's example programs (src/qasm/examples/source in a qvnt checkout), from the
# environment only; the tests that read them are skipped when it is unset.
EXAMPLE_DIR = os.environ.get("QVNT_QASM_EXAMPLES", "")


def test_eval_expr():
    assert eval_expr("2 * pi / 16") == 2.0 * math.pi / 16.0
    assert eval_expr("2 * x / 16", [("x", math.pi)]) == 2.0 * math.pi / 16.0
    with pytest.raises(QasmError):
        eval_expr("2 * x / 16")
    assert eval_expr("-2^2") == -4.0 and eval_expr("2^3^2") == 512.0
    assert eval_expr("sqrt(2.0)") == math.sqrt(2.0) and eval_expr("atan2(1, 1)") == math.atan2(1, 1)
    assert eval_expr("max(1, 5, 2) - min(3, -1)") == 6.0 and eval_expr("1e-3 * 2") == 2e-3
    assert eval_expr("1/0") == math.inf and math.isnan(eval_expr("sqrt(-1)")) and eval_expr("ln(0)") == -math.inf
    with pytest.raises(QasmError):
        eval_expr("sin(1)")  # qvnt's context has no trigonometric functions (parse.rs:5-25)


def strip(nodes):
    out = []
    for n in nodes:
        if n[0] == "apply":
            out.append(("apply", n[1], n[2], [e.replace(" ", "") for e in n[3]]))
        else:
            out.append(n)
    return out


def test_ast_reference_cases():
    ast = Ast.from_source("OPENQASM 2.0; qreg a[3]; rx(pi, sqrt(2.0)) a[0], a[1];")
    assert strip(ast.nodes) == [("qreg", "a", 3), ("apply", "rx", [("a", 0), ("a", 1)], ["pi", "sqrt(2.0)"])]
    for bad in ("", "OPENQASM 0.0; qreg a[3]; CX a[0], a[1];", "OPENQASM 2.0 qreg a[3]; CX a[0], a[1];",
                "OPENQASM 2.0; qreg a[]; CX a[0], a[1];", "OPENQASM 2.0; qreg a[3]; a[0], a[1];"):
        with pytest.raises(QasmError):
            Ast.from_source(bad)


def test_ast_gate_definition():
    src = """OPENQASM 2.0;
    include "qelib1.inc";   // skipped
    qreg q[2]; creg c[2];
    gate foo(x, y) a, b { rx(x) a; }
    h q[0];
    cx q[0], q[1];
    foo(3.141592653589793, 0) q[0], q[1];
    """
    nodes = strip(Ast.from_source(src).nodes)
    assert nodes[:2] == [("qreg", "q", 2), ("creg", "c", 2)]
    assert nodes[2] == ("gate", "foo", ["a", "b"], ["x", "y"], [("apply", "rx", [("a", None)], ["x"])])
    assert nodes[3:] == [("apply", "h", [("q", 0)], []), ("apply", "cx", [("q", 0), ("q", 1)], []),
                         ("apply", "foo", [("q", 0), ("q", 1)], ["3.141592653589793", "0"])]


def test_int_registers():
    i = Int.from_source("OPENQASM 2.0; qreg a[1]; qreg b[2]; creg c[3]; creg e[4];")
    assert i.get_q_alias() == '["a", "b", "b"]' and i.get_c_alias() == '["c", "c", "c", "e", "e", "e", "e"]'
    assert Int.from_source("qreg a[1]; h a;").q_ops == Int.from_source("qreg b[1]; h b;").q_ops
    assert i.get_q_idx(("a", None)) == 1 and i.get_q_idx(("b", 1)) == 4
    assert i.get_c_idx(("c", None)) == 7 and i.get_c_idx(("e", None)) == 120
    for bad in (lambda: i.get_q_idx(("b", 2)), lambda: i.get_q_idx(("c", None)), lambda: i.get_c_idx(("d", None))):
        with pytest.raises(QasmError):
            bad()
    assert Int.from_source("qreg q[5]; h q[2];").q_reg == ["q"] * 5  # no header needed


REJECTED_SOURCES = [
    "h q[2];", "qreg q[2]; measure q -> c;", "qreg q[3]; qreg q[2];", "creg c[5]; creg c[1];",
    "qreg x[5]; creg x[1];", "creg x[1]; qreg x[5];", "qreg q[2]; h q[2];", "qreg q[2]; h q[3];",
    "qreg q[3]; g q[2];", "qreg q[4]; cx q[0], q;", "qreg q[4]; rx(2*a) q[0];", "qreg q[4]; rx(pi) q[0], q[2];",
    "qreg q[4]; rx(pi, 2*pi) q[0];", "qreg q[4]; creg c[3]; measure q -> c;", "gate m q { h q; }  gate m q { x q; }",
    "qreg q[1]; creg c[1]; if (c==1) measure q -> c;", "qreg " + "AAaaaaaaaaa" * 6 + "[1];", "qreg q[64];",
    "gate M q { h q[0]; }", "gate M(a, b, c) x, y { rx(a) x; ry(b) y; rz(c) z; }",
    "gate M(a, b) x, y, z { rx(a) x; ry(b) y; rz(c) z; }", "gate r q { r q; } qreg a[1]; r a;",
    "qreg q[2]; U(0, 0, 0) q[0];",
]


@pytest.mark.parametrize("src", REJECTED_SOURCES)
def test_int_rejects(src):
    with pytest.raises(QasmError):
        Int.from_source(src)


OPERATION_TREE_SRC = """OPENQASM 2.0; qreg q[2]; creg c[2];
    gate foo(x, y) a, b { rx(y*x) a; }
    h q[0]; cx q[0], q[1]; foo(pi, 1) q[0], q[1];
    measure q -> c;
    if (c==1) h q[0]; if (c==2) h q[1]; if (c==3) h q[0], q[1];
    measure q -> c;"""


def test_int_operation_tree():
    """qvnt's `operation_tree` source (int/mod.rs:444-476), lowered by the interpreter's rules: the
    gates before the first measure ride in its block; each `if` after a separator is its own block;
    the last measure has an empty block."""
    i = Int.from_source(OPERATION_TREE_SRC)
    assert [sep for _, sep in i.q_ops.blocks] == [("measure", 3, 3), ("if", 3, 1), ("if", 3, 2), ("if", 3, 3),
                                                  ("measure", 3, 3)]
    assert i.get_ops_tree() == ("[H1, C1_X2, RX1(3.141592653589793)] -> Measure(11 => 11) -> if c[11] == 1 { [H1] }"
                                " -> if c[11] == 10 { [H2] } -> if c[11] == 11 { [H3] } -> Measure(11 => 11)")


def test_if_after_gates_is_unconditional_as_in_qvnt():
    i = Int.from_source("qreg q[2]; creg c[1]; h q[0]; if (c==1) x q[1];")
    assert i.q_ops.blocks == [(i.q_ops.blocks[0][0], NOP)] and len(i.q_ops.blocks[0][0]) == 2
    assert i.get_ops_tree() == "[H1, X2]"


def test_builtin_gate_table():
    i = Int.from_source("""qreg q[3]; ccx q[0], q[1], q[2]; sdg q[0]; tdg q[1]; CX q[0], q[1];
        u3(0.1, 0.2, 0.3) q[2]; u2(0.1, 0.2) q[2]; u1(0.5) q[0]; cu1(pi/4) q[0], q[1]; rzz(0.3) q[0], q[2];
        i_swap q[0], q[1]; sqrt_swap q[1], q[2]; qft q; x q[0], q[2];""")
    names = i.get_ops_tree()
    # c-prefix controls by the first register; sdg/tdg build S/T (gates.rs:92-95); a register list ORs
    assert names.startswith("[C3_X4, S1, T2, C1_X2, ")
    # u3 = rz(lam) ry(the) rz(phi), u2 = rz(lam) ry(pi/2) rz(phi), u1 = rz (operator/mod.rs:472-501)
    assert "RZ4(0.3), RY4(0.1), RZ4(0.19999999999999998), RZ4(0.19999999999999998), RY4(1.5707963267948966), " \
           "RZ4(0.1), RZ1(0.5), C1_RZ2(0.7853981633974484), RZZ5(0.3), iSWAP3, sqrt(SWAP6), H1, " in names
    assert names.endswith("H4, X5]")  # qft q (no swaps), then x over both listed qubits


def run_int(exe, i, seed):
    n, c_num = len(i.q_reg), len(i.c_reg)
    p = i.q_ops
    rng = SplitMix64(seed)
    draws = [rng.uniform() for _ in range(p.measure_count())]
    st, used, c, psi = run_harness(exe, n, c_num, p, 0, 0, draws, i.m_op)
    want, wc, wd = sym_finish_ref(n, c_num, p, 0, 0, draws, i.m_op)
    assert st == 0 and used == wd and c == wc
    assert np.array_equal(psi, want)
    return c, psi


def test_teleport_qasm(harness):  # noqa: F811
    src = """OPENQASM 2.0;
    qreg q[3]; creg m0[1]; creg m1[1];
    ry(1.1) q[0]; rz(0.7) q[0];
    h q[1]; cx q[1], q[2];
    cx q[0], q[1]; h q[0];
    measure q[0] -> m0[0]; measure q[1] -> m1[0];
    if (m1==1) x q[2];
    if (m0==1) z q[2];"""
    i = Int.from_source(src)
    ref = orc.new_state(1, 0)
    orc.apply((Int.from_source("qreg q[1]; ry(1.1) q[0]; rz(0.7) q[0];").q_ops.last).gates(), ref)
    want = ref[:2] / np.linalg.norm(ref[:2])
    seen = set()
    for seed in range(40):
        c, psi = run_int(harness, i, seed)
        seen.add(c)
        amps = psi[[c, c | 0b100]]
        amps = amps / np.linalg.norm(amps)
        assert abs(abs(np.vdot(want, amps)) - 1.0) <= 1e-12
    assert seen == {0, 1, 2, 3}


def test_ghz_measurement_agrees(harness):  # noqa: F811
    i = Int.from_source("qreg q[4]; creg c[4]; h q[0]; cx q[0], q[1]; cx q[1], q[2]; cx q[2], q[3]; measure q -> c;")
    outcomes = {run_int(harness, i, seed)[0] for seed in range(30)}
    assert outcomes == {0, 0b1111}


@pytest.mark.skipif(not (EXAMPLE_DIR and os.path.isdir(EXAMPLE_DIR)),
                    reason="QVNT_QASM_EXAMPLES does not name a directory of qvnt's example programs")
@pytest.mark.parametrize("name", EXAMPLES)
def test_reference_examples_run(name, harness):  # noqa: F811
    with open(os.path.join(EXAMPLE_DIR, name + ".qasm")) as f:
        i = Int.from_source(f.read())
    for seed in (1, 2):
        run_int(harness, i, seed)


# ------------------------------------------------------------------------------ the C++ front end

OWN_SOURCES = [
    """OPENQASM 2.0; include "qelib1.inc"; qreg q[3]; creg c[2];
    gate foo(a, b) x, y { rx(a) x; cx x, y; u1(b/2) y; }
    h q[0]; cx q[0], q[1]; foo(pi/2, 0.5) q[1], q[2];
    measure q[0] -> c[0]; measure q[1] -> c[1]; if (c == 1) x q[2]; reset q[0]; barrier q;""",
    """qreg a[2]; qreg b[3]; creg m[2]; gate maj a, b, c { cx c, b; cx c, a; ccx a, b, c; }
    maj a[0], b[0], b[1]; u3(0.1, -0.2e1, 3/4) b[2]; sdg a[1]; tdg b; cu1(pi^2 % 1) a[0], a[1];
    rzz(max(0.1, 0.2)) a[0], b[2]; h a; if (m==3) sqrt_swap b[0], b[2]; measure a -> m; qft b;""",
    "qreg q[1]; U(0, 0, 0) q[0];",
    "qreg q[2]; creg c[2]; h q[0]; if (c==1) x q[1]; measure q -> c;",
]


def native_view(src):
    from qvnt_gb300.qasm import compile_native
    p, q, c = compile_native(src)
    return q, c, [(sep, [bytes(g) for g in ops.gates()]) for ops, sep in p.blocks], [bytes(g) for g in p.last.gates()]


def python_view(src):
    i = Int.from_source(src)
    return (len(i.q_reg), len(i.c_reg), [(sep, [bytes(g) for g in ops.gates()]) for ops, sep in i.q_ops.blocks],
            [bytes(g) for g in i.q_ops.last.gates()])


def same_outcome(src):
    from qvnt_gb300._abi import QvntError
    try:
        want = python_view(src)
    except QasmError:
        want = "rejected"
    try:
        got = native_view(src)
    except QvntError:
        got = "rejected"
    assert got == want, src[:200]
    return want != "rejected"


def test_native_front_end_matches(lib_built):
    """qvnt_qasm_compile (C++) lowers every program exactly as the Python front end does, and rejects
    the same ones, on this file's programs and the reference error cases."""
    srcs = OWN_SOURCES + [OPERATION_TREE_SRC]
    accepted = sum(same_outcome(s) for s in srcs)
    assert accepted == len(srcs) - 1  # the U(...) program is rejected by both
    for bad in REJECTED_SOURCES:
        assert not same_outcome(bad)
    if EXAMPLE_DIR and os.path.isdir(EXAMPLE_DIR):
        for name in EXAMPLES:
            with open(os.path.join(EXAMPLE_DIR, name + ".qasm")) as f:
                assert same_outcome(f.read()), name


def test_native_front_end_matches_on_mutations(lib_built):
    rng = SplitMix64(77)
    alpha = "qcrgx[](){};,->=0123456789.+-*/^pi hmeasurtif\n\""
    accepted = 0
    for k in range(2000):
        s = list(OWN_SOURCES[k % 2])
        for _ in range(1 + rng.below(4)):
            i = rng.below(len(s))
            r = rng.below(10)
            if r < 4:
                s[i] = alpha[rng.below(len(alpha))]
            elif r < 7:
                del s[i]
            else:
                s.insert(i, alpha[rng.below(len(alpha))])
        accepted += same_outcome("".join(s))
    assert accepted > 30
