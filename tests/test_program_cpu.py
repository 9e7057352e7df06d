"""CPU tests of the QASM runner (`Sym::finish`, src/qasm/sym.rs:40-74).

The runner loop that qvnt_program_run executes (qvnt_gb300/csrc/program.h) is compiled here into a
small program over the CPU oracle's register (tests/program_oracle.cpp) and compared, on seeded
random programs, with a direct restatement of `Sym::finish` over the oracle.  The program builder
(`int::Op` push/append, src/qasm/int/ext_op.rs:22-50) is pinned on qvnt's own `append_left` /
`append_right` tests (ext_op.rs:131-175).  No kernel runs here.
"""
import ctypes
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

import oracle_ref as orc
from qvnt_gb300 import _abi, op
from qvnt_gb300._abi import KIND, QvntError
from qvnt_gb300.circuits import SplitMix64
from qvnt_gb300.operator import MultiOp
from qvnt_gb300.qasm import NOP, Program, run_program
from qvnt_gb300.register import CReg, bits_iter
from test_gpu_parity import all_kinds_circuit

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no C++ compiler")
    orc.lib()  # builds the oracle library when missing
    exe = tmp_path_factory.mktemp("program") / "program_oracle"
    libdir = os.path.dirname(orc.LIB)
    r = subprocess.run([cxx, "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-ffp-contract=off",
                        os.path.join(ROOT, "tests", "program_oracle.cpp"), "-o", str(exe), "-L", libdir,
                        "-lqvnt_oracle", "-Wl,-rpath," + libdir], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def run_harness(exe, n, c_num, program, state=0, creg=0, draws=(), measure_op="set", blocks_override=None):
    garr, ng, barr, nb, tail = program.lower()
    if blocks_override is not None:
        barr, nb = blocks_override, len(blocks_override)
    m = {"set": _abi.MEASURE_SET, "xor": _abi.MEASURE_XOR}.get(measure_op, measure_op)
    data = struct.pack("=IIiIQQQQII", n, c_num, m, nb, state, creg, ng, tail, len(draws), 0)
    data += bytes(garr)[:ng * 304] + bytes(barr)[:nb * ctypes.sizeof(_abi.QvntBlock)]
    data += struct.pack("=%dd" % len(draws), *draws)
    d = os.path.dirname(exe)
    inp, out = os.path.join(d, "in.bin"), os.path.join(d, "out.bin")
    with open(inp, "wb") as f:
        f.write(data)
    r = subprocess.run([str(exe), inp, out], capture_output=True, text=True)
    assert r.returncode == 0, (r.returncode, r.stderr)
    raw = open(out, "rb").read()
    st, used, c, length = struct.unpack_from("=iIQQ", raw)
    psi = np.frombuffer(raw[24:], dtype=np.complex128)
    assert psi.size == length
    return st, used, c, psi


def sym_finish_ref(n, c_num, program, state, creg, draws, measure_op):
    """`Sym::finish` (sym.rs:40-74), statement by statement over the oracle."""
    psi = orc.new_state(n, state)
    c = CReg(c_num, creg)
    d = 0

    def apply(ops):
        if len(ops):
            orc.apply(ops.gates(), psi)

    for ops, sep in program.blocks:
        if sep[0] == "nop":
            apply(ops)
        elif sep[0] == "measure":
            apply(ops)
            v, _ = orc.measure_mask(psi, n, sep[1], draws[d])
            d += 1
            for q, cb in zip(bits_iter(sep[1]), bits_iter(sep[2])):
                (c.set if measure_op == "set" else c.xor)(v & q != 0, cb)
        elif sep[0] == "if":
            if c.get_by_mask(sep[1]) == sep[2]:
                apply(ops)
        else:
            apply(ops)
            orc.reset_by_mask(psi, n, sep[1])
    apply(program.last)
    return psi, c.get(), d


def random_program(n, c_num, statements, seed, circuit=all_kinds_circuit):
    """Seeded programs built statement by statement, as qvnt's interpreter builds them."""
    rng = SplitMix64(seed)
    p = Program()
    nmeas = 0
    for s in range(statements):
        k = rng.below(10)
        if k < 4:
            p.apply(circuit(max(n, 3), 1 + rng.below(5), seed * 1000 + s))
        elif k < 6:
            w = 1 + rng.below(min(n, c_num))
            qs = sorted(rng.below(n) for _ in range(w))
            cs = sorted(rng.below(c_num) for _ in range(w))
            qm = sum(1 << q for q in set(qs))
            cm = sum(1 << x for x in set(cs))
            if bin(qm).count("1") != bin(cm).count("1"):
                # direct block with unequal counts: the zip stops at the shorter list (sym.rs:52-54)
                p.append(Program([(MultiOp(), ("measure", qm, cm))]))
            else:
                p.measure(qm, cm)
            nmeas += 1
        elif k < 7:
            p.reset((rng.next_u64() & ((1 << n) - 1)) or 1)
        else:
            cm = (rng.next_u64() & ((1 << (c_num + 1)) - 1)) or 1  # may name a bit beyond c_num
            width = bin(cm & ((1 << c_num) - 1)).count("1")
            v = rng.below(1 << width) if rng.below(5) else (1 << width)  # sometimes never equal
            p.if_branch(cm, v, circuit(max(n, 3), 1 + rng.below(2), seed * 1000 + s + 500))
    if rng.below(2):
        p.apply(circuit(max(n, 3), 3, seed * 7 + 1))
    return p, nmeas


def test_builder_matches_reference_append():
    """ext_op.rs:131-175: `append_left` and `append_right`."""
    x6, h7, z2, y3 = op.x(0b110), op.h(0b111), op.z(0b010), op.y(0b011)
    left = Program([(x6, NOP)], h7)
    right = Program([(z2, ("measure", 0, 0))], y3)
    got = left * right
    assert got.blocks == [(x6 * h7, NOP), (z2, ("measure", 0, 0))] and got.last == y3
    got = right * left
    assert got.blocks == [(z2, ("measure", 0, 0)), (y3, NOP), (x6, NOP)] and got.last == h7


def test_builder_statements():
    """The interpreter's lowering on one program (int/mod.rs:207-305, 374-384): measure and reset
    close the pending gates, even none, into their block; an if after a separator is its own block."""
    p = Program().apply(op.h(0b11)).apply(op.x(1)).measure(0b11, 0b11)
    assert p.blocks == [(op.h(0b11) * op.x(1), ("measure", 3, 3))] and len(p.last) == 0
    p.if_branch(0b1, 1, op.z(2)).reset(0b10).apply(op.y(1))
    assert p.blocks[1:] == [(op.z(2), ("if", 1, 1)), (MultiOp(), ("reset", 2))] and p.last == op.y(1)
    with pytest.raises(ValueError):
        Program().measure(0b11, 0b1)


def test_builder_if_after_gates_quirk(harness):
    """qvnt's interpreter: branch(Nop) turns the pending gates into a NOP block, `push` then joins the
    if-gate to that block (ext_op.rs:40-50) and branch(If) finds nothing pending -- the gate runs
    unconditionally.  After a separator the if keeps its condition."""
    p = Program().apply(op.h(0b1)).if_branch(0b1, 1, op.x(0b10))
    assert p.blocks == [(op.h(0b1) * op.x(0b10), NOP)] and len(p.last) == 0
    st, _, _, psi = run_harness(harness, 3, 1, p, creg=0)
    want = orc.new_state(3, 0)
    orc.apply((op.h(0b1) * op.x(0b10)).gates(), want)
    assert st == 0 and np.array_equal(psi, want)
    p = Program().apply(op.h(0b1)).measure(0b1, 0b1).if_branch(0b1, 1, op.x(0b10))
    assert p.blocks[-1] == (op.x(0b10), ("if", 1, 1))


def test_get_by_mask_and_zip_rules(harness):
    # c_num 3, c = 0b101: get_by_mask(0b101) packs bits 0 and 2 -> 0b11; bit 3 is outside the register
    n = 3
    for cm, v, taken in ((0b101, 0b11, True), (0b101, 0b01, False), (0b1101, 0b11, True), (0b1000, 0, True),
                         (0b010, 0, True), (0b010, 1, False)):
        p = Program().if_branch(cm, v, op.x(0b100))
        st, used, c, psi = run_harness(harness, n, 3, p, creg=0b101)
        assert (st, used, c) == (0, 0, 0b101)
        assert np.array_equal(psi, orc.new_state(n, 0b100 if taken else 0))
    # measured bits feed classical bits in increasing order, the shorter mask ends the zip
    p = Program([(MultiOp(), ("measure", 0b110, 0b1001))])
    for m_op, c0, want in (("set", 0b0110, 0b1111), ("xor", 0b1001, 0), ("set", 0b1111, 0b1111)):
        st, used, c, _ = run_harness(harness, 3, 4, p, state=0b110, creg=c0, draws=[0.5], measure_op=m_op)
        assert (st, used, c) == (0, 1, want)
    p = Program([(MultiOp(), ("measure", 0b110, 0b1))])  # only q bit 1 -> c bit 0
    st, used, c, _ = run_harness(harness, 3, 2, p, state=0b100, creg=0b11, draws=[0.5])
    assert (st, c) == (0, 0b10)


@pytest.mark.parametrize("measure_op", ["set", "xor"])
def test_runner_matches_restatement(harness, measure_op):
    for seed in range(1, 41):
        n = 3 + seed % 6
        c_num = 1 + seed % 5
        p, nmeas = random_program(n, c_num, 12 + seed % 9, seed)
        rng = SplitMix64(seed + 99)
        draws = [rng.uniform() for _ in range(nmeas)]
        state = rng.next_u64() & ((1 << n) - 1)
        creg = rng.next_u64() & ((1 << c_num) - 1)
        st, used, c, psi = run_harness(harness, n, c_num, p, state, creg, draws, measure_op)
        want, wc, wd = sym_finish_ref(n, c_num, p, state, creg, draws, measure_op)
        assert st == 0 and used == wd == nmeas
        assert c == wc, seed
        assert np.array_equal(psi, want), seed


def test_teleport_program(harness):
    """A teleport-style program: the state prepared on qubit 0 reaches qubit 2 after the Bell
    measurement and the classically controlled corrections, for every outcome."""
    th, ph = 1.1, 0.7
    prep = op.ry(th, 0b001) * op.rz(ph, 0b001)
    p = (Program().apply(prep).apply(op.h(0b010)).apply(op.x(0b100).c(0b010))
         .apply(op.x(0b010).c(0b001)).apply(op.h(0b001)).measure(0b011, 0b011)
         .if_branch(0b10, 1, op.x(0b100)).if_branch(0b01, 1, op.z(0b100)))
    ref = orc.new_state(1, 0)
    orc.apply(prep.gates(), ref)
    want = ref[:2] / np.linalg.norm(ref[:2])
    outcomes = set()
    for u in np.linspace(0.01, 0.99, 25):
        st, used, c, psi = run_harness(harness, 3, 2, p, draws=[u])
        assert st == 0 and used == 1
        outcomes.add(c)
        amps = psi[[c, c | 0b100]]  # qubits 0, 1 collapsed onto the measured bits
        amps = amps / np.linalg.norm(amps)
        assert abs(abs(np.vdot(want, amps)) - 1.0) <= 1e-12
    assert outcomes == {0, 1, 2, 3}


def blocks_of(*rows):
    arr = (_abi.QvntBlock * len(rows))()
    for i, (sep, count, a, b, res) in enumerate(rows):
        arr[i].sep, arr[i].gate_count, arr[i].a, arr[i].b, arr[i].reserved = sep, count, a, b, res
    return arr


def test_invalid_programs_change_nothing(harness):
    base = Program().apply(op.h(0b111)).measure(0b1, 0b1)
    cases = [
        dict(draws=[]),                                   # a measurement without a draw
        dict(draws=[1.0]),                                # draw outside [0, 1)
        dict(draws=[float("nan")]),
        dict(draws=[0.5], measure_op=7),                  # unknown measure op
        dict(draws=[0.5], c_num=65),
        dict(draws=[0.5], blocks_override=blocks_of((_abi.SEP_NOP, 2, 0, 0, 0), (9, 0, 0, 0, 0))),
        dict(draws=[0.5], blocks_override=blocks_of((_abi.SEP_NOP, 2, 0, 0, 1))),
    ]
    for case in cases:
        c_num = case.pop("c_num", 2)
        st, used, c, psi = run_harness(harness, 3, c_num, base, creg=0b10, **case)
        assert st == _abi.ERR_BAD_ARG, case
        assert (used, c) == (0, 0b10)
        assert np.array_equal(psi, orc.new_state(3, 0))


def test_python_entry_marshals_to_the_library(lib_built):
    """run_program's ctypes call reaches qvnt_program_run, which rejects a null register first."""
    p = Program().apply(op.h(0b11)).measure(0b1, 0b1).if_branch(1, 1, op.x(2))
    with pytest.raises(QvntError) as e:
        run_program(None, p, 2, 0, [0.25])
    assert e.value.status == _abi.ERR_BAD_HANDLE


# ------------------------------------------------------------------------------ ops-tree text

def test_ops_tree_format():
    """qvnt's `Debug` of `int::Op` (ext_op.rs:77-112): the first block prints its list with `{:?}`,
    later empty lists print nothing, an IF block always starts with " -> ", masks print in binary."""
    x6, h7, z2, y3 = op.x(0b110), op.h(0b111), op.z(0b010), op.y(0b011)
    dummy = Program([(x6, NOP), (h7 * z2, ("measure", 0, 0))], y3)  # ext_op.rs:120-129
    assert dummy.ops_tree() == "[X6] -> [H3, H4, Z2] -> Measure(0 => 0) -> [Y3]"
    assert Program().ops_tree() == "[]"
    assert Program(last=x6).ops_tree() == "[X6]"
    assert Program().if_branch(0b1, 0, op.x(4)).ops_tree() == " -> if c[1] == 0 { [X4] }"
    p = Program().measure(0b11, 0b110).reset(0b101)
    assert p.ops_tree() == "[] -> Measure(11 => 110) -> Reset(101)"
    p = Program().apply(h7).measure(0b11, 0b11).if_branch(0b10, 0b1, x6).apply(z2)
    assert p.ops_tree() == "[H3, H4] -> Measure(11 => 11) -> if c[10] == 1 { [X6] } -> [Z2]"
    assert repr(p) == p.ops_tree()


LOSSY_IN_NAMES = {KIND["S"], KIND["T"], KIND["ISWAP"], KIND["SQRT_SWAP"], KIND["SQRT_ISWAP"]}
ROTATION_KINDS = {KIND[k] for k in ("RX", "RY", "RZ", "RXX", "RYY", "RZZ")}


def name_safe_circuit(rotations):
    """all_kinds_circuit without the gates whose names lose a field (daggered S/T/iSWAP/sqrt gates,
    a U2 whose a bit is the higher one) and, optionally, without rotations."""
    def make(n, count, seed):
        keep = []
        for s in all_kinds_circuit(n, count, seed):
            g = s.g
            if (g.dagger and g.kind in LOSSY_IN_NAMES) or (g.kind == KIND["U2"] and g.a_mask > g.b_mask):
                continue
            if not rotations and g.kind in ROTATION_KINDS:
                continue
            keep.append(s)
        return MultiOp(keep)
    return make


def test_ops_tree_text_is_a_fixed_point():
    for seed in range(1, 31):
        p, _ = random_program(3 + seed % 6, 1 + seed % 5, 15, seed, name_safe_circuit(False))
        text = p.ops_tree()
        assert Program.parse(text).ops_tree() == text, seed


def test_ops_tree_parse_runs_the_same(harness):
    for seed in range(1, 31):
        n, c_num = 3 + seed % 6, 1 + seed % 5
        p, nmeas = random_program(n, c_num, 15, seed, name_safe_circuit(True))
        q = Program.parse(p.ops_tree())
        assert [s for _, s in q.blocks if s != NOP] == [s for _, s in p.blocks if s != NOP]
        rng = SplitMix64(seed)
        draws = [rng.uniform() for _ in range(nmeas)]
        st, used, c, psi = run_harness(harness, n, c_num, p, 1, 0, draws)
        st2, used2, c2, psi2 = run_harness(harness, n, c_num, q, 1, 0, draws)
        assert (st, used, c) == (st2, used2, c2) == (0, nmeas, c)
        assert np.max(np.abs(psi - psi2)) <= 1e-12, seed  # rotations come back within an ulp or two


@pytest.mark.parametrize("text", [
    "[X1] Measure(1 => 1)", "[X1] -> Measure(2 => 1)", "[X1] -> Measure(1 => )", "[X1] -> Reset()",
    "-> if c[1] == 1 [X1]", " -> if c[1] == 1 { [X1] ", "[X1] -> ", "[X1] -> Q",
    "[X1] -> Measure(" + "1" * 65 + " => 1)", "[X1, ] -> [X2]",
])
def test_ops_tree_rejects(text, lib_built):
    with pytest.raises(QvntError) as e:
        Program.parse(text)
    assert e.value.status == _abi.ERR_BAD_ARG
