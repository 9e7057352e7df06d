"""CPU tests of the C ABI library: it loads, exports every declared symbol, and its gate builders
agree with the oracle's restatement of qvnt's constructors.  No kernel runs here."""
import ctypes
import os
import re

import numpy as np
import pytest

import oracle_ref as orc
from qvnt_gb300 import _abi, op
from qvnt_gb300._abi import KIND, QvntGate

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    names = []
    for fn in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not fn.endswith(".h"):
            continue
        src = open(os.path.join(ROOT, "include", fn)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"^[A-Za-z_][\w\s\*]*?\b(qvnt_\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol(lib_built):
    names = header_functions()
    assert len(names) > 30
    for n in names:
        assert hasattr(lib_built, n), n
    assert set(names) == set(_abi.exported_symbols()), set(names) ^ set(_abi.exported_symbols())


def test_abi_version(lib_built):
    assert lib_built.qvnt_abi_version() >> 16 == 1


def gate_bytes(g):
    return bytes(g)


def test_builders_match_oracle(lib_built):
    for mask in (0, 1, 0b1111, 0b10101, 0xFFFFF, (1 << 30) - 1, 0b1001011):
        assert [gate_bytes(s.g) for s in op.h(mask)] == [gate_bytes(g) for g in orc.op_h(mask)]
        assert [gate_bytes(s.g) for s in op.qft(mask)] == [gate_bytes(g) for g in orc.op_qft(mask)]
        assert [gate_bytes(s.g) for s in op.qft_swapped(mask)] == [gate_bytes(g) for g in orc.op_qft_swapped(mask)]
    for (th, ph, la) in ((0.1, 0.2, 0.3), (6.0, 1e-9, 3.14159)):
        assert [gate_bytes(s.g) for s in op.u3(th, ph, la, 1 << 5)] == [gate_bytes(g) for g in orc.op_u3(th, ph, la, 1 << 5)]
    for kind, mask in (("RX", 4), ("RY", 8), ("RZ", 1), ("RXX", 5), ("RYY", 6), ("RZZ", 9)):
        for ang in (1.23456, -7.5, 0.0, 100.25):
            ours = {"RX": op.rx, "RY": op.ry, "RZ": op.rz, "RXX": op.rxx, "RYY": op.ryy, "RZZ": op.rzz}[kind](ang, mask)
            assert gate_bytes(ours[0].g) == gate_bytes(orc.make(kind, mask, angle=ang))
            assert gate_bytes(ours.dgr()[0].g) == gate_bytes(orc.dgr(orc.make(kind, mask, angle=ang)))


def test_names_match_reference(golden, lib_built):
    # single-gate names of every matrix_repr test, SingleOp::name (single/mod.rs:72-78)
    for case in golden["matrix_cases"]:
        spec = case["gates"][0]
        s = op.SingleOp._make(spec["kind"], spec["a"], spec["b"], spec["angle"],
                              None if spec["matrix"] is None else
                              [complex(spec["matrix"][2 * i], spec["matrix"][2 * i + 1])
                               for i in range(len(spec["matrix"]) // 2)])
        assert s is not None, case["cite"]
        if spec["dgr"]:
            s = s.dgr()
        assert s.name() == case["name"], case["cite"]
    for case in golden["name_cases"]:
        s = op.x(case["gate"]["a"])[0]
        assert s.name() == case["name"]
        assert s.c(case["c"]).name() == case["c_name"]
    for case in golden["register_cases"]:
        ops = op.h(0b1111) * op.h(0b0011).c(0b1000) * op.swap(0b1001).c(0b0010)
        assert repr(ops) == case["names"]


def test_invalid_gates_rejected(golden, lib_built):
    for case in golden["invalid_cases"] + golden["non_unitary_cases"]:
        s = case["gate"]
        m = [complex(s["matrix"][2 * i], s["matrix"][2 * i + 1]) for i in range(len(s["matrix"]) // 2)]
        if s["kind"] == "U1":
            assert op.u1_matrix(s["a"], m) is None, case["cite"]
        else:
            assert op.u2_matrix(s["a"], s["b"], m) is None, case["cite"]
    with pytest.raises(ValueError):
        op.rx(1.0, 0b11)
    with pytest.raises(ValueError):
        op.rxx(1.0, 0b1)
    with pytest.raises(ValueError):
        op.swap(0b111)


def test_ctrl_rules(golden, lib_built):
    for case in golden["ctrl_cases"]:
        g = op.ryy(case["gate"]["angle"], case["gate"]["a"])[0]
        assert g.act_on() & case["reject"] != 0
        assert g.c(case["reject"]) is None
        assert g.c(case["accept"]) is not None
    # `op::h(0b001).c(0b010)` and friends; MultiOp::c rejects overlaps (multi/mod.rs:125-132)
    assert op.h(0b001).c(0b001) is None
    assert op.qft(0b0111).c(0b1000) is not None


def test_multiop_queue(golden, lib_built):
    case = golden["multi_cases"][0]
    pend = op.id() * op.h(0b001).c(0b010) * op.x(0b011).c(0b100) * op.rz(5.0, 0b001)
    assert len(pend) == case["len"]
    a = op.x(0x010101) * op.y(0x101010) * op.z(0x011011)
    b = op.y(0x101010) * op.z(0x011011)
    assert b.ends_with(a)
    # dgr reverses and daggers (multi/mod.rs:120-123)
    q = op.s(1) * op.t(2) * op.i_swap(3)
    d = q.dgr()
    assert [s.name() for s in d] == ["iSWAP3", "T2", "S1"]
    assert [s.g.dagger for s in d] == [1, 1, 1]


def test_bits_iter_vreg_creg(golden):
    from qvnt_gb300 import CReg, VReg, bits_iter
    for case in golden["bits_iter_cases"]:
        assert list(bits_iter(case["number"])) == case["bits"]
    v = golden["vreg_cases"][0]
    r = VReg.new(v["num"])
    for k, m in v["index"].items():
        assert r[int(k)] == m
    assert r[lambda i: i % 2 == 0] == v["even"]
    assert r[lambda i: i % 2 != 0] == v["odd"]
    assert r[:] == v["all"]
    assert r[v["pick"][0]] == v["pick"][1]
    for mask, idx, full in golden["vreg_cases"][1]["mask_cases"]:
        r = VReg.new_with_mask(mask)
        for k, m in idx.items():
            assert r[int(k)] == m
        assert r[:] == full
    c = CReg.with_state(8, 0b10110010)
    assert c.get_by_mask(0b11110000) == 0b1011
    assert repr(CReg.with_state(4, 0b0101)) == "(0101)"
    assert repr(CReg.with_state(8, 123)) == "(01111011)" and CReg.with_state(8, 123).get() == 123  # class.rs:39-47
    assert (CReg.with_state(2, 0b01) * CReg.with_state(2, 0b10)).get() == 0b1001
    assert CReg.with_state(4, 11) * CReg.with_state(4, 7) == CReg.with_state(8, 123)  # class.rs:24-31


def test_circuit_sizes(lib_built):
    from qvnt_gb300.circuits import plain_circuit, random_circuit
    c1 = plain_circuit(20, 20, seed=1)
    assert 1600 <= len(c1) <= 1620
    c2 = random_circuit(30, 40, seed=2)
    assert 2800 <= len(c2) <= 3200


def test_fused_planner_terminates_and_covers(lib_built):
    """The fused planner runs on the host: every gate list gets a finite plan at every tile width."""
    from qvnt_gb300.circuits import plain_circuit, random_circuit
    from test_gpu_parity import all_kinds_circuit
    for n in (3, 4, 5, 7, 12, 14, 20):
        circ = all_kinds_circuit(max(n, 3), 300, seed=n)
        for k in (0, 6, 8, 10, 12, 13):
            passes, stages, eg = op.plan_info(circ, n, k)
            assert 0 < passes <= max(eg, 1) + len(circ)
            if n >= 4:
                assert stages >= passes - len(circ)
    p30, s30, e30 = op.plan_info(random_circuit(30, 40, seed=2), 30)
    assert p30 < e30
    p20, _, _ = op.plan_info(plain_circuit(20, 20, seed=1), 20)
    assert p20 < 1610


def test_c_program_uses_the_abi(tmp_path):
    """The header is plain C: a C99 program includes it, links the library and drives the host-side
    entry points (builders, names, planner, wire formats, program text, QASM) that need no GPU."""
    import shutil
    import subprocess

    from qvnt_gb300._abi import LIB_PATH

    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    src = tmp_path / "abi_check.c"
    src.write_text(r"""
#include <stdio.h>
#include <string.h>
#include "qvnt_gb300.h"
int main(void) {
    qvnt_gate g[512];
    size_t n = 0;
    if (qvnt_op_qft(0xFull, g, 512, &n) != QVNT_OK || n != 10) return 1;          /* 4 H + 6 CRZ */
    qvnt_gate x;
    if (qvnt_gate_make(QVNT_GATE_X, 0x4, 0, 0.0, NULL, &x) != QVNT_OK) return 2;
    if (qvnt_gate_c(&x, 0x3) != QVNT_OK) return 3;
    char name[64];
    size_t need = 0;
    if (qvnt_gate_name(&x, name, sizeof name, &need) != QVNT_OK || strcmp(name, "C3_X4") != 0) return 4;
    if (qvnt_gate_make(QVNT_GATE_RX, 0x3, 0, 1.0, NULL, &x) != QVNT_ERR_BAD_MASK) return 5;
    uint64_t passes = 0, stages = 0, eg = 0;
    if (qvnt_plan_info(g, n, 4, 0, &passes, &stages, &eg) != QVNT_OK || passes == 0) return 6;
    /* wire formats: names -> gates -> binary stream -> gates -> names */
    const char* text = "[C3_X4, H3, RZ1(0.5)]";
    qvnt_gate p[8], back[8];
    size_t np = 0, nb = 0, len = 0;
    if (qvnt_ops_parse(text, strlen(text), p, 8, &np) != QVNT_OK || np != 3) return 7;
    unsigned char buf[1024];
    if (qvnt_wire_encode_gates(p, np, buf, sizeof buf, &len) != QVNT_OK || len > sizeof buf) return 8;
    if (qvnt_wire_decode_gates(buf, len, back, 8, &nb) != QVNT_OK || nb != 3) return 9;
    if (memcmp(p, back, 3 * sizeof(qvnt_gate)) != 0) return 10;
    buf[len / 2] ^= 1;
    if (qvnt_wire_decode_gates(buf, len, back, 8, &nb) != QVNT_ERR_BAD_ARG) return 11;
    char names[256];
    if (qvnt_ops_name(back, nb, names, sizeof names, &need) != QVNT_OK || strcmp(names, text) != 0) return 12;
    /* a runner program as qvnt's ops-tree text */
    const char* prog = "[H1] -> Measure(1 => 1) -> if c[1] == 1 { [X2] } -> [Z2]";
    qvnt_block blk[4];
    uint32_t nblk = 0;
    uint64_t tail = 0;
    if (qvnt_program_parse(prog, strlen(prog), p, 8, &np, blk, 4, &nblk, &tail) != QVNT_OK) return 13;
    if (np != 3 || nblk != 2 || tail != 1 || blk[0].sep != QVNT_SEP_MEASURE || blk[1].sep != QVNT_SEP_IF) return 14;
    if (qvnt_program_format(p, blk, nblk, tail, names, sizeof names, &need) != QVNT_OK || strcmp(names, prog) != 0)
        return 15;
    /* OpenQASM text to a runner program */
    const char* src = "OPENQASM 2.0; qreg q[2]; creg c[2]; h q[0]; cx q[0], q[1]; measure q -> c;";
    uint32_t qn = 0, cn = 0;
    if (qvnt_qasm_compile(src, strlen(src), &qn, &cn, p, 8, &np, blk, 4, &nblk, &tail) != QVNT_OK) return 16;
    if (qn != 2 || cn != 2 || np != 2 || nblk != 1 || blk[0].sep != QVNT_SEP_MEASURE || blk[0].a != 3) return 17;
    if (qvnt_qasm_compile("qreg q[1]; g q;", 15, &qn, &cn, p, 8, &np, blk, 4, &nblk, &tail) != QVNT_ERR_BAD_ARG)
        return 18;
    printf("%s %zu %llu\n", name, n, (unsigned long long)passes);
    return 0;
}
""")
    exe = tmp_path / "abi_check"
    inc = os.path.join(ROOT, "include")
    libdir = os.path.dirname(LIB_PATH)
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-I", inc, str(src), "-o", str(exe), "-L", libdir,
                        "-lqvnt_gb300", "-Wl,-rpath," + libdir], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True)
    assert run.returncode == 0, (run.returncode, run.stdout, run.stderr)
    assert run.stdout.startswith("C3_X4 10 ")


def test_norm_noalloc_argument_checks_without_gpu(lib_built):
    """qvnt_norm_sqr_noalloc refuses misaligned, null and oversized arguments on the host, before any
    CUDA call (dummy pointers: nothing is dereferenced)."""
    import ctypes

    from qvnt_gb300 import _abi

    f = lib_built.qvnt_norm_sqr_noalloc
    cases = [
        (0x1008, 64, 0x2000, b"16-byte aligned"),   # d_psi only 8-byte aligned
        (0x1000, 64, 0x2004, b"8-byte aligned"),    # d_out misaligned
        (0, 64, 0x2000, b"null"),
        (0x1000, 0, 0x2000, b"empty"),
        (0x1000, (1 << 28) + 1, 0x2000, b"allocation-free limit"),
    ]
    for psi, n, out, msg in cases:
        st = f(ctypes.c_void_p(psi), n, ctypes.c_void_p(out), None)
        assert st == _abi.ERR_BAD_ARG, (psi, n, out)
        assert msg in lib_built.qvnt_last_error(), lib_built.qvnt_last_error()
