"""The Rust shim under rust/ (qvnt's `gb300` feature: src/gpu/{ffi,reg}.rs, the per-op lowering
modules src/operator/atomic/<op>/gb300.rs, build.rs) checked on the CPU; no Rust toolchain exists
here, so the shim is read as text and its lowering is mirrored.

* ffi.rs declares exactly the C layout of `qvnt_gate`, the kind and engine numbers of the header, and
  entry points the header declares (same argument counts) and the library exports.
* Every atomic op's lowering statements (`g.<field> = self.<field> ...`), run on the fields qvnt's
  op structs store (src/operator/atomic/*.rs, e.g. rx.rs `a_mask, phase`; rxx.rs `ab_mask, phase`;
  s.rs `a_mask, dagger`; u2.rs `a_mask, b_mask, matrix`), give byte for byte the record the
  engine's builders make for the same gate; `SingleOp`'s lowering adds `ctrl`
  (src/operator/single/mod.rs:42-47), `MultiOp`'s keeps queue order.
* build.rs compiles the same units with the same FMA settings as qvnt_gb300/build.py.
"""
import ctypes
import os
import re

import pytest

import oracle_ref as orc
from qvnt_gb300 import _abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
RUST = os.path.join(ROOT, "rust")
HEADER = os.path.join(ROOT, "include", "qvnt_gb300.h")

OP_FILES = {"Id": "id", "X": "x", "RX": "rx", "RXX": "rxx", "Y": "y", "RY": "ry", "RYY": "ryy", "Z": "z", "S": "s",
            "T": "t", "RZ": "rz", "RZZ": "rzz", "U1": "u1", "U2": "u2", "H1": "h1", "H2": "h2", "Swap": "swap",
            "ISwap": "i_swap", "SqrtSwap": "sqrt_swap", "SqrtISwap": "sqrt_i_swap"}
KIND_OF_VARIANT = {"Id": "ID", "X": "X", "RX": "RX", "RXX": "RXX", "Y": "Y", "RY": "RY", "RYY": "RYY", "Z": "Z",
                   "S": "S", "T": "T", "RZ": "RZ", "RZZ": "RZZ", "U1": "U1", "U2": "U2", "H1": "H1", "H2": "H2",
                   "Swap": "SWAP", "ISwap": "ISWAP", "SqrtSwap": "SQRT_SWAP", "SqrtISwap": "SQRT_ISWAP"}


def read(*parts):
    with open(os.path.join(RUST, *parts)) as f:
        return f.read()


def test_ffi_gate_layout_and_numbers():
    src = read("src", "gpu", "ffi.rs")
    body = re.search(r"pub struct qvnt_gate \{(.*?)\}", src, re.S).group(1)
    fields = re.findall(r"pub (\w+): ([\w\[\]; 0-9]+),", body)
    want = [(name, t) for name, t in _abi.QvntGate._fields_]
    assert [f[0] for f in fields] == [w[0] for w in want]
    rust_of = {ctypes.c_uint32: "u32", ctypes.c_uint64: "u64"}
    for (name, rt), (_, ct) in zip(fields, want):
        if ct in rust_of:
            assert rt == rust_of[ct], name
        else:  # c_double arrays
            assert rt == "[f64; %d]" % ct._length_, name
    assert "size_of::<qvnt_gate>() == 304" in src
    kinds = dict((k, int(v)) for k, v in re.findall(r"pub const KIND_(\w+): u32 = (\d+);", src))
    assert kinds == _abi.KIND
    with open(HEADER) as f:
        hdr = f.read()
    for name, v in re.findall(r"pub const ENGINE_(\w+): c_int = (\d+);", src):
        assert re.search(r"QVNT_ENGINE_%s = %s\b" % (name, v), hdr), name


def test_ffi_entry_points_match_header_and_library(lib_built):
    src = read("src", "gpu", "ffi.rs")
    block = src[src.index('extern "C" {'):]
    decls = re.findall(r"pub fn (qvnt_\w+)\((.*?)\)\s*(?:->[^;]*)?;", block, re.S)
    assert len(decls) >= 20
    with open(HEADER) as f:
        hdr = f.read()
    exported = set(_abi.exported_symbols())
    for name, args in decls:
        m = re.search(r"\b%s\(([^)]*)\);" % name, hdr)
        assert m, "%s is not declared in the header" % name
        c_args = [a for a in m.group(1).split(",") if a.strip() and a.strip() != "void"]
        r_args = [a for a in args.split(",") if a.strip()]
        assert len(c_args) == len(r_args), name
        assert name in exported, name


def parse_lowering(variant):
    src = read("src", "operator", "atomic", OP_FILES[variant], "gb300.rs")
    return [ln.strip() for ln in src[src.index("fn gb300_lower"):].splitlines()[1:] if ln.strip() not in ("}", "")]


def run_lowering(stmts, op):
    """Executes the Rust lowering statements on a dict of the op's stored fields."""
    g = _abi.QvntGate()
    i = 0
    while i < len(stmts):
        s = stmts[i]
        if s.startswith("//"):
            i += 1
            continue
        m = re.fullmatch(r"g\.kind = KIND_(\w+);", s)
        if m:
            g.kind = _abi.KIND[m.group(1)]
        elif re.fullmatch(r"g\.(a_mask|b_mask) = self\.(\w+) as u64;", s):
            dst, fld = re.fullmatch(r"g\.(a_mask|b_mask) = self\.(\w+) as u64;", s).groups()
            setattr(g, dst, op[fld])
        elif s == "g.dagger = self.dagger as u32;":
            g.dagger = int(op["dagger"])
        elif s == "g.phase = [self.phase.re, self.phase.im];":
            g.phase[0], g.phase[1] = op["phase"]
        elif s == "for (i, c) in self.matrix.iter().enumerate() {":
            assert stmts[i + 1] == "g.matrix[2 * i] = c.re;" and stmts[i + 2] == "g.matrix[2 * i + 1] = c.im;"
            for k, c in enumerate(op["matrix"]):
                g.matrix[2 * k], g.matrix[2 * k + 1] = c.real, c.imag
            i += 3
            continue
        else:
            raise AssertionError("unexpected lowering statement: %r" % s)
        i += 1
    return g


def stored_fields(g):
    """The fields qvnt's op struct of this gate holds (src/operator/atomic/<op>.rs), read back
    from the record the builders made: what the Rust op would store."""
    k = _abi.KINDS[g.kind]
    two = k in ("RXX", "RYY", "RZZ", "SWAP", "ISWAP", "SQRT_SWAP", "SQRT_ISWAP")
    f = {("ab_mask" if two else "a_mask"): g.a_mask}
    if k in ("H2", "U2"):
        f["b_mask"] = g.b_mask
        f["ab_mask"] = g.a_mask | g.b_mask
    if k in ("RX", "RY", "RZ", "RXX", "RYY", "RZZ"):
        f["phase"] = (g.phase[0], g.phase[1])
    if k in ("S", "T", "ISWAP", "SQRT_SWAP", "SQRT_ISWAP"):
        f["dagger"] = bool(g.dagger)
    if k in ("U1", "U2"):
        n = 4 if k == "U1" else 16
        f["matrix"] = [complex(g.matrix[2 * i], g.matrix[2 * i + 1]) for i in range(n)]
    return f


def sample_gates():
    import math
    hh = 1 / math.sqrt(2)
    gs = [orc.make("X", 0b1011), orc.make("Y", 0b110), orc.make("Z", 0b101), orc.make("S", 0b11),
          orc.make("T", 0b1001), orc.make("RX", 0b100, angle=0.7), orc.make("RY", 0b1, angle=-2.1),
          orc.make("RZ", 0b10, angle=5.0), orc.make("RXX", 0b101, angle=1.3), orc.make("RYY", 0b1010, angle=0.2),
          orc.make("RZZ", 0b11, angle=4.4), orc.make("H1", 0b1000), orc.make("H2", 0b1, 0b100),
          orc.make("SWAP", 0b11000), orc.make("ISWAP", 0b101), orc.make("SQRT_SWAP", 0b110),
          orc.make("SQRT_ISWAP", 0b1001),
          orc.make("U1", 0b10, matrix=[hh, 0, hh, 0, hh, 0, -hh, 0]),
          orc.make("U2", 0b1, 0b10, matrix=[v for z in [hh, hh, 0, 0, hh, -hh, 0, 0, 0, 0, 1j * hh, 1j * hh, 0, 0, hh,
                                                        -hh] for v in (complex(z).real, complex(z).imag)]),
          orc.make("ID", 0)]
    out = []
    for g in gs:
        assert g is not None
        out.append(g)
        if _abi.KINDS[g.kind] in ("S", "T", "ISWAP", "SQRT_SWAP", "SQRT_ISWAP", "RX", "RXX", "U1", "U2"):
            out.append(orc.dgr(g))
        c = orc.c(g, 1 << 6)
        if c is not None:
            out.append(c)
    return out


def test_op_lowering_matches_the_engine_records():
    variant_of_kind = {v: k for k, v in KIND_OF_VARIANT.items()}
    for g in sample_gates():
        variant = variant_of_kind[_abi.KINDS[g.kind]]
        got = run_lowering(parse_lowering(variant), stored_fields(g))
        got.ctrl = g.ctrl  # SingleOp's lowering: ctrl from `SingleOp::ctrl`
        assert bytes(got) == bytes(g), (variant, _abi.KINDS[g.kind])


def test_single_and_multi_lowering():
    single = read("src", "operator", "single", "gb300.rs")
    assert "self.func.gb300_lower(&mut g);" in single and "g.ctrl = self.ctrl as u64;" in single
    multi = read("src", "operator", "multi", "gb300.rs")
    assert "for op in self.0.iter()" in multi and "out.push(op.gb300_gate());" in multi
    dispatch = read("src", "operator", "atomic", "gb300.rs")
    arms = re.findall(r"AtomicOpDispatch::(\w+)\(op\) => op\.gb300_lower\(g\),", dispatch)
    assert arms == list(OP_FILES)  # every variant, in AtomicOpDispatch order (dispatch.rs:82-105)
    assert [_abi.KIND[KIND_OF_VARIANT[a]] for a in arms] == list(range(20))


def test_build_script_compiles_the_library_units():
    from qvnt_gb300 import build
    src = read("build.rs")
    cuda = re.findall(r'\("(\w+\.cu)", (true|false)\)', src)
    want_cuda = [(u, "false" if "--fmad=false" in flags else "true") for u, flags in build.UNITS if flags is not None]
    assert sorted(cuda) == sorted(want_cuda)
    cpp = re.findall(r'"(\w+\.cpp)"', src)
    assert sorted(cpp) == sorted(u for u, flags in build.UNITS if flags is None)
    assert "arch=compute_103a,code=sm_103a" in src


def test_register_shim_covers_qreg_surface():
    src = read("src", "gpu", "reg.rs")
    for fn in ("new", "with_state", "num", "apply", "measure_mask", "measure", "get_probabilities", "get_absolute",
               "get_polar", "reset", "reset_by_mask"):
        assert re.search(r"pub fn %s\b" % fn, src), fn
    assert "impl Mul for GpuReg" in src and "impl Clone for GpuReg" in src and "impl Drop for GpuReg" in src
    # every ffi function the shim calls is declared in ffi.rs
    ffi = read("src", "gpu", "ffi.rs")
    for name in set(re.findall(r"ffi::(qvnt_\w+)\(", src)):
        assert "pub fn %s(" % name in ffi, name
