"""The QASM runner (`qvnt::qasm::Sym`, src/qasm/sym.rs) over the engine's ``qvnt_program_run``.

A program is qvnt's interpreted form ``int::Op`` (src/qasm/int/ext_op.rs:6-16): ``(MultiOp, Sep)``
blocks and a trailing MultiOp.  ``Program`` builds it the way qvnt's interpreter does statement by
statement (``apply``, ``measure``, ``reset``, ``if_branch``; src/qasm/int/mod.rs:207-305, 374-384),
including its quirk: an ``if`` right after unitary gates joins their NOP block unconditionally
(``branch(Nop)`` then ``push`` merges into that block, and the IF separator is then dropped), and
``Sym`` runs it on a device register with one ``qvnt_program_run`` call per ``finish``.  The
OpenQASM text parser (qvnt's ``Ast``/``Int`` front end, from the qvnt-qasm crate) is not part of this
package: the caller builds the program.

Separators are tuples: ``("nop",)``, ``("measure", q_mask, c_mask)``, ``("if", c_mask, value)``,
``("reset", q_mask)``.  Measurements take uniform draws in [0, 1): passed to ``finish``, or drawn
from Python's ``random`` when omitted (qvnt draws from ``thread_rng``).
"""
import ctypes
import random

from . import _abi
from ._abi import QvntBlock, check, gate_array, lib
from .operator import MultiOp, SingleOp
from .register import CReg, QReg

NOP = ("nop",)
_SEP_CODE = {"nop": _abi.SEP_NOP, "measure": _abi.SEP_MEASURE, "if": _abi.SEP_IF, "reset": _abi.SEP_RESET}


def _multi(op):
    if op is None:
        return MultiOp()
    if isinstance(op, SingleOp):
        return MultiOp.from_single(op)
    return op


class Program:
    """``int::Op``: ``blocks`` = [(MultiOp, sep)], ``last`` = trailing MultiOp."""

    def __init__(self, blocks=None, last=None):
        self.blocks = list(blocks or [])
        self.last = _multi(last)

    def is_empty(self):
        return not self.blocks and len(self.last) == 0

    def push(self, op):
        """ext_op.rs:40-50: joins a trailing Nop block when nothing is pending."""
        op = _multi(op)
        if len(self.last) == 0:
            if self.blocks and self.blocks[-1][1] == NOP:
                ops, sep = self.blocks[-1]
                self.blocks[-1] = (ops * op, sep)
            else:
                self.last = op
        else:
            self.last = self.last * op
        return self

    def append(self, other):
        """ext_op.rs:22-38: this program, then ``other``."""
        last, self.last = self.last, other.last
        if len(last):
            if self.blocks and self.blocks[-1][1] == NOP:
                ops, sep = self.blocks[-1]
                self.blocks[-1] = (ops * last, sep)
            else:
                self.blocks.append((last, NOP))
        self.blocks.extend(other.blocks)
        return self

    def __mul__(self, other):
        return Program(self.blocks, self.last).append(Program(other.blocks, other.last))

    def _branch(self, sep):
        """int/mod.rs:374-379: the pending gates become a block, if there are any."""
        if len(self.last):
            self.blocks.append((self.last, sep))
            self.last = MultiOp()

    def _branch_with_id(self, sep):
        """int/mod.rs:381-384: the pending gates, even none, become a block."""
        self.blocks.append((self.last, sep))
        self.last = MultiOp()

    # One statement each, on the program being built, as the interpreter processes them.
    def apply(self, op):
        """A gate statement (int/mod.rs:233-260): `push`."""
        return self.push(op)

    def measure(self, q_mask, c_mask):
        """`measure q -> c` (int/mod.rs:213-231): bit counts must match."""
        if bin(q_mask).count("1") != bin(c_mask).count("1"):
            raise ValueError("measure: %d qubits into %d bits" % (bin(q_mask).count("1"), bin(c_mask).count("1")))
        self._branch_with_id(("measure", q_mask, c_mask))
        return self

    def reset(self, q_mask):
        """`reset q` (int/mod.rs:207-211)."""
        self._branch_with_id(("reset", q_mask))
        return self

    def if_branch(self, c_mask, value, op):
        """`if (c == value) gate` (int/mod.rs:286-305): branch(Nop), push the gate, branch(If).
        After unitary gates the push joins their NOP block and the gate runs unconditionally."""
        self._branch(NOP)
        self.push(op)
        self._branch(("if", c_mask, value))
        return self

    def measure_count(self):
        return sum(1 for _, sep in self.blocks if sep[0] == "measure")

    def lower(self):
        """(gate array, gate count, block array, block count, trailing gate count)."""
        gates, blocks = [], (QvntBlock * max(len(self.blocks), 1))()
        for i, (ops, sep) in enumerate(self.blocks):
            g = ops.gates()
            gates += g
            blocks[i].sep = _SEP_CODE[sep[0]]
            blocks[i].gate_count = len(g)
            if len(sep) > 1:
                blocks[i].a = sep[1]
            if len(sep) > 2:
                blocks[i].b = sep[2]
        tail = self.last.gates()
        gates += tail
        return gate_array(gates), len(gates), blocks, len(self.blocks), len(tail)

    def ops_tree(self):
        """qvnt's `Debug` of `int::Op` (ext_op.rs:77-112), `Int::get_ops_tree`'s text."""
        garr, _, barr, nb, tail = self.lower()
        need = ctypes.c_size_t()
        check(lib().qvnt_program_format(garr, barr, nb, tail, None, 0, ctypes.byref(need)))
        buf = ctypes.create_string_buffer(need.value + 1)
        check(lib().qvnt_program_format(garr, barr, nb, tail, buf, need.value + 1, ctypes.byref(need)))
        return buf.value.decode()

    @staticmethod
    def parse(text):
        """The program of an ops-tree text (qvnt_program_parse)."""
        raw = text.encode() if isinstance(text, str) else bytes(text)
        ng, nb, tail = ctypes.c_size_t(), ctypes.c_uint32(), ctypes.c_uint64()
        check(lib().qvnt_program_parse(raw, len(raw), None, 0, ctypes.byref(ng), None, 0, ctypes.byref(nb),
                                       ctypes.byref(tail)))
        garr = (_abi.QvntGate * max(ng.value, 1))()
        barr = (QvntBlock * max(nb.value, 1))()
        check(lib().qvnt_program_parse(raw, len(raw), garr, ng.value, ctypes.byref(ng), barr, nb.value,
                                       ctypes.byref(nb), ctypes.byref(tail)))
        names = {v: k for k, v in _SEP_CODE.items()}
        ops = [SingleOp(_copy(garr[i])) for i in range(ng.value)]
        p, g0 = Program(), 0
        for i in range(nb.value):
            k = barr[i]
            name = names[k.sep]
            sep = {"nop": NOP, "measure": ("measure", k.a, k.b), "if": ("if", k.a, k.b), "reset": ("reset", k.a)}[name]
            p.blocks.append((MultiOp(ops[g0:g0 + k.gate_count]), sep))
            g0 += k.gate_count
        p.last = MultiOp(ops[g0:])
        return p

    def __repr__(self):
        return self.ops_tree()


def _copy(g):
    out = _abi.QvntGate()
    ctypes.memmove(ctypes.byref(out), ctypes.byref(g), ctypes.sizeof(_abi.QvntGate))
    return out


def run_program(reg, program, c_num, creg_value=0, draws=None, measure_op="set"):
    """One ``qvnt_program_run``: returns (classical value, draws used)."""
    garr, _, barr, nb, tail = program.lower()
    nm = program.measure_count()
    if draws is None:
        draws = [random.random() for _ in range(nm)]
    darr = (ctypes.c_double * max(len(draws), 1))(*[float(u) for u in draws])
    c = ctypes.c_uint64(creg_value)
    used = ctypes.c_uint32()
    op_code = {"set": _abi.MEASURE_SET, "xor": _abi.MEASURE_XOR}[measure_op]
    check(lib().qvnt_program_run(reg.h if reg is not None else None, c_num, op_code, garr, barr, nb, tail, darr,
                                 len(draws), ctypes.byref(c), ctypes.byref(used)))
    return c.value, used.value


class Sym:
    """``qvnt::qasm::Sym`` (sym.rs:7-99): a program with its quantum and classical registers."""

    def __init__(self, program, q_num, c_num, measure_op="set", ctx=None, engine=None):
        self.program = program
        self.m_op = measure_op
        self.q_reg = QReg(q_num, 0, ctx, engine)
        self.c_reg = CReg.new(c_num)

    def reset(self):
        """sym.rs:35-38"""
        self.q_reg.reset(0)
        self.c_reg.reset(0)

    def finish(self, draws=None):
        """sym.rs:40-74: runs every block, then the trailing gates."""
        value, _ = run_program(self.q_reg, self.program, self.c_reg.num(), self.c_reg.get(), draws, self.m_op)
        self.c_reg.value = value
        return self

    def measure(self, q_arg, c_arg, u01=None):
        """sym.rs:76-87: one measurement outside the program."""
        p = Program([(MultiOp(), ("measure", q_arg, c_arg))])
        value, _ = run_program(self.q_reg, p, self.c_reg.num(), self.c_reg.get(),
                               None if u01 is None else [u01], self.m_op)
        self.c_reg.value = value

    def get_class(self):
        return CReg(self.c_reg.num(), self.c_reg.get())

    def get_polar_wavefunction(self):
        return self.q_reg.get_polar()

    def get_probabilities(self):
        return self.q_reg.get_probabilities()

    def amplitudes(self):
        return self.q_reg.amplitudes()


__all__ = ["Program", "Sym", "run_program", "NOP"]
