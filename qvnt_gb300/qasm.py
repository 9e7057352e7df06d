"""The QASM runner (`qvnt::qasm::Sym`, src/qasm/sym.rs) over the engine's ``qvnt_program_run``.

A program is qvnt's interpreted form ``int::Op`` (src/qasm/int/ext_op.rs:6-16): ``(MultiOp, Sep)``
blocks and a trailing MultiOp.  ``Program`` builds it the way qvnt's interpreter does statement by
statement (``apply``, ``measure``, ``reset``, ``if_branch``; src/qasm/int/mod.rs:207-305, 374-384),
including its quirk: an ``if`` right after unitary gates joins their NOP block unconditionally
(``branch(Nop)`` then ``push`` merges into that block, and the IF separator is then dropped), and
``Sym`` runs it on a device register with one ``qvnt_program_run`` call per ``finish``.  ``Ast``
and ``Int`` are the OpenQASM 2.0 front end (``Ast::from_source``, src/qasm/ast/mod.rs:13-25, whose
lexer and parser come from the qvnt-qasm crate, and ``Int::new``, src/qasm/int/mod.rs:56-60): host
code that turns program text into a ``Program``.

Separators are tuples: ``("nop",)``, ``("measure", q_mask, c_mask)``, ``("if", c_mask, value)``,
``("reset", q_mask)``.  Measurements take uniform draws in [0, 1): passed to ``finish``, or drawn
from Python's ``random`` when omitted (qvnt draws from ``thread_rng``).
"""
import ctypes
import math
import random
import re

from . import _abi
from ._abi import QvntBlock, check, gate_array, lib
from . import operator as op
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
        return Program._from_arrays(garr, ng.value, barr, nb.value)

    @staticmethod
    def _from_arrays(garr, ng, barr, nb):
        names = {v: k for k, v in _SEP_CODE.items()}
        ops = [SingleOp(_copy(garr[i])) for i in range(ng)]
        p, g0 = Program(), 0
        for i in range(nb):
            k = barr[i]
            name = names[k.sep]
            sep = {"nop": NOP, "measure": ("measure", k.a, k.b), "if": ("if", k.a, k.b), "reset": ("reset", k.a)}[name]
            p.blocks.append((MultiOp(ops[g0:g0 + k.gate_count]), sep))
            g0 += k.gate_count
        p.last = MultiOp(ops[g0:])
        return p

    def __eq__(self, other):
        return isinstance(other, Program) and self.blocks == other.blocks and self.last == other.last

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
        self.engine = engine
        self.q_reg = QReg(q_num, 0, ctx, engine)
        self.c_reg = CReg.new(c_num)

    def init(self, int_):
        """sym.rs:25-33: a new machine only when the program or the register sizes changed."""
        if (self.m_op != int_.m_op or self.program != int_.q_ops or self.q_reg.num() != len(int_.q_reg)
                or self.c_reg.num() != len(int_.c_reg)):
            ctx, self.q_reg = self.q_reg.ctx, None
            self.__init__(int_.q_ops, len(int_.q_reg), len(int_.c_reg), int_.m_op, ctx, self.engine)
        return self

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


class QasmError(ValueError):
    """A program the front end rejects (qvnt's `ast::Error` / `int::Error`)."""


# ------------------------------------------------------------------------------ expressions
# Gate arguments are expression strings evaluated as qvnt does with meval in a context holding only
# `pi` and sqrt, exp, ln, abs, floor, ceil, round, atan2, max, min (src/qasm/int/parse.rs:5-25):
# numbers, variables, + - * / % ^ (right-associative, above unary minus), parentheses, calls.

# Rust f64 semantics where Python's math module raises: NaN for domain errors, infinities for
# overflow and poles.
def _sqrt(v):
    return math.sqrt(v) if v >= 0 else (v if v != v else float("nan"))


def _ln(v):
    if v > 0:
        return math.log(v)
    return float("-inf") if v == 0 else float("nan")


def _exp(v):
    try:
        return math.exp(v)
    except OverflowError:
        return float("inf")


def _finite_only(f):
    return lambda v: float(f(v)) if math.isfinite(v) else v


def _round(v):  # half away from zero, as f64::round
    if not math.isfinite(v):
        return v
    r = math.floor(abs(v))
    return math.copysign(r + 1.0 if abs(v) - r >= 0.5 else r, v)


def _fmax(m, x):  # f64::max: a NaN operand yields the other one
    return m if x != x else (x if m != m or x > m else m)


def _fmin(m, x):
    return m if x != x else (x if m != m or x < m else m)


def _max_array(*xs):  # meval's max_array / min_array: a fold from -inf / +inf
    m = float("-inf")
    for x in xs:
        m = _fmax(m, x)
    return m


def _min_array(*xs):
    m = float("inf")
    for x in xs:
        m = _fmin(m, x)
    return m


def _div(a, b):
    if b != 0:
        return a / b
    if a != a or a == 0:
        return float("nan")
    return math.copysign(float("inf"), a) * math.copysign(1.0, b)


def _fmod(a, b):
    try:
        return math.fmod(a, b)
    except ValueError:
        return float("nan")


def _pow(a, b):
    try:
        return math.pow(a, b)
    except OverflowError:
        return float("inf")
    except ValueError:  # 0 to a negative power, or a negative base to a fractional one
        return float("inf") if a == 0 else float("nan")


_FUNCS = {"sqrt": (1, _sqrt), "exp": (1, _exp), "ln": (1, _ln), "abs": (1, abs),
          "floor": (1, _finite_only(math.floor)), "ceil": (1, _finite_only(math.ceil)), "round": (1, _round),
          "atan2": (2, math.atan2), "max": (-1, _max_array), "min": (-1, _min_array)}


def eval_expr(text, variables=()):
    """`eval_extended` (parse.rs:30-40)."""
    toks = re.findall(r"\s*(\d+\.?\d*(?:[eE][+-]?\d+)?|\.\d+(?:[eE][+-]?\d+)?|[A-Za-z_]\w*|\S)", text)
    if "".join(toks).replace(" ", "") != re.sub(r"\s+", "", text):
        raise QasmError("cannot read expression %r" % text)
    env = {"pi": math.pi}
    env.update(dict(variables))
    pos = [0]

    def peek():
        return toks[pos[0]] if pos[0] < len(toks) else None

    def take(t=None):
        tok = peek()
        if tok is None or (t is not None and tok != t):
            raise QasmError("expression %r: expected %r" % (text, t or "a term"))
        pos[0] += 1
        return tok

    def atom():
        tok = take()
        if tok == "(":
            v = add()
            take(")")
            return v
        if re.match(r"\d|\.\d", tok):
            return float(tok)
        if re.match(r"[A-Za-z_]", tok):
            if peek() == "(":
                take("(")
                args = [add()]
                while peek() == ",":
                    take(",")
                    args.append(add())
                take(")")
                if tok not in _FUNCS:
                    raise QasmError("expression %r: unknown function %r" % (text, tok))
                n, f = _FUNCS[tok]
                if n >= 0 and len(args) != n:
                    raise QasmError("expression %r: %s takes %d arguments" % (text, tok, n))
                return float(f(*args))
            if tok not in env:
                raise QasmError("expression %r: unknown variable %r" % (text, tok))
            return float(env[tok])
        raise QasmError("expression %r: unexpected %r" % (text, tok))

    def power():
        base = atom()
        if peek() == "^":
            take("^")
            return _pow(base, unary())
        return base

    def unary():
        if peek() in ("-", "+"):
            sign = -1.0 if take() == "-" else 1.0
            return sign * unary()
        return power()

    def mul():
        v = unary()
        while peek() in ("*", "/", "%"):
            o = take()
            r = unary()
            v = v * r if o == "*" else (_div(v, r) if o == "/" else _fmod(v, r))
        return v

    def add():
        v = mul()
        while peek() in ("+", "-"):
            o = take()
            r = mul()
            v = v + r if o == "+" else v - r
        return v

    v = add()
    if peek() is not None:
        raise QasmError("expression %r: trailing %r" % (text, peek()))
    return v


# ------------------------------------------------------------------------------ source -> statements

_TOKEN = re.compile(r"\s*(?:(//[^\n]*)|(\"[^\"]*\")|(->|==|[A-Za-z_][\w]*|\d+(?:\.\d*)?(?:[eE][+-]?\d+)?|\.\d+(?:[eE][+-]?\d+)?|\S))")


class Ast:
    """`Ast::from_source` (ast/mod.rs:13-25): OpenQASM 2.0 text into statements.

    Statements: ("qreg", name, size), ("creg", name, size), ("barrier",), ("reset", arg),
    ("measure", q_arg, c_arg), ("apply", name, [arg], [expr]), ("opaque",),
    ("gate", name, [reg], [param], [(name, [arg], [expr])]), ("if", creg, value, apply statement);
    an arg is (name, index) or (name, None) for a whole register; expressions stay text.
    `include` lines are skipped: the gates qelib1 defines are built in (int/gates.rs:86-126)."""

    def __init__(self, source, nodes):
        self.source = source
        self.nodes = nodes

    @staticmethod
    def from_source(source):
        toks = []
        for m in _TOKEN.finditer(source):
            if m.group(1):
                continue
            toks.append(m.group(2) or m.group(3))
        if not toks:
            raise QasmError("empty source")
        return Ast(source, _Parser(toks).program())


class _Parser:
    def __init__(self, toks):
        self.toks, self.i = toks, 0

    def peek(self, k=0):
        return self.toks[self.i + k] if self.i + k < len(self.toks) else None

    def take(self, want=None):
        t = self.peek()
        if t is None or (want is not None and t != want):
            raise QasmError("expected %r, found %r (token %d)" % (want or "a token", t, self.i))
        self.i += 1
        return t

    def ident(self):
        t = self.peek()
        if t is None or not re.match(r"[A-Za-z_]\w*$", t):
            raise QasmError("missing identifier (token %d)" % self.i)
        self.i += 1
        return t

    def integer(self):
        t = self.peek()
        if t is None or not re.match(r"[0-9]+$", t):
            raise QasmError("missing integer (token %d)" % self.i)
        if len(t) > 18:
            raise QasmError("integer too large (token %d)" % self.i)
        self.i += 1
        return int(t)

    def semi(self):
        if self.peek() != ";":
            raise QasmError("missing semicolon (token %d)" % self.i)
        self.i += 1

    def program(self):
        if self.peek() == "OPENQASM":
            self.take()
            ver = self.take()
            if ver not in ("2.0", "2"):
                raise QasmError("unsupported version %s" % ver)
            self.semi()
        nodes = []
        while self.peek() is not None:
            nodes.append(self.statement())
        return [n for n in nodes if n is not None]

    def arg(self):
        name = self.ident()
        if self.peek() == "[":
            self.take("[")
            idx = self.integer()
            self.take("]")
            return (name, idx)
        return (name, None)

    def args(self):
        out = [self.arg()]
        while self.peek() == ",":
            self.take(",")
            out.append(self.arg())
        return out

    def exprs(self):
        """Comma-separated expressions inside ( ), kept as text."""
        self.take("(")
        out, cur, depth = [], [], 0
        while True:
            t = self.take()
            if t == "(":
                depth += 1
            elif t == ")":
                if depth == 0:
                    break
                depth -= 1
            elif t == "," and depth == 0:
                out.append(" ".join(cur))
                cur = []
                continue
            cur.append(t)
        if cur or out:
            out.append(" ".join(cur))
        return out

    def apply(self):
        name = self.ident()
        params = self.exprs() if self.peek() == "(" else []
        regs = self.args()
        self.semi()
        return ("apply", name, regs, params)

    def statement(self):
        t = self.peek()
        if t == "include":
            self.take()
            self.take()
            self.semi()
            return None
        if t in ("qreg", "creg"):
            self.take()
            name = self.ident()
            self.take("[")
            size = self.integer()
            self.take("]")
            self.semi()
            return (t, name, size)
        if t == "barrier":
            self.take()
            self.args()
            self.semi()
            return ("barrier",)
        if t == "reset":
            self.take()
            a = self.arg()
            self.semi()
            return ("reset", a)
        if t == "measure":
            self.take()
            q = self.arg()
            self.take("->")
            c = self.arg()
            self.semi()
            return ("measure", q, c)
        if t == "opaque":
            self.take()
            self.ident()
            if self.peek() == "(":
                self.exprs()
            self.args()
            self.semi()
            return ("opaque",)
        if t == "gate":
            self.take()
            name = self.ident()
            params = [p.strip() for p in self.exprs()] if self.peek() == "(" else []
            regs = [a[0] for a in self.args()]
            self.take("{")
            body = []
            while self.peek() != "}":
                if self.peek() is None:
                    raise QasmError("unterminated gate %s" % name)
                if self.peek() in ("measure", "reset", "barrier", "if", "qreg", "creg", "gate"):
                    if self.peek() == "barrier":  # qelib-style bodies may hold barriers
                        self.take()
                        self.args()
                        self.semi()
                        continue
                    raise QasmError("operation %s is not allowed in gate %s" % (self.peek(), name))
                body.append(self.apply())
            self.take("}")
            return ("gate", name, regs, params, body)
        if t == "if":
            self.take()
            self.take("(")
            creg = self.ident()
            self.take("==")
            value = self.integer()
            self.take(")")
            if self.peek() in ("measure", "reset", "barrier"):
                raise QasmError("%s is not allowed in an if" % self.peek())
            return ("if", creg, value, self.apply())
        return self.apply()


# ------------------------------------------------------------------------------ statements -> program

def _bits(mask):
    return bin(mask).count("1")


def _builtin_gate(name, regs, args):
    """`gates::process` (src/qasm/int/gates.rs:86-126): a leading c/C controls the rest of the name
    by its first register; registers are OR-ed into one mask; sdg and tdg build S and T as qvnt's
    table does (its `dgr` arm calls the same constructor)."""
    if name[:1] in ("c", "C"):
        if not regs:
            raise QasmError("%s: no control register" % name)
        sub = _builtin_gate(name[1:], regs[1:], args)
        ctrl = regs[0]
        out = sub.c(ctrl)
        if out is None:
            raise QasmError("%s: control mask %d overlaps %d" % (name, ctrl, sub.act_on()))
        return out
    regs_or = 0
    for r in regs:
        regs_or |= r
    lname = name.lower()
    anymask = {"x": op.x, "y": op.y, "z": op.z, "s": op.s, "sdg": op.s, "t": op.t, "tdg": op.t, "h": op.h,
               "qft": op.qft}
    if lname in anymask and name in (lname, lname.upper()):
        if regs_or == 0:
            raise QasmError("%s: no qubits" % name)
        if args:
            raise QasmError("%s: takes no arguments" % name)
        return anymask[lname](regs_or)
    rot = {"rx": (op.rx, 1), "ry": (op.ry, 1), "rz": (op.rz, 1), "rxx": (op.rxx, 2), "ryy": (op.ryy, 2),
           "rzz": (op.rzz, 2)}
    if lname in rot and name in (lname, lname.upper()):
        f, nb = rot[lname]
        if _bits(regs_or) != nb:
            raise QasmError("%s: needs %d qubits, got %d" % (name, nb, _bits(regs_or)))
        if len(args) != 1:
            raise QasmError("%s: takes 1 argument" % name)
        return f(args[0], regs_or)
    two = {"swap": op.swap, "sqrt_swap": op.sqrt_swap, "i_swap": op.i_swap, "sqrt_i_swap": op.sqrt_i_swap}
    if lname in two and name in (lname, lname.upper()):
        if _bits(regs_or) != 2:
            raise QasmError("%s: needs 2 qubits, got %d" % (name, _bits(regs_or)))
        if args:
            raise QasmError("%s: takes no arguments" % name)
        return two[lname](regs_or)
    us = {"u1": (op.u1, 1), "u2": (op.u2, 2), "u3": (op.u3, 3)}
    if lname in us and name in (lname, lname.upper()):
        f, na = us[lname]
        if _bits(regs_or) != 1:
            raise QasmError("%s: needs 1 qubit, got %d" % (name, _bits(regs_or)))
        if len(args) != na:
            raise QasmError("%s: takes %d arguments" % (name, na))
        return f(*args, regs_or)
    raise QasmError("unknown gate %s" % name)


class _Macro:
    """`Macro` (src/qasm/int/macros.rs:57-148): a gate definition expanded at each use."""

    def __init__(self, name, regs, params, body):
        for gname, gregs, gargs in [(b[1], b[2], b[3]) for b in body]:
            for reg, idx in gregs:
                if idx is not None:
                    raise QasmError("indexing qubits (%s[%d]) isn't allowed in gate %s" % (reg, idx, name))
                if reg not in regs:
                    raise QasmError("no register %s in gate %s" % (reg, name))
            for a in gargs:  # evaluates with the parameters bound: unknown names are errors
                try:
                    eval_expr(a, [(p, 1.0) for p in params])
                except QasmError as e:
                    raise QasmError("gate %s: %s" % (name, e)) from None
        self.name, self.regs, self.params = name, regs, params
        self.body = [(b[1], [r for r, _ in b[2]], b[3]) for b in body]

    def process(self, name, regs, args, macros):
        if len(regs) != len(self.regs):
            raise QasmError("%s: takes %d registers, got %d" % (name, len(self.regs), len(regs)))
        if len(args) != len(self.params):
            raise QasmError("%s: takes %d arguments, got %d" % (name, len(self.params), len(args)))
        rmap = dict(zip(self.regs, regs))
        env = list(zip(self.params, args))
        out = MultiOp()
        for gname, gregs, gargs in self.body:
            r = [rmap[g] for g in gregs]
            a = [eval_expr(x, env) for x in gargs]
            if gname in macros:
                if gname == name:
                    raise QasmError("recursive gate %s" % name)
                out = out * macros[gname].process(gname, r, a, macros)
            else:
                out = out * _builtin_gate(gname, r, a)
        return out


class Int:
    """`Int` (src/qasm/int/mod.rs:33-400): the interpreted program, its register aliases and macros."""

    def __init__(self):
        self.m_op = "set"
        self.q_reg, self.c_reg = [], []
        self.q_ops = Program()
        self.macros = {}

    @staticmethod
    def new(ast):
        i = Int()
        i.add_ast(ast)
        return i

    @staticmethod
    def from_source(source):
        return Int.new(Ast.from_source(source))

    def xor(self):
        """`Int::xor` (mod.rs:105-110): measurements xor into the classical bits."""
        self.m_op = "xor"
        return self

    def get_ops_tree(self):
        """mod.rs:398-400"""
        return self.q_ops.ops_tree()

    def get_q_alias(self):
        """mod.rs:402-404: `{:?}` of the qubit aliases, one per qubit."""
        return "[" + ", ".join('"%s"' % a for a in self.q_reg) + "]"

    def get_c_alias(self):
        """mod.rs:406-408"""
        return "[" + ", ".join('"%s"' % a for a in self.c_reg) + "]"

    def add_ast(self, ast):
        for node in ast.nodes:
            self._node(node)
        return self

    def _mask(self, regs, alias):
        m = 0
        for i, a in enumerate(regs):
            if a == alias:
                m |= 1 << i
        return m

    def get_q_idx(self, arg):
        """arg: (name, index) or (name, None) for the whole register."""
        return self._idx(self.q_reg, arg, "qreg")

    def get_c_idx(self, arg):
        return self._idx(self.c_reg, arg, "creg")

    def _idx(self, regs, arg, what):
        """`get_q_idx` / `get_c_idx` (mod.rs:319-371): a whole register's mask, or its idx-th bit."""
        name, idx = arg
        m = self._mask(regs, name)
        if m == 0:
            raise QasmError("no %s %s" % (what, name))
        if idx is None:
            return m
        bits = [b for b in range(64) if (m >> b) & 1]
        if idx >= len(bits):
            raise QasmError("index %s[%d] out of range" % (name, idx))
        return 1 << bits[idx]

    def _declare(self, regs, name, size):
        if len(name.encode()) >= 32:
            raise QasmError("identifier %s is too long" % name)
        if size >= 64:
            raise QasmError("register %s[%d] is too large" % (name, size))
        if name in self.q_reg or name in self.c_reg:
            raise QasmError("register %s is declared twice" % name)
        if len(regs) + size > 64:
            raise QasmError("more than 64 qubits or bits in all (a mask holds 64)")
        regs.extend([name] * size)

    def _apply(self, node):
        _, name, regs, params = node
        r = [self.get_q_idx(a) for a in regs]
        a = [eval_expr(p) for p in params]
        ops = self.macros[name].process(name, r, a, self.macros) if name in self.macros else _builtin_gate(name, r, a)
        self.q_ops.push(ops)

    def _node(self, node):
        kind = node[0]
        if kind == "qreg":
            self._declare(self.q_reg, node[1], node[2])
        elif kind == "creg":
            self._declare(self.c_reg, node[1], node[2])
        elif kind in ("barrier", "opaque"):
            pass
        elif kind == "reset":
            self.q_ops.reset(self.get_q_idx(node[1]))
        elif kind == "measure":
            q, c = self.get_q_idx(node[1]), self.get_c_idx(node[2])
            if _bits(q) != _bits(c):
                raise QasmError("measure: %d qubits into %d bits" % (_bits(q), _bits(c)))
            self.q_ops.measure(q, c)
        elif kind == "apply":
            self._apply(node)
        elif kind == "gate":
            _, name, regs, params, body = node
            if name in self.macros:
                raise QasmError("gate %s is defined twice" % name)
            if len(name.encode()) >= 32:
                raise QasmError("identifier %s is too long" % name)
            self.macros[name] = _Macro(name, regs, params, body)
        elif kind == "if":
            # process_if (mod.rs:286-305): branch(Nop), the gate, branch(If)
            _, creg, value, gate = node
            val = self.get_c_idx((creg, None))
            self.q_ops._branch(NOP)
            self._apply(gate)
            self.q_ops._branch(("if", val, value))


def compile_native(source):
    """The library's C++ front end, ``qvnt_qasm_compile``: (Program, qubits, bits) for the same text
    that ``Int.from_source`` reads; raises QvntError where ``Int`` raises QasmError."""
    raw = source.encode() if isinstance(source, str) else bytes(source)
    q, c, ng, nb, tail = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_size_t(), ctypes.c_uint32(), ctypes.c_uint64()
    refs = (ctypes.byref(q), ctypes.byref(c))
    check(lib().qvnt_qasm_compile(raw, len(raw), *refs, None, 0, ctypes.byref(ng), None, 0, ctypes.byref(nb),
                                  ctypes.byref(tail)))
    garr = (_abi.QvntGate * max(ng.value, 1))()
    barr = (QvntBlock * max(nb.value, 1))()
    check(lib().qvnt_qasm_compile(raw, len(raw), *refs, garr, ng.value, ctypes.byref(ng), barr, nb.value,
                                  ctypes.byref(nb), ctypes.byref(tail)))
    return Program._from_arrays(garr, ng.value, barr, nb.value), q.value, c.value


def sym_from_int(int_, ctx=None, engine=None):
    """`Sym::new(int)` (sym.rs:16-23): registers sized by the program's declarations."""
    return Sym(int_.q_ops, len(int_.q_reg), len(int_.c_reg), int_.m_op, ctx, engine)


__all__ = ["Program", "Sym", "run_program", "NOP", "Ast", "Int", "QasmError", "eval_expr", "sym_from_int",
           "compile_native"]
