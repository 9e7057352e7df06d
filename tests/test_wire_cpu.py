"""CPU tests of the gate-list wire formats (host-only entry points; no kernel runs).

Text: qvnt's own operator names from its tests (the golden fixture) parse back to the gates the
constructors build, and print again unchanged.  Binary: streams decode to the same bytes for any
field contents, match an independent encoder written from the format's description, and every
corruption (bit flip, truncation, extension, bad counts) is rejected without a crash.
"""
import ctypes
import math
import random
import struct
import zlib

import pytest

from qvnt_gb300 import _abi, op, wire
from qvnt_gb300._abi import KIND, QvntError, QvntGate
from qvnt_gb300.operator import MultiOp, SingleOp

# Kinds whose names carry no dagger (s.rs:27-29, t.rs:37-39, i_swap.rs:39-41, sqrt_swap.rs:39-41,
# sqrt_i_swap.rs:39-41).
NO_DAGGER_IN_NAME = {"S", "T", "ISWAP", "SQRT_SWAP", "SQRT_ISWAP"}
ROTATIONS = {"RX", "RY", "RZ", "RXX", "RYY", "RZZ"}
KIND_NAME = {v: k for k, v in KIND.items()}


def gbytes(g):
    return bytes(g)


def build_case_gate(spec):
    s = op.SingleOp._make(spec["kind"], spec["a"], spec["b"], spec["angle"],
                          None if spec["matrix"] is None else
                          [complex(spec["matrix"][2 * i], spec["matrix"][2 * i + 1])
                           for i in range(len(spec["matrix"]) // 2)])
    assert s is not None
    return s.dgr() if spec["dgr"] else s


def test_parse_reference_gate_names(golden, lib_built):
    """Every single-gate name asserted by qvnt's atomic tests parses to that gate."""
    checked = 0
    for case in golden["matrix_cases"]:
        spec = case["gates"][0]
        built = build_case_gate(spec)
        parsed = wire.parse_ops(case["name"])
        assert len(parsed) == 1, case["cite"]
        assert parsed[0].name() == case["name"], case["cite"]
        kind = spec["kind"]
        if spec["dgr"] and kind in NO_DAGGER_IN_NAME:
            # the name is that of the undaggered gate
            assert gbytes(parsed[0].g) == gbytes(build_case_gate(dict(spec, dgr=False)).g), case["cite"]
        elif spec["dgr"] and kind in ROTATIONS:
            # R(theta).dgr() prints -theta; parsing builds R(-theta), the same rotation
            assert parsed[0].g.kind == built.g.kind and parsed[0].g.a_mask == built.g.a_mask
            assert abs(parsed[0].g.phase[0] - built.g.phase[0]) <= 1e-15
            assert abs(parsed[0].g.phase[1] - built.g.phase[1]) <= 1e-15
        elif kind == "H2":
            # "H3" holds a | b only; parsing pairs the bits as op::h does (a the higher bit), the
            # atomic test built (a, b) = (1, 2).  H (x) H is symmetric in a and b.
            p = parsed[0].g
            assert (p.kind, p.a_mask | p.b_mask, p.ctrl) == (built.g.kind, built.g.a_mask | built.g.b_mask, 0)
            assert p.a_mask > p.b_mask
        else:
            assert gbytes(parsed[0].g) == gbytes(built.g), case["cite"]
        checked += 1
    assert checked == len(golden["matrix_cases"]) >= 20


def test_parse_reference_list_and_control_names(golden, lib_built):
    for case in golden["register_cases"]:
        ops = op.h(0b1111) * op.h(0b0011).c(0b1000) * op.swap(0b1001).c(0b0010)
        assert wire.ops_name(ops) == case["names"] == repr(ops)
        parsed = wire.parse_ops(case["names"])
        assert [gbytes(g) for g in parsed.gates()] == [gbytes(g) for g in ops.gates()]
    for case in golden["name_cases"]:
        s = op.x(case["gate"]["a"])[0]
        assert gbytes(wire.parse_ops(case["name"])[0].g) == gbytes(s.g)
        assert gbytes(wire.parse_ops(case["c_name"])[0].g) == gbytes(s.c(case["c"]).g)


def random_ops(rng, count, q=10):
    """A list of valid gates of every kind, some controlled, some daggered."""
    out = []
    while len(out) < count:
        kind = rng.choice(sorted(KIND))
        bits = rng.sample(range(q), 4)
        one, two = 1 << bits[0], (1 << bits[0]) | (1 << bits[1])
        ang = rng.uniform(-7, 7)
        if kind in ("X", "Y", "Z", "S", "T"):
            s = op.SingleOp._make(kind, one | ((1 << bits[1]) if rng.random() < .5 else 0))
        elif kind in ("RX", "RY", "RZ"):
            s = op.SingleOp._make(kind, one, angle=ang)
        elif kind in ("RXX", "RYY", "RZZ"):
            s = op.SingleOp._make(kind, two, angle=ang)
        elif kind in ("SWAP", "ISWAP", "SQRT_SWAP", "SQRT_ISWAP"):
            s = op.SingleOp._make(kind, two)
        elif kind == "H1":
            s = op.SingleOp._make(kind, one)
        elif kind == "H2":
            lo, hi = sorted([1 << bits[0], 1 << bits[1]])
            s = op.SingleOp._make(kind, hi, lo)  # op::h's pairing (multi/h.rs:14-45)
        elif kind == "U1":
            c, sn = math.cos(ang), math.sin(ang)
            s = op.u1_matrix(one, [c, 1j * sn, 1j * sn, c])
        elif kind == "U2":
            a, b = sorted([1 << bits[0], 1 << bits[1]])
            th = rng.uniform(0, 3)
            c, sn = math.cos(th), math.sin(th)
            m = [c, 1j * sn, 0, 0, 1j * sn, c, 0, 0, 0, 0, c, -sn, 0, 0, sn, c]
            s = op.SingleOp._make(kind, a, b, matrix=m)
        else:  # ID
            s = op.SingleOp._make(kind, 0)
        if s is None:
            continue
        if rng.random() < 0.3:
            s = s.dgr()
        if rng.random() < 0.4:
            c = s.c(1 << bits[2])
            s = c if c is not None else s
        out.append(s)
    return MultiOp(out)


def test_text_round_trip_of_random_lists(lib_built):
    rng = random.Random(7)
    for trial in range(20):
        ops = random_ops(rng, 40)
        text = wire.ops_name(ops)
        assert text == repr(ops)
        parsed = wire.parse_ops(text)
        assert len(parsed) == len(ops)
        for a, b in zip(ops, parsed):
            ka = KIND_NAME[a.g.kind]
            assert (b.g.kind, b.g.ctrl, b.g.a_mask | b.g.b_mask) == (a.g.kind, a.g.ctrl, a.g.a_mask | a.g.b_mask)
            if ka in ROTATIONS:
                assert abs(b.g.phase[0] - a.g.phase[0]) <= 2e-16 * 4
                assert abs(b.g.phase[1] - a.g.phase[1]) <= 2e-16 * 4
            elif ka in NO_DAGGER_IN_NAME:
                assert b.g.dagger == 0
            elif ka in ("U1", "U2"):
                # shortest round-trip digits: the matrix comes back bit for bit
                assert bytes(b.g.matrix) == bytes(a.g.matrix)
                assert (b.g.a_mask, b.g.b_mask) == (a.g.a_mask, a.g.b_mask)
            else:
                assert gbytes(b.g) == gbytes(a.g)


def test_matrix_names_parse_exactly(lib_built):
    # Debug forms with exponents and negative zero (u1.rs:27-33 prints the matrix with {:?})
    z = ("Complex { re: 0.7071067811865476, im: 0.0 }", "Complex { re: 0.7071067811865476, im: -0.0 }",
         "Complex { re: 0.7071067811865476, im: 0.0 }", "Complex { re: -0.7071067811865476, im: 1e-300 }")
    text = "U4[[%s, %s], [%s, %s]]" % z
    g = wire.parse_ops(text)[0]
    assert g.name() == text
    assert math.copysign(1.0, g.g.matrix[3]) == -1.0 and g.g.matrix[7] == 1e-300
    with pytest.raises(QvntError):
        wire.parse_ops("U4[[Complex { re: 1.0, im: 0.0 }, Complex { re: 1.0, im: 0.0 }], "
                       "[Complex { re: 0.0, im: 0.0 }, Complex { re: 1.0, im: 0.0 }]]")  # not unitary


@pytest.mark.parametrize("text", [
    "", "X", "Q1", "RX1(", "RX1()", "RX1(nan)", "RX1(inf)", "RX1(1e999)", "[X1,", "[X1 Y2]", "X1 Y2", "RX3(0.5)",
    "C1_X1", "C_X1", "H7", "SWAP1", "sqrt(SWAP3", "X18446744073709551616", "U1[[Complex { re: 1.0, im: 0.0 }]]",
    "U1[[Complex { re: 1.0, im: 0.0 }, Complex { re: 0.0, im: 0.0 }], [Complex { re: 0.0, im: 0.0 }]]",
    "[[X1]]", "x1", "X-1", "X+1", "RX1(+1)", "RX1(0x10)",
])
def test_parse_rejects(text, lib_built):
    with pytest.raises(QvntError) as e:
        wire.parse_ops(text)
    assert e.value.status == _abi.ERR_BAD_ARG


def test_parse_never_crashes_on_mutations(lib_built):
    rng = random.Random(11)
    base = repr(random_ops(rng, 12))
    alphabet = "[](){},_:. -0123456789eCXYZSTHUIdRiqrtsWAPmlxpnf"
    for _ in range(3000):
        s = list(base)
        for _ in range(rng.randint(1, 4)):
            i = rng.randrange(len(s))
            r = rng.random()
            if r < 0.4:
                s[i] = rng.choice(alphabet)
            elif r < 0.7:
                del s[i]
            else:
                s.insert(i, rng.choice(alphabet))
        try:
            wire.parse_ops("".join(s))
        except QvntError as e:
            assert e.status == _abi.ERR_BAD_ARG


# ------------------------------------------------------------------------------------------ binary

def py_varint(v):
    out = bytearray()
    while v >= 0x80:
        out.append((v & 0x7F) | 0x80)
        v >>= 7
    out.append(v)
    return bytes(out)


def py_encode_gates(gates, typ=1, request=None):
    """The stream written from the format's description, independently of the library."""
    b = bytearray(b"QVNW" + bytes([1, typ, 0, 0]))
    b += py_varint(len(gates))
    if request is not None:
        q, st, fl, calls = request
        b += py_varint(q) + py_varint(st) + py_varint(fl) + py_varint(len(calls))
    for g in gates:
        ph = bytes((ctypes.c_double * 2)(*g.phase))
        m = bytes((ctypes.c_double * 32)(*g.matrix))
        f = (g.dagger and 1) | (2 if g.b_mask else 0) | (4 if g.ctrl else 0) | (8 if any(ph) else 0) | \
            (16 if any(m[:64]) else 0) | (32 if any(m[64:]) else 0)
        b += bytes([g.kind, f]) + py_varint(g.a_mask)
        if g.b_mask:
            b += py_varint(g.b_mask)
        if g.ctrl:
            b += py_varint(g.ctrl)
        if f & 8:
            b += ph
        if f & 16:
            b += m[:64]
        if f & 32:
            b += m[64:]
    if request is not None:
        for c in request[3]:
            b += bytes([c.op]) + py_varint(c.gate_count) + py_varint(c.mask) + struct.pack("<d", c.u01)
    return bytes(b + struct.pack("<I", zlib.crc32(bytes(b))))


def random_raw_gates(rng, n):
    """Gates with arbitrary field contents: NaN and denormal bit patterns, any masks."""
    gates = []
    for _ in range(n):
        g = QvntGate()
        raw = bytearray(rng.getrandbits(8) for _ in range(ctypes.sizeof(QvntGate)))
        ctypes.memmove(ctypes.byref(g), bytes(raw), len(raw))
        g.kind = rng.randrange(20)
        g.dagger = rng.randrange(2)
        r = rng.random()
        if r < 0.3:
            g.b_mask = 0
        if r < 0.5:
            g.ctrl = 0
        if rng.random() < 0.5:
            for k in range(32):
                g.matrix[k] = 0.0
        elif rng.random() < 0.5:
            for k in range(8, 32):
                g.matrix[k] = 0.0
        if rng.random() < 0.3:
            g.phase[0] = g.phase[1] = 0.0
        gates.append(g)
    return gates


def test_binary_round_trip_is_bit_exact(lib_built):
    rng = random.Random(3)
    for n in (0, 1, 2, 17, 300):
        gates = random_raw_gates(rng, n)
        data = wire.encode_gates(gates)
        assert data == py_encode_gates(gates)
        back = wire.decode_gates(data)
        assert [gbytes(g) for g in back.gates()] == [gbytes(g) for g in gates]
    ops = op.qft(0xFFFF) * random_ops(rng, 100)
    assert wire.decode_gates(wire.encode_gates(ops)) == ops


def test_binary_frame(lib_built):
    data = wire.encode_gates(op.x(1))
    assert data[:8] == b"QVNW\x01\x01\x00\x00"
    assert struct.unpack("<I", data[-4:])[0] == zlib.crc32(data[:-4])
    assert zlib.crc32(b"123456789") == 0xCBF43926  # the CRC's published check value
    with pytest.raises(QvntError):
        wire.decode_request(data)  # a gate list is not a request


def expect_bad(fn, data):
    with pytest.raises(QvntError) as e:
        fn(data)
    assert e.value.status == _abi.ERR_BAD_ARG


def test_binary_rejects_corruption(lib_built):
    rng = random.Random(5)
    data = wire.encode_gates(random_raw_gates(rng, 6))
    for i in range(len(data)):
        for bit in range(8):
            bad = bytearray(data)
            bad[i] ^= 1 << bit
            expect_bad(wire.decode_gates, bytes(bad))
    for k in range(len(data)):
        expect_bad(wire.decode_gates, data[:k])
    expect_bad(wire.decode_gates, data + b"\0")


def with_crc(body):
    return bytes(body) + struct.pack("<I", zlib.crc32(bytes(body)))


def test_binary_rejects_malformed_contents(lib_built):
    """Streams with a valid CRC whose contents are wrong."""
    hdr = b"QVNW\x01\x01\x00\x00"
    expect_bad(wire.decode_gates, with_crc(b"QVNX\x01\x01\x00\x00\x00"))       # magic
    expect_bad(wire.decode_gates, with_crc(b"QVNW\x02\x01\x00\x00\x00"))       # version
    expect_bad(wire.decode_gates, with_crc(b"QVNW\x01\x01\x01\x00\x00"))       # reserved
    expect_bad(wire.decode_gates, with_crc(hdr + py_varint(1) + bytes([20, 0, 1])))   # kind
    expect_bad(wire.decode_gates, with_crc(hdr + py_varint(1) + bytes([1, 64, 1])))   # field bits
    expect_bad(wire.decode_gates, with_crc(hdr + py_varint(1) + bytes([1, 0]) + b"\xff" * 10 + b"\x01"))  # varint
    expect_bad(wire.decode_gates, with_crc(hdr + py_varint(1) + bytes([1, 0]) + b"\xff" * 9 + b"\x02"))   # 65 bits
    expect_bad(wire.decode_gates, with_crc(hdr + py_varint(2**64 - 1) + bytes([1, 0, 1])))  # huge count
    expect_bad(wire.decode_gates, with_crc(hdr + py_varint(2) + bytes([1, 0, 1])))  # count beyond the records
    expect_bad(wire.decode_gates, with_crc(hdr + py_varint(1) + bytes([1, 8, 1]) + b"\0" * 15))  # short phase
    ok = with_crc(hdr + py_varint(1) + bytes([1, 0]) + b"\xff" * 9 + b"\x01")  # 2^64 - 1 fits
    assert wire.decode_gates(ok)[0].g.a_mask == 2**64 - 1
    with pytest.raises(QvntError):
        wire.encode_gates([QvntGate(kind=20)])
    with pytest.raises(QvntError):
        wire.encode_gates([QvntGate(kind=1, dagger=2)])


def test_binary_decoder_never_crashes(lib_built):
    rng = random.Random(9)
    base = wire.encode_gates(random_raw_gates(rng, 5))
    accepted = 0
    for _ in range(4000):
        body = bytearray(base[:-4])
        for _ in range(rng.randint(1, 3)):
            i = rng.randrange(8, len(body))
            r = rng.random()
            if r < 0.5:
                body[i] = rng.getrandbits(8)
            elif r < 0.75 and len(body) > 9:
                del body[i]
            else:
                body.insert(i, rng.getrandbits(8))
        try:
            wire.decode_gates(with_crc(body))
            accepted += 1
        except QvntError as e:
            assert e.status == _abi.ERR_BAD_ARG
    assert accepted > 0  # mutations of the float payloads stay valid


def test_request_round_trip(lib_built):
    rng = random.Random(13)
    ops = random_ops(rng, 30)
    calls = [("apply", 10), ("measure", 0b101, 0.25), ("apply", 0), ("apply", 20), ("measure", 1, 0.0)]
    data = wire.encode_request(12, 77, ops, calls, keep_amplitudes=True)
    carr = (_abi.QvntCall * len(calls))()
    for i, c in enumerate(calls):
        carr[i].op = _abi.CALL_APPLY if c[0] == "apply" else _abi.CALL_MEASURE
        if c[0] == "apply":
            carr[i].gate_count = c[1]
        else:
            carr[i].mask, carr[i].u01 = c[1], c[2]
    assert data == py_encode_gates(ops.gates(), typ=2, request=(12, 77, 1, list(carr)))
    r = wire.decode_request(data)
    assert (r["q_num"], r["state"], r["keep_amplitudes"], r["detached"]) == (12, 77, True, False)
    assert r["ops"] == ops and r["calls"] == calls
    r = wire.decode_request(wire.encode_request(3, 0, None, [], detached=True))
    assert (r["q_num"], len(r["ops"]), r["calls"], r["detached"]) == (3, 0, [], True)


def test_request_rejects_inconsistent_calls(lib_built):
    ops = op.h(0b111)
    with pytest.raises(QvntError):
        wire.encode_request(3, 0, ops, [("apply", 1)])              # the list holds 2 gates
    with pytest.raises(QvntError):
        wire.encode_request(3, 0, ops, [("apply", 3)])
    good = bytearray(wire.encode_request(3, 0, ops, [("apply", 2), ("measure", 1, 0.5)])[:-4])
    bad = bytearray(good)
    bad[-11] = 9   # op byte of the measure call (the last 11-byte record): unknown op
    expect_bad(wire.decode_request, with_crc(bad))
    body = b"QVNW\x01\x02\x00\x00" + py_varint(0) + py_varint(3) + py_varint(0) + py_varint(0) + py_varint(1)
    expect_bad(wire.decode_request, with_crc(body + bytes([0]) + py_varint(5) + py_varint(0) + b"\0" * 8))
    expect_bad(wire.decode_request, with_crc(body))  # one call announced, none present


def test_server_submit_request_glue(lib_built):
    """Server.submit_request hands the decoded request to Server.submit unchanged (a recording
    stand-in replaces the device submit)."""
    from qvnt_gb300.serve import Server

    class Recorder(Server):
        def __init__(self):
            self.seen = None

        def submit(self, q_num, state, gates, calls, arrival=-1.0, keep_amplitudes=False, detached=False):
            n = sum(c[1] for c in calls if c[0] == "apply")
            self.seen = (q_num, state, [bytes(gates[i]) for i in range(n)] if gates is not None else None, calls,
                         arrival, keep_amplitudes, detached)
            return 7

    ops = op.qft(0b1111) * op.x(1)
    calls = [("apply", 5), ("measure", 0b11, 0.5), ("apply", len(ops) - 5)]
    rec = Recorder()
    assert rec.submit_request(wire.encode_request(4, 2, ops, calls, keep_amplitudes=True), arrival=1.5) == 7
    assert rec.seen == (4, 2, [bytes(g) for g in ops.gates()], calls, 1.5, True, False)
    rec.submit_request(wire.encode_request(3, 0, None, [("measure", 1, 0.25)], detached=True))
    assert rec.seen == (3, 0, None, [("measure", 1, 0.25)], -1.0, False, True)
