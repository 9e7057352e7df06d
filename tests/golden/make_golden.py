"""Writes reference_tests.json: the known answers held by qvnt 0.4.4's own unit tests.

qvnt is Rust and cannot be built in this environment, so its tests cannot run here.  Each case
below restates, value for value, an `assert_eq!` / `assert!` of a qvnt test (file:line cited, paths
relative to the qvnt crate root).  Expected values that qvnt writes as expressions, e.g.
`(0.5 * ANGLE).cos()`, are evaluated with the same IEEE-754 double operations here.

Run:  python tests/golden/make_golden.py   (rewrites tests/golden/reference_tests.json)
"""
import json
import math
import os

ANGLE = 1.23456
FRAC_1_SQRT_2 = 0.7071067811865476  # std::f64::consts::FRAC_1_SQRT_2

O = (0.0, 0.0)
I = (1.0, 0.0)
i_ = (0.0, 1.0)


def neg(z):
    return (-z[0], -z[1])


def conj(z):
    return (z[0], -z[1])


COS = (math.cos(0.5 * ANGLE), 0.0)
SIN = (math.sin(0.5 * ANGLE), 0.0)
I_SIN = (0.0, math.sin(0.5 * ANGLE))
EXP = (math.cos(0.5 * ANGLE), math.sin(0.5 * ANGLE))
S2 = (FRAC_1_SQRT_2, 0.0)
H5 = (0.5, 0.0)
EXP_I_PI_4 = (FRAC_1_SQRT_2, FRAC_1_SQRT_2)
SQRT_I = (0.5, 0.5)


def g(kind, a=0, b=0, angle=0.0, matrix=None, dgr=False, ctrl=0):
    return {"kind": kind, "a": a, "b": b, "angle": angle, "matrix": matrix, "dgr": dgr, "ctrl": ctrl}


def flat(m):
    """Row-major complex matrix -> interleaved doubles (the qvnt_gate matrix field)."""
    out = []
    for z in m:
        out += [z[0], z[1]]
    return out


def dbg(z):
    """Rust `{:?}` of Complex<f64> for the values used in qvnt's U1/U2 name tests."""
    return "Complex { re: %r, im: %r }" % (z[0], z[1])


matrix_cases = [
    # (cite, gates, size, expected matrix, expected name of the single gate)
    ("src/operator/atomic/id.rs:36-38", [g("ID")], 1, [[I, O], [O, I]], "Id"),
    ("src/operator/atomic/x.rs:44-46", [g("X", 0b1)], 1, [[O, I], [I, O]], "X1"),
    ("src/operator/atomic/x.rs:48-53", [g("X", 0b01)], 2,
     [[O, I, O, O], [I, O, O, O], [O, O, O, I], [O, O, I, O]], "X1"),
    ("src/operator/atomic/y.rs:51-53", [g("Y", 0b1)], 1, [[O, neg(i_)], [i_, O]], "Y1"),
    ("src/operator/atomic/y.rs:55-60", [g("Y", 0b11)], 2,
     [[O, O, O, neg(I)], [O, O, I, O], [O, I, O, O], [neg(I), O, O, O]], "Y3"),
    ("src/operator/atomic/z.rs:48-50", [g("Z", 0b1)], 1, [[I, O], [O, neg(I)]], "Z1"),
    ("src/operator/atomic/s.rs:56-59", [g("S", 0b1, dgr=True)], 1, [[I, O], [O, neg(i_)]], "S1"),
    ("src/operator/atomic/t.rs:65-68", [g("T", 0b1, dgr=True)], 1, [[I, O], [O, conj(EXP_I_PI_4)]], "T1"),
    ("src/operator/atomic/rx.rs:66-68", [g("RX", 0b1, angle=ANGLE)], 1,
     [[COS, neg(I_SIN)], [neg(I_SIN), COS]], "RX1(1.23456)"),
    ("src/operator/atomic/ry.rs:71-73", [g("RY", 0b1, angle=ANGLE)], 1,
     [[COS, neg(SIN)], [SIN, COS]], "RY1(1.23456)"),
    ("src/operator/atomic/rz.rs:64-66", [g("RZ", 0b1, angle=ANGLE)], 1,
     [[conj(EXP), O], [O, EXP]], "RZ1(1.23456)"),
    ("src/operator/atomic/rxx.rs:68-78", [g("RXX", 0b11, angle=ANGLE)], 2,
     [[COS, O, O, neg(I_SIN)], [O, COS, neg(I_SIN), O], [O, neg(I_SIN), COS, O], [neg(I_SIN), O, O, COS]],
     "RXX3(1.23456)"),
    ("src/operator/atomic/ryy.rs:72-82", [g("RYY", 0b11, angle=ANGLE)], 2,
     [[COS, O, O, I_SIN], [O, COS, neg(I_SIN), O], [O, neg(I_SIN), COS, O], [I_SIN, O, O, COS]],
     "RYY3(1.23456)"),
    ("src/operator/atomic/ryy.rs:84-98", [g("RYY", 0b110, angle=ANGLE)], 3,
     [[COS, O, O, O, O, O, I_SIN, O],
      [O, COS, O, O, O, O, O, I_SIN],
      [O, O, COS, O, neg(I_SIN), O, O, O],
      [O, O, O, COS, O, neg(I_SIN), O, O],
      [O, O, neg(I_SIN), O, COS, O, O, O],
      [O, O, O, neg(I_SIN), O, COS, O, O],
      [I_SIN, O, O, O, O, O, COS, O],
      [O, I_SIN, O, O, O, O, O, COS]], "RYY6(1.23456)"),
    ("src/operator/atomic/ryy.rs:100-114", [g("RYY", 0b101, angle=ANGLE)], 3,
     [[COS, O, O, O, O, I_SIN, O, O],
      [O, COS, O, O, neg(I_SIN), O, O, O],
      [O, O, COS, O, O, O, O, I_SIN],
      [O, O, O, COS, O, O, neg(I_SIN), O],
      [O, neg(I_SIN), O, O, COS, O, O, O],
      [I_SIN, O, O, O, O, COS, O, O],
      [O, O, O, neg(I_SIN), O, O, COS, O],
      [O, O, I_SIN, O, O, O, O, COS]], "RYY5(1.23456)"),
    ("src/operator/atomic/rzz.rs:64-74", [g("RZZ", 0b11, angle=ANGLE)], 2,
     [[conj(EXP), O, O, O], [O, EXP, O, O], [O, O, EXP, O], [O, O, O, conj(EXP)]], "RZZ3(1.23456)"),
    ("src/operator/atomic/u1.rs:67-72", [g("U1", 0b1, matrix=flat([I, O, O, I]))], 1, [[I, O], [O, I]],
     "U1[[%s, %s], [%s, %s]]" % (dbg(I), dbg(O), dbg(O), dbg(I))),
    ("src/operator/atomic/u1.rs:80-91", [g("U1", 0b1, matrix=flat([S2, S2, S2, neg(S2)]))], 1,
     [[S2, S2], [S2, neg(S2)]],
     "U1[[%s, %s], [%s, %s]]" % (dbg(S2), dbg(S2), dbg(S2), dbg(neg(S2)))),
    ("src/operator/atomic/u2.rs:98-106",
     [g("U2", 0b01, 0b10, matrix=flat([I, O, O, O, O, I, O, O, O, O, I, O, O, O, O, I]))], 2,
     [[I, O, O, O], [O, I, O, O], [O, O, I, O], [O, O, O, I]],
     "U3[[%s, %s, %s, %s], [%s, %s, %s, %s], [%s, %s, %s, %s], [%s, %s, %s, %s]]"
     % tuple(dbg(z) for z in [I, O, O, O, O, I, O, O, O, O, I, O, O, O, O, I])),
    ("src/operator/atomic/u2.rs:114-134",
     [g("U2", 0b01, 0b10, matrix=flat([S2, S2, O, O, S2, neg(S2), O, O, O, O, neg(S2), neg(S2), O, O,
                                       neg(S2), S2]))], 2,
     [[S2, S2, O, O], [S2, neg(S2), O, O], [O, O, neg(S2), neg(S2)], [O, O, neg(S2), S2]],
     "U3[[%s, %s, %s, %s], [%s, %s, %s, %s], [%s, %s, %s, %s], [%s, %s, %s, %s]]"
     % tuple(dbg(z) for z in [S2, S2, O, O, S2, neg(S2), O, O, O, O, neg(S2), neg(S2), O, O, neg(S2), S2])),
    ("src/operator/atomic/h1.rs:55-57", [g("H1", 0b1)], 1, [[S2, S2], [S2, neg(S2)]], "H1"),
    ("src/operator/atomic/h2.rs:70-80", [g("H2", 0b01, 0b10)], 2,
     [[H5, H5, H5, H5], [H5, neg(H5), H5, neg(H5)], [H5, H5, neg(H5), neg(H5)], [H5, neg(H5), neg(H5), H5]],
     "H3"),
    ("src/operator/atomic/swap.rs:53-58", [g("SWAP", 0b11)], 2,
     [[I, O, O, O], [O, O, I, O], [O, I, O, O], [O, O, O, I]], "SWAP3"),
    ("src/operator/atomic/i_swap.rs:72-78", [g("ISWAP", 0b11, dgr=True)], 2,
     [[I, O, O, O], [O, O, neg(i_), O], [O, neg(i_), O, O], [O, O, O, I]], "iSWAP3"),
    ("src/operator/atomic/sqrt_swap.rs:72-82", [g("SQRT_SWAP", 0b11)], 2,
     [[I, O, O, O], [O, SQRT_I, conj(SQRT_I), O], [O, conj(SQRT_I), SQRT_I, O], [O, O, O, I]],
     "sqrt(SWAP3)"),
    ("src/operator/atomic/sqrt_i_swap.rs:72-82", [g("SQRT_ISWAP", 0b11)], 2,
     [[I, O, O, O], [O, (FRAC_1_SQRT_2 * 1.0, FRAC_1_SQRT_2 * 0.0), (FRAC_1_SQRT_2 * 0.0, FRAC_1_SQRT_2 * 1.0), O],
      [O, (FRAC_1_SQRT_2 * 0.0, FRAC_1_SQRT_2 * 1.0), (FRAC_1_SQRT_2 * 1.0, FRAC_1_SQRT_2 * 0.0), O],
      [O, O, O, I]], "sqrt(iSWAP3)"),
]

# Gates that qvnt's tests reject (`assert!(!op.is_valid())`).
invalid_cases = [
    ("src/operator/atomic/u1.rs:77-78", g("U1", 0b11, matrix=flat([I, O, O, I]))),
    ("src/operator/atomic/u2.rs:111-112", g("U2", 0b11, 0b10, matrix=flat([I, O, O, O, O, I, O, O, O, O, I, O, O, O, O, I]))),
]

# Non-unitary matrices that qvnt's tests reject through is_unitary (masks are fine).
non_unitary_cases = [
    ("src/operator/atomic/u1.rs:74-75", g("U1", 0b1, matrix=flat([I, I, O, I]))),
    ("src/operator/atomic/u2.rs:108-109", g("U2", 0b01, 0b10, matrix=flat([I, O, O, O, I, I, O, O, O, O, I, O, O, O, O, I]))),
]

register_cases = [
    {
        "cite": "src/register/quant.rs:642-677 (quantum_reg)",
        "q_num": 4,
        "state": 0b1100,
        # op::h(0b1111) * op::h(0b0011).c(0b1000).unwrap() * op::swap(0b1001).c(0b0010).unwrap()
        "program": [["h", 0b1111, 0], ["h", 0b0011, 0b1000], ["swap", 0b1001, 0b0010]],
        "names": "[H3, H12, C8_H3, C2_SWAP9]",
        "psi": [(0.25, 0.0), (0.25, 0.0), (0.25, 0.0), (0.0, 0.0), (-0.25, 0.0), (-0.25, 0.0), (-0.25, 0.0),
                (0.0, 0.0), (-0.5, 0.0), (0.0, 0.0), (0.25, 0.0), (0.0, 0.0), (0.5, 0.0), (0.0, 0.0),
                (-0.25, 0.0), (0.0, 0.0)],
        "measure_mask": 0b0110,
    },
]

tensor_cases = [
    {
        "cite": "src/register/quant.rs:679-711 (tensor)",
        "eps": 1e-9,
        # reg1 = with_state(2, 0b01).apply(h(0b01)); reg2 = with_state(1, 0b1).apply(h(0b01)); reg1 * reg2
        "a": {"q_num": 2, "state": 0b01, "h": 0b01},
        "b": {"q_num": 1, "state": 0b1, "h": 0b01},
        "prob": [0.25, 0.25, 0.0, 0.0, 0.25, 0.25, 0.0, 0.0],
    },
]

prob_cases = [
    {
        "cite": "src/register/quant.rs:701-710 (tensor, reg3)",
        "eps": 1e-9,
        "q_num": 3, "state": 0b101, "h": 0b101,
        "prob": [0.25, 0.25, 0.0, 0.0, 0.25, 0.25, 0.0, 0.0],
    },
]

name_cases = [
    {"cite": "src/operator/single/mod.rs:143-149", "gate": g("X", 123), "name": "X123",
     "c": 4, "c_name": "C4_X123"},
]

ctrl_cases = [
    {"cite": "src/operator/single/mod.rs:154-160", "gate": g("RYY", 0b101, angle=1.35),
     "reject": 0b001, "accept": 0b010},
]

multi_cases = [
    {"cite": "src/operator/multi/mod.rs:201-207",
     # op::id() * op::h(0b001).c(0b010) * op::x(0b011).c(0b100) * op::rz(5.0, 0b001) -> 3 ops
     "len": 3},
]

bits_iter_cases = [
    {"cite": "src/math/bits_iter.rs:36-48", "number": 0b10011001101010,
     "bits": [1 << 1, 1 << 3, 1 << 5, 1 << 6, 1 << 9, 1 << 10, 1 << 13]},
]

vreg_cases = [
    {"cite": "src/register/virtl.rs:166-180", "num": 8,
     "index": {"3": 0b00001000}, "even": 0b01010101, "odd": 0b10101010, "all": 0b11111111,
     "pick": [[0, 7], 0b10000001]},
    {"cite": "src/register/virtl.rs:183-218", "mask_cases": [
        [0b11111, {"0": 0b00001, "1": 0b00010, "2": 0b00100, "3": 0b01000, "4": 0b10000}, 0b11111],
        [0b01101, {"0": 0b00001, "1": 0b00100, "2": 0b01000}, 0b01101],
        [0b00111, {"0": 0b00001, "1": 0b00010, "2": 0b00100}, 0b00111],
        [0b11000, {"0": 0b01000, "1": 0b10000}, 0b11000]]},
]


def main():
    data = {
        "source": "qvnt 0.4.4 unit tests, restated by tests/golden/make_golden.py",
        "matrix_cases": [
            {"cite": c, "gates": gs, "size": sz, "matrix": [[list(z) for z in row] for row in m], "name": nm}
            for (c, gs, sz, m, nm) in matrix_cases
        ],
        "invalid_cases": [{"cite": c, "gate": gt} for (c, gt) in invalid_cases],
        "non_unitary_cases": [{"cite": c, "gate": gt} for (c, gt) in non_unitary_cases],
        "register_cases": [dict(rc, psi=[list(z) for z in rc["psi"]]) for rc in register_cases],
        "tensor_cases": tensor_cases,
        "prob_cases": prob_cases,
        "name_cases": name_cases,
        "ctrl_cases": ctrl_cases,
        "multi_cases": multi_cases,
        "bits_iter_cases": bits_iter_cases,
        "vreg_cases": vreg_cases,
    }
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_tests.json")
    with open(path, "w") as f:
        json.dump(data, f, separators=(",", ":"))
    print("wrote", path)


if __name__ == "__main__":
    main()
