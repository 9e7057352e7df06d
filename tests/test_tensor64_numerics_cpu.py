"""The TENSOR64 pass arithmetic restated on the CPU (test infrastructure, no GPU): the digit split of
the block-floating-point state and of round(W 2^55), the eight levels of digit-pair products, and the
read-back that forms X' = sum_l L_l 2^(41 - 8 l) from 32-bit words (magic-number bits for levels 0-3,
exact integers for 4-5, levels 6-7 summed in FP32 and rounded), as qvnt_gb300/csrc/tensor64.cu does.

Checks: every level is an integer below 2^23 (exact FP32 accumulation), levels 0-3 below 2^22 (the
magic-number conversion), and X' within 0.54 of the exact Y / 2^55, for Haar-random and permutation
blocks and for random and all-extreme state rows.
"""
import numpy as np

BIAS = 0x80808080808080
MAGIC = 0x4B400000
MASK64 = (1 << 64) - 1


def state_digits(X):
    """Digits of X + bias, byte 6 (most significant) first, minus 128: balanced, |d| <= 128."""
    out = np.zeros((7, len(X)), dtype=np.int64)
    for i, v in enumerate(X):
        y = (int(v) + BIAS) & MASK64
        for s in range(7):
            out[s, i] = ((y >> (8 * (6 - s))) & 0xFF) - 128
    return out


def weight_digits(W):
    """Balanced base-256 digits of the integers W, most significant first (the host's split)."""
    out = np.zeros((7, len(W)), dtype=np.int64)
    for i, v in enumerate(W):
        rest = int(v)
        for t in range(6, 0, -1):
            d = ((rest + 128) % 256) - 128
            out[t, i] = d
            rest = (rest - d) // 256
        out[0, i] = rest
    return out


def f32(x):
    return np.float32(x)


def readback(L):
    """The kernel's combine of the eight levels into X' (64-bit two's complement)."""
    assert all(abs(L[l]) < 2 ** 22 for l in range(4)), L
    m = [(L[l] + MAGIC) & 0xFFFFFFFF for l in range(4)]  # bits of f + 1.5 * 2^23
    vm = (m[0] * 256 + m[1]) & 0xFFFFFFFF
    um = (m[2] * 256 + m[3]) & 0xFFFFFFFF

    def i32(x):
        x &= 0xFFFFFFFF
        return x - (1 << 32) if x >= (1 << 31) else x

    V, U = i32(vm - 257 * MAGIC), i32(um - 257 * MAGIC)
    acc = (((2 * V) & 0xFFFFFFFF) << 32) + ((U << 17) & MASK64)
    acc = (acc + ((L[4] << 9) & MASK64) + ((L[5] << 1) & MASK64)) & MASK64
    # fmaf(L6, 2^-7, L7 * 2^-15): one rounding of the exact value (exact in f64 at these sizes)
    t = np.float32(float(L[6]) * 2.0 ** -7 + float(f32(L[7]) * f32(2.0 ** -15)))
    q = int(np.float32(t + np.float32(12582912.0))) - 12582912
    acc = (acc + (q & MASK64)) & MASK64
    return acc - (1 << 64) if acc >= (1 << 63) else acc


def unitary(rng, kind):
    if kind == "perm":
        return np.eye(32)[rng.permutation(32)].astype(complex)
    A = rng.normal(size=(32, 32)) + 1j * rng.normal(size=(32, 32))
    Q, R = np.linalg.qr(A)
    return Q * (np.diag(R) / np.abs(np.diag(R)))


def test_levels_exact_and_readback_within_bound():
    rng = np.random.default_rng(7)
    worst = 0.0
    for trial in range(12):
        U = unitary(rng, "perm" if trial % 3 == 0 else "haar")
        W = np.zeros((64, 64))
        W[0::2, 0::2], W[0::2, 1::2] = U.real, -U.imag
        W[1::2, 0::2], W[1::2, 1::2] = U.imag, U.real
        Wi = [[int(np.rint(np.ldexp(w, 55))) for w in row] for row in W]
        wd = [weight_digits(Wi[n]) for n in range(64)]
        top = 2 ** 54
        if trial % 4 == 1:
            X = [top * (1 if rng.random() < 0.5 else -1) for _ in range(64)]
        else:
            X = [int(v) for v in rng.integers(-top, top, 64, dtype=np.int64)]
        xd = state_digits(X)
        assert np.all(np.abs(xd) <= 128)
        for n in range(0, 64, 3):
            assert np.all(np.abs(wd[n]) <= 128)
            L = [0] * 8
            for s in range(7):
                for t in range(7):
                    if s + t <= 7:
                        L[s + t] += int(np.dot(xd[s], wd[n][t]))
            assert all(abs(v) < 2 ** 23 for v in L), L
            exact = sum(X[k] * Wi[n][k] for k in range(64))
            got = readback(L)
            worst = max(worst, abs(got * 2 ** 55 - exact) / 2 ** 55)
    assert worst <= 0.54, worst
