// The 20 atomic gate functions of qvnt, as device code.
//
// Callable from host code too (the precision engine builds dense gate matrices with it).
// `atomic_op(g, idx, psi)` returns qvnt's `AtomicOp::atomic_op(psi, idx)` for the gate kind, where
// `psi(j)` yields the input amplitude at index j.  Operand order and association follow each
// reference file line by line; translation units that include this header are compiled with
// --fmad=false so that every product and sum rounds separately, as in qvnt's release build.
#pragma once

#include "common.cuh"

namespace qvnt {

__host__ __device__ __forceinline__ amp_t c_add(amp_t a, amp_t b) { return make_double2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ amp_t c_neg(amp_t a) { return make_double2(-a.x, -a.y); }
// num-complex Mul: re = a.re*b.re - a.im*b.im, im = a.re*b.im + a.im*b.re
__host__ __device__ __forceinline__ amp_t c_mul(amp_t a, amp_t b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ __forceinline__ amp_t c_scale(amp_t a, double t) { return make_double2(a.x * t, a.y * t); }

// `rotate(z, q)`: z * i^q (src/math/mod.rs:40-50).
__host__ __device__ __forceinline__ amp_t rotate(amp_t z, uint64_t q) {
    if (q & 2) z = c_neg(z);
    if (q & 1) z = make_double2(-z.y, z.x);
    return z;
}

constexpr double kFrac1Sqrt2 = 0.70710678118654752440084436210484903;

__host__ __device__ __forceinline__ amp_t gate_m(const DevGate& g, int k) { return make_double2(g.m[2 * k], g.m[2 * k + 1]); }

template <class Psi>
__host__ __device__ __forceinline__ amp_t atomic_op(const DevGate& g, uint64_t idx, Psi&& psi) {
    const uint64_t a = g.a;
    switch (g.kind) {
    case QVNT_GATE_X:  // x.rs:15-17
        return psi(idx ^ a);
    case QVNT_GATE_Y: {  // y.rs:17-23
        uint64_t i_pow = g.y_ipow;
        if ((popc64(idx & a) & 1u) == 0) i_pow ^= 2;
        return rotate(psi(idx ^ a), i_pow);
    }
    case QVNT_GATE_Z:  // z.rs:15-21
        return (popc64(idx & a) & 1u) ? c_neg(psi(idx)) : psi(idx);
    case QVNT_GATE_S: {  // s.rs:19-25
        uint64_t count = popc64(idx & a);
        if (g.dagger) count = (~count) + 1ull;
        return rotate(psi(idx), count);
    }
    case QVNT_GATE_T: {  // t.rs:24-35
        uint64_t count = popc64(idx & a);
        if (g.dagger) count = (~count) + 1ull;
        amp_t p = rotate(psi(idx), count >> 1);
        return (count & 1ull) ? c_mul(make_double2(kFrac1Sqrt2, kFrac1Sqrt2), p) : p;
    }
    case QVNT_GATE_RX:     // rx.rs:18-24
    case QVNT_GATE_RXX: {  // rxx.rs:19-25
        amp_t p0 = psi(idx), p1 = psi(idx ^ a);
        return make_double2(p0.x * g.ph_re + p1.y * g.ph_im, p0.y * g.ph_re - p1.x * g.ph_im);
    }
    case QVNT_GATE_RY: {  // ry.rs:19-29
        double pr = g.ph_re, pi = g.ph_im;
        amp_t p0 = psi(idx), p1 = psi(idx ^ a);
        if ((idx & a) == 0) pi = -pi;
        return make_double2(p0.x * pr + p1.x * pi, p0.y * pr + p1.y * pi);
    }
    case QVNT_GATE_RYY: {  // ryy.rs:19-29
        double pr = g.ph_re, pi = g.ph_im;
        amp_t p0 = psi(idx), p1 = psi(idx ^ a);
        if ((popc64(idx & a) & 1u) == 0) pi = -pi;
        return make_double2(p0.x * pr + p1.y * pi, p0.y * pr - p1.x * pi);
    }
    case QVNT_GATE_RZ: {  // rz.rs:19-25
        amp_t ph = make_double2(g.ph_re, g.ph_im);
        if ((idx & a) == 0) ph.y = -ph.y;
        return c_mul(ph, psi(idx));
    }
    case QVNT_GATE_RZZ: {  // rzz.rs:19-25
        amp_t ph = make_double2(g.ph_re, g.ph_im);
        if ((popc64(idx & a) & 1u) == 0) ph.y = -ph.y;
        return c_mul(ph, psi(idx));
    }
    case QVNT_GATE_U1: {  // u1.rs:17-25
        const bool a_bit = (idx & a) != 0;
        const uint64_t i = idx & ~a;
        const int r = a_bit ? 2 : 0;
        return c_add(c_mul(gate_m(g, r), psi(i)), c_mul(gate_m(g, r + 1), psi(i | a)));
    }
    case QVNT_GATE_U2: {  // u2.rs:22-49
        const uint64_t b = g.b;
        const int row = (((idx & b) != 0) << 1) | ((idx & a) != 0);
        const uint64_t i = idx & ~a & ~b;
        amp_t s = c_mul(gate_m(g, 4 * row + 0), psi(i));
        s = c_add(s, c_mul(gate_m(g, 4 * row + 1), psi(i | a)));
        s = c_add(s, c_mul(gate_m(g, 4 * row + 2), psi(i | b)));
        s = c_add(s, c_mul(gate_m(g, 4 * row + 3), psi(i | a | b)));
        return s;
    }
    case QVNT_GATE_H1: {  // h1.rs:16-22
        amp_t p0 = psi(idx), p1 = psi(idx ^ a);
        if (idx & a) p0 = c_neg(p0);
        return c_scale(c_add(p0, p1), kFrac1Sqrt2);
    }
    case QVNT_GATE_H2: {  // h2.rs:22-38
        const uint64_t b = g.b;
        amp_t p0 = psi(idx), p1 = psi(idx ^ a), p2 = psi(idx ^ b), p3 = psi(idx ^ (a | b));
        if (idx & a) {
            p0 = c_neg(p0);
            p2 = c_neg(p2);
        }
        if (idx & b) {
            p0 = c_neg(p0);
            p1 = c_neg(p1);
        }
        return c_scale(c_add(c_add(c_add(p0, p1), p2), p3), 0.5);
    }
    case QVNT_GATE_SWAP:  // swap.rs:16-22
        return (popc64(idx & a) & 1u) ? psi(idx ^ a) : psi(idx);
    case QVNT_GATE_ISWAP: {  // i_swap.rs:20-37
        if (popc64(idx & a) & 1u) {
            amp_t p = psi(idx ^ a);
            return g.dagger ? make_double2(p.y, -p.x) : make_double2(-p.y, p.x);
        }
        return psi(idx);
    }
    case QVNT_GATE_SQRT_SWAP: {  // sqrt_swap.rs:20-37
        if (popc64(idx & a) & 1u) {
            amp_t p0 = psi(idx), p1 = psi(idx ^ a);
            if (g.dagger)
                return make_double2(0.5 * (p0.x + p0.y + p1.x - p1.y), 0.5 * (p0.y - p0.x + p1.y + p1.x));
            return make_double2(0.5 * (p0.x - p0.y + p1.x + p1.y), 0.5 * (p0.y + p0.x + p1.y - p1.x));
        }
        return psi(idx);
    }
    case QVNT_GATE_SQRT_ISWAP: {  // sqrt_i_swap.rs:20-37
        if (popc64(idx & a) & 1u) {
            amp_t p0 = psi(idx), p1 = psi(idx ^ a);
            if (g.dagger) return make_double2(kFrac1Sqrt2 * (p0.x + p1.y), kFrac1Sqrt2 * (p0.y - p1.x));
            return make_double2(kFrac1Sqrt2 * (p0.x - p1.y), kFrac1Sqrt2 * (p0.y + p1.x));
        }
        return psi(idx);
    }
    default:  // QVNT_GATE_ID, id.rs:7-9
        return psi(idx);
    }
}

}  // namespace qvnt
