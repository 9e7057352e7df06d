// Double-float ("df64") arithmetic and the two amplitude storage formats.
//
// GB300 issues FP32 FMA at ~114 per clock per SM but FP64 at ~1.6 (measured), so the fused engine
// keeps each f64 amplitude component as an unevaluated sum hi + lo of two floats (|lo| <= ulp(hi)/2,
// a 48-bit significand) and computes with error-free transformations on the FP32 pipes:
//   two_sum      s + e == a + b exactly                     (Knuth)
//   fast_two_sum s + e == a + b exactly when |a| >= |b|      (Dekker)
//   two_prod     p + e == a * b exactly, e = fma(a, b, -p)
// Relative error per operation is ~2^-47; amplitudes of a unit-norm state never leave the float
// exponent range except below 1e-38, where the absolute error is below 1e-38.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace qvnt {

struct df {
    float h, l;
};

// One df64 amplitude: 16 bytes, (re.h, re.l, im.h, im.l).
struct dfc {
    df re, im;
};

__device__ __forceinline__ df df_make(float h, float l) { return df{h, l}; }

__device__ __forceinline__ df two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return df{s, e};
}

__device__ __forceinline__ df fast_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return df{s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ df df_neg(df a) { return df{-a.h, -a.l}; }

__device__ __forceinline__ df df_add(df a, df b) {
    df s = two_sum(a.h, b.h);
    const float e = __fadd_rn(s.l, __fadd_rn(a.l, b.l));
    return fast_two_sum(s.h, e);
}

__device__ __forceinline__ df df_sub(df a, df b) { return df_add(a, df_neg(b)); }

// c * x for a df constant c, unnormalised: hi + lo == c*x up to ~2^-48 relative.
__device__ __forceinline__ df df_mul_raw(df c, df x) {
    const float p = __fmul_rn(c.h, x.h);
    float e = __fmaf_rn(c.h, x.h, -p);
    e = __fmaf_rn(c.h, x.l, e);
    e = __fmaf_rn(c.l, x.h, e);
    return df{p, e};
}

__device__ __forceinline__ df df_mul(df c, df x) {
    const df r = df_mul_raw(c, x);
    return fast_two_sum(r.h, r.l);
}

// Sum of N unnormalised terms: hi parts through a two_sum chain, all error parts summed in float.
// The result is left UNNORMALISED (hi = the rounded sum of the hi parts, lo = everything else): the
// gate kernels renormalise once per register stage (df_renorm) instead of after every gate.  Until
// then |lo| stays within a few ulp(hi) of the inputs' magnitude, so the absolute error of every
// later error-free product stays at ~2^-48 of the amplitudes involved.
template <int N>
__device__ __forceinline__ df df_sum_raw(const df (&t)[N]) {
    float s = t[0].h;
    float e = t[0].l;
#pragma unroll
    for (int k = 1; k < N; ++k) {
        const df q = two_sum(s, t[k].h);
        s = q.h;
        e = __fadd_rn(e, __fadd_rn(q.l, t[k].l));
    }
    return df{s, e};
}

template <int N>
__device__ __forceinline__ df df_sum(const df (&t)[N]) {
    const df r = df_sum_raw<N>(t);
    return fast_two_sum(r.h, r.l);
}

// Renormalisation of an unnormalised pair (no magnitude assumption).
__device__ __forceinline__ df df_renorm(df a) { return two_sum(a.h, a.l); }

// c0*x0 + c1*x1 (real df constants, df values), unnormalised.
__device__ __forceinline__ df df_lin2(df c0, df x0, df c1, df x1) {
    const df t[2] = {df_mul_raw(c0, x0), df_mul_raw(c1, x1)};
    return df_sum_raw<2>(t);
}

// c0*x0 + c1*x1 + c2*x2 + c3*x3, unnormalised.
__device__ __forceinline__ df df_lin4(df c0, df x0, df c1, df x1, df c2, df x2, df c3, df x3) {
    const df t[4] = {df_mul_raw(c0, x0), df_mul_raw(c1, x1), df_mul_raw(c2, x2), df_mul_raw(c3, x3)};
    return df_sum_raw<4>(t);
}

// x0 + x1 and x0 - x1 (the unscaled Hadamard butterfly), unnormalised.
__device__ __forceinline__ df df_add_raw(df a, df b) {
    const df s = two_sum(a.h, b.h);
    return df{s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l))};
}
__device__ __forceinline__ df df_sub_raw(df a, df b) {
    const df s = two_sum(a.h, -b.h);
    return df{s.h, __fadd_rn(s.l, __fsub_rn(a.l, b.l))};
}

// Complex multiply by a df complex constant: (cr + i ci) * (xr + i xi).
__device__ __forceinline__ dfc dfc_mul(df cr, df ci, dfc x) {
    dfc r;
    r.re = df_lin2(cr, x.re, df_neg(ci), x.im);
    r.im = df_lin2(cr, x.im, ci, x.re);
    return r;
}

// z * i^q, exact.
__device__ __forceinline__ dfc dfc_rotate(dfc z, uint32_t q) {
    if (q & 2) {
        z.re = df_neg(z.re);
        z.im = df_neg(z.im);
    }
    if (q & 1) {
        const df t = df_neg(z.im);
        z.im = z.re;
        z.re = t;
    }
    return z;
}

// ---- conversions (only at API boundaries and in register-wide passes) -----------------------------
// On the device the float <-> double conversions are done on the bit patterns with integer
// instructions: GB300 converts between the two formats far more slowly than it issues integer ops.
// Results are those of the IEEE conversions (round to nearest even); zeros, subnormals, overflow,
// infinities and NaNs take the hardware conversion.
__device__ __forceinline__ float d2f_rn_bits(double x) {
    const uint64_t u = (uint64_t)__double_as_longlong(x);
    const uint32_t sign = (uint32_t)(u >> 32) & 0x80000000u;
    const int fe = (int)((u >> 52) & 0x7ffu) - 1023 + 127;
    if (fe <= 0 || fe >= 255) return __double2float_rn(x);
    const uint32_t top = (uint32_t)((u >> 29) & 0x7fffffu);  // 23 mantissa bits kept
    const uint32_t rest = (uint32_t)(u & 0x1fffffffu);       // 29 bits dropped
    uint32_t bits = ((uint32_t)fe << 23) | top;
    if (rest > 0x10000000u || (rest == 0x10000000u && (top & 1u))) bits += 1u;  // a carry bumps the exponent
    return __uint_as_float(sign | bits);
}

__device__ __forceinline__ double f2d_bits(float f) {
    const uint32_t b = __float_as_uint(f);
    const uint32_t e = (b >> 23) & 0xffu;
    if (e == 0u || e == 255u) return (double)f;
    const uint64_t u = ((uint64_t)(b & 0x80000000u) << 32) | ((uint64_t)(e - 127u + 1023u) << 52) |
                       ((uint64_t)(b & 0x7fffffu) << 29);
    return __longlong_as_double((long long)u);
}

__host__ __device__ __forceinline__ df df_from_double(double x) {
#ifdef __CUDA_ARCH__
    const float h = d2f_rn_bits(x);
    return df{h, d2f_rn_bits(x - f2d_bits(h))};
#else
    const float h = (float)x;
    const float l = (float)(x - (double)h);
    return df{h, l};
#endif
}

__host__ __device__ __forceinline__ double df_to_double(df a) {
#ifdef __CUDA_ARCH__
    return f2d_bits(a.h) + f2d_bits(a.l);
#else
    return (double)a.h + (double)a.l;
#endif
}

// ---- amplitude accessors: register-wide kernels are written once for every storage format ------
// Storage is 16 bytes per amplitude for F64 and DF64, 8 bytes (complex<f32>) for C32; the pointer
// is passed as double2* and each accessor indexes its own element size.
struct AccF64 {
    static __device__ __forceinline__ double2 load(const double2* p, uint64_t i) { return p[i]; }
    static __device__ __forceinline__ void store(double2* p, uint64_t i, double2 v) { p[i] = v; }
};

struct AccDF64 {
    static __device__ __forceinline__ double2 load(const double2* p, uint64_t i) {
        const float4 v = reinterpret_cast<const float4*>(p)[i];
        return make_double2(df_to_double(df{v.x, v.y}), df_to_double(df{v.z, v.w}));
    }
    static __device__ __forceinline__ void store(double2* p, uint64_t i, double2 v) {
        const df r = df_from_double(v.x), m = df_from_double(v.y);
        reinterpret_cast<float4*>(p)[i] = make_float4(r.h, r.l, m.h, m.l);
    }
};

struct AccC32 {
    static __device__ __forceinline__ double2 load(const double2* p, uint64_t i) {
        const float2 v = reinterpret_cast<const float2*>(p)[i];
        return make_double2((double)v.x, (double)v.y);
    }
    static __device__ __forceinline__ void store(double2* p, uint64_t i, double2 v) {
        reinterpret_cast<float2*>(p)[i] = make_float2((float)v.x, (float)v.y);
    }
};

}  // namespace qvnt
