// Shared device/host helpers of the GB300 state-vector engine.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/qvnt_gb300.h"

namespace qvnt {

// One amplitude: Complex<f64>, interleaved (re, im), 16 bytes (num-complex layout).
using amp_t = double2;

// Device-side gate descriptor: the host decodes a qvnt_gate into this once per apply call.
// Masks are in the register's index space; `pivot` is the bit inserted as 0 to enumerate orbits.
struct DevGate {
    uint32_t kind;
    uint32_t dagger;
    uint64_t a;      // a_mask / ab_mask
    uint64_t b;      // H2/U2 b_mask
    uint64_t ctrl;   // control mask
    uint64_t y_ipow; // Y: the stored i power (y.rs:10-13)
    double ph_re, ph_im;
    double m[32];
};

// Enumeration of gate orbits: `nins` zero bits inserted at ascending positions `ins[]`, then the
// control bits OR-ed in.  Orbit base index of enumeration counter j.
struct Enum {
    uint32_t nins;
    uint32_t ins[40];
    uint64_t ones;    // bits forced to 1 (controls)
    uint64_t count;   // number of orbits
};

__host__ __device__ inline uint64_t insert_zero_bit(uint64_t j, uint32_t p) {
    uint64_t low = j & ((1ull << p) - 1ull);
    return ((j >> p) << (p + 1)) | low;
}

__host__ __device__ inline uint64_t enum_index(const Enum& e, uint64_t j) {
    for (uint32_t k = 0; k < e.nins; ++k) j = insert_zero_bit(j, e.ins[k]);
    return j | e.ones;
}

__host__ __device__ __forceinline__ unsigned popc64(uint64_t x) {
#ifdef __CUDA_ARCH__
    return (unsigned)__popcll(x);
#else
    return (unsigned)__builtin_popcountll(x);
#endif
}

// Launch geometry: grid sized in multiples of the SM count (152 on GB300).
struct Geometry {
    int sms = 152;
    int blocks_per_sm = 8;
};

}  // namespace qvnt

#define QVNT_CUDA_TRY(expr)                                                   \
    do {                                                                      \
        cudaError_t _e = (expr);                                              \
        if (_e != cudaSuccess) return ::qvnt::set_cuda_error(_e, #expr);      \
    } while (0)

namespace qvnt {
int set_error(int status, const char* fmt, ...);
int set_cuda_error(cudaError_t e, const char* what);
}  // namespace qvnt
