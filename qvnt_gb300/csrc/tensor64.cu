// Tensor-core f64 engine: IEEE f64 amplitudes in HBM (qvnt's Complex<f64> layout, the PLAIN
// format) at every call boundary, runs of gates fused into dense 5-qubit blocks (32 x 32 complex
// unitaries, the planner of dense_blocks.h) and contracted on the tcgen05 tensor cores with 54-bit
// operands by exact integer slicing (the Ozaki splitting of a matrix product into exactly
// representable digit products).
//
// Number format between the passes of one apply call: 64-bit block floating point.  Every real
// component is an int64 X with one scale 2^-S for the whole register (x = X 2^-S); before a pass
// reads it, the register is renormalised (a uniform shift) so that its largest |X| is 2^53 .. 2^54.
// A pass therefore rounds every component to 2^-54 .. 2^-55 of the register's largest component,
// finer than IEEE f64 rounds the largest amplitudes.  The first pass of a call reads IEEE f64 (sliced
// against the register's largest exponent, found by a reduction kernel first) and the last one
// writes IEEE f64, so only the passes in between see the integer format.
//
// Arithmetic of a pass.  The block matrix in its real 64 x 64 form W (row = output component,
// column = input component) is held as round(W 2^55), |.| <= 2^55; it and the state are split into
// seven balanced base-256 digits (|digit| <= 128), exact in fp16.  The product is the sum over digit
// pairs (s, t) of A_s B_t^T weighted by 2^(96 - 8 (s + t)); the 34 pairs with s + t <= 7 are issued as
// tcgen05.mma kind::f16 (M = 128 rows, K = 16) into eight FP32 accumulators in tensor memory, one per
// level l = s + t: the pairs of one digit s into adjacent levels are one MMA of N = 64 m, m <= 4, so a
// K step takes 11 MMAs instead of 34 (an MMA of N = 64 costs 97 cycles, one of N = 256 128).  Every
// partial sum is an integer below 2^23 in magnitude (at most 7 products of 64 terms of |digit product|
// <= 2^14, those with a top digit smaller), so the FP32 accumulation is exact.  Levels >= 8 are
// dropped (2^-23 of an output unit per level-8 unit: typically 0.01 unit).  The accumulators are read
// back (tcgen05.ld): levels 0-3 as integers by a magic-number add (below 2^22), levels 4-5 by an exact
// float-to-int conversion, and L6 2^-7 + L7 2^-15 summed in FP32; they combine into the output
// X' = sum_l L_l 2^(41 - 8 l) with one rounding (of the levels 6 and 7 part, to within 1/2 + 2^-9 of
// a unit).  No FP64 instruction is issued.
//
// Kernel (one pass = one block): persistent CTAs, one per SM (tensor memory: all 512 columns), of
// 18 warps (10 in the 16-amplitude layout) in three roles synchronised by mbarriers only.  Per tile of
// 4096 amplitudes (12 tile qubits: the 7 lowest, so a tile is 2 KB runs, plus the block's):
//   * the copy warp keeps two shared-memory tile buffers filled with TMA bulk loads and stores each
//     tile once its results are written (into the other buffer, whose tile was sliced just before:
//     a buffer is reloaded more than a tile ahead of its use);
//   * 16 math warps each take one operand row (lane quadrant) and 8 of its 32 amplitudes (or 8 warps
//     and 16 amplitudes): the digits, stored one by one to two ping-pong operand slots in tensor
//     memory (a slot takes digit s once the MMAs of digit s - 2 are done); then the read-back of the
//     eight levels and the output;
//   * the MMA warp issues each digit's products once its slot is full and commits them to the
//     slot's mbarrier.
// Level l is final once digit l's products are done; level 0 sits in level 7's columns, which the
// math warps clear right after reading level 0.  The next tile is read once this tile's levels
// are, and this tile's results are written while the next tile's first digits multiply.
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "dense_blocks.h"
#include "engine.h"
#include "kernels.h"
#include "tc_ptx.cuh"

#define TRY_T(expr)             \
    do {                        \
        const int _s = (expr);  \
        if (_s) return _s;      \
    } while (0)

namespace qvnt {

namespace {

using namespace tc;

constexpr int kTQ = 12;                         // tile qubits
constexpr uint32_t kTileAmps = 1u << kTQ;       // 4096 amplitudes, 64 KB
constexpr uint32_t kLowQ = 7;                   // lowest qubits always in the tile (2 KB runs)
// Block layout for NA amplitudes per math thread (8 or 16): 4 lane quadrants x 32 / NA column
// groups of math warps, then the MMA warp and the copy warp.
template <int NA>
struct Layout {
    static constexpr uint32_t kCG = 32 / NA;             // column groups per row
    static constexpr uint32_t kMathWarps = 4 * kCG;
    static constexpr uint32_t kMmaWarp = kMathWarps;     // issues the MMAs
    static constexpr uint32_t kTmaWarp = kMathWarps + 1; // issues the tile copies
    static constexpr uint32_t kNT = 32 * (kMathWarps + 2);
};
constexpr int kDigits = 7;                      // base-256 digits per operand
constexpr int kWScale = 55;                     // block matrices are held as round(W 2^55)
constexpr int kTopBits = 54;                    // fixed-point inputs are renormalised to |X| <= 2^54
constexpr uint32_t kWDigitBytes = 64 * 64 * 2;  // one fp16 digit matrix of a block (8 KB)
constexpr uint32_t kWBlockBytes = kDigits * kWDigitBytes;
constexpr uint32_t kWaitLimit = 1u << 22;       // mbarrier polls before a wait gives up
constexpr uint32_t kSlotCol = 448;              // tensor-memory columns of the two operand slots (448, 480)
// Tensor-memory column of level l's accumulator: levels 1..7 side by side from column 0 (so that the
// pairs of one digit s >= 1, levels s .. 7, are adjacent), level 0 in level 7's columns (level 0 is
// read back and its columns cleared before the first level-7 product).
__host__ __device__ constexpr uint32_t level_col(int l) { return l == 0 ? 384u : 64u * (uint32_t)(l - 1); }
constexpr uint64_t kBias = 0x80808080808080ull; // 128 in each of the 7 digit bytes
constexpr uint32_t kMagic = 0x4B400000u;        // bits of 1.5 * 2^23
// shared memory: two tile buffers, the block's 7 digit matrices and a copy of digit 0 after digit 6
// (so that the pairs (0, 5), (0, 6), (0, 0) into levels 5, 6, 0 are one operand)
constexpr size_t kSmemDyn = 2 * (size_t)kTileAmps * 16 + kWBlockBytes + kWDigitBytes;

// Instruction descriptor of kind::f16: FP32 accumulator, A and B fp16 and K-major, M = 128, N = 64 m
// (m levels side by side: m digit matrices of a block, stacked 8 KB apart, are one operand of 64 m
// rows in the shared-memory layout below).
__host__ __device__ constexpr uint32_t idesc16(uint32_t m) {
    return (1u << 4) | (((64u * m) >> 3) << 17) | ((128u >> 4) << 24);
}

// fp16 element offset of B[row][k] (row = output real, k = input real) in the no-swizzle K-major
// operand layout: core matrices of 8 rows x 16 bytes; adjacent along K 128 B apart, 8-row groups
// 1024 B apart.
__host__ __device__ constexpr uint32_t w_off16(uint32_t row, uint32_t k) {
    return (row >> 3) * 512u + (k >> 3) * 64u + (row & 7u) * 8u + (k & 7u);
}

// Register scale of one pass, in a ring of three per register (pass p reads slot p mod 3, writes the
// next slot, and clears the one after it for pass p + 1).  mag: before the first pass of a call, the
// largest biased f64 exponent of the state; after a fixed-point pass, the OR of its outputs' high
// words in sign-magnitude-like form (x ^ (x >> 31)), whose bit length is that of the largest output.
// S: the scale exponent (x = X 2^-S) of the outputs of the pass that wrote the slot.
struct ScaleSlot {
    uint32_t mag;
    int32_t S;
};

struct TPassParams {
    uint64_t ntiles;
    uint64_t w_off;      // byte offset of the block's weights in the weight buffer
    ScaleSlot* slots;    // the register's scale ring
    uint32_t cur;        // slot this pass reads
    uint32_t c;          // tile qubits 0 .. c-1 are the register's lowest: runs of 2^c amplitudes
    uint32_t tq[kTQ];    // tile qubits, ascending
    uint8_t bits[dense::kBQ];  // tile-local bit of block bit j
};

__device__ __forceinline__ void mma_f16_ta(uint32_t d_tmem, uint32_t a_tmem, uint64_t b, uint32_t idesc,
                                           uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}" ::"r"(d_tmem),
        "r"(a_tmem), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

// Fixed point of an IEEE f64 x against the register's largest exponent E (biased, >= x's):
// X = round(x 2^(1075 - E)), |X| < 2^53; returns Y = X + kBias, whose byte j minus 128 is the
// balanced digit j of X.  Zeros and f64 subnormals give X = 0.
__device__ __forceinline__ uint64_t slice(double x, uint32_t E) {
    const uint64_t b = (uint64_t)__double_as_longlong(x);
    const uint32_t e = (uint32_t)(b >> 52) & 0x7ffu;
    uint64_t v = 0;
    if (e != 0) {
        const uint64_t m = (b & 0xfffffffffffffull) | (1ull << 52);
        const uint32_t sh = E - e;
        v = sh == 0 ? m : sh < 54 ? (m + (1ull << (sh - 1))) >> sh : 0ull;
    }
    return ((b >> 63) ? (0ull - v) : v) + kBias;
}

// A fixed-point component renormalised by 2^sigma (a left shift, or a right shift rounding half up)
// and biased for the digit split.
__device__ __forceinline__ uint64_t renorm(long long X, int sigma) {
    if (sigma > 0) X = (long long)((unsigned long long)X << sigma);
    else if (sigma < 0) X = (X + (1ll << (-sigma - 1))) >> (-sigma);
    return (uint64_t)X + kBias;
}

// Digit byte `byte` of two reals as a packed fp16 pair: fp16(1024 + c) has the bits 0x6400 + c for
// a byte c, and subtracting 1152 leaves c - 128 exactly.
__device__ __forceinline__ uint32_t digit_pair(uint64_t y0, uint64_t y1, int byte) {
    const uint32_t w0 = byte < 4 ? (uint32_t)y0 : (uint32_t)(y0 >> 32);
    const uint32_t w1 = byte < 4 ? (uint32_t)y1 : (uint32_t)(y1 >> 32);
    const uint32_t j = (uint32_t)(byte & 3);
    uint32_t h = (__byte_perm(w0, w1, j | (j << 4) | ((4u + j) << 8) | ((4u + j) << 12)) & 0x00ff00ffu) | 0x64006400u;
    __half2 v = *reinterpret_cast<__half2*>(&h);
    v = __hsub2(v, __halves2half2(__ushort_as_half((unsigned short)0x6480), __ushort_as_half((unsigned short)0x6480)));
    return *reinterpret_cast<uint32_t*>(&v);
}

// An integer-valued float f, |f| < 2^22, as the bits of f + 1.5 * 2^23: the integer plus kMagic.
__device__ __forceinline__ uint32_t mbits(float f) { return __float_as_uint(f + 12582912.0f); }

// v * 2^T rounded to the nearest f64 (ties to even); below the normal range: signed zero.
__device__ __forceinline__ double scaled_to_f64(int64_t v, int T) {
    const uint64_t sgn = (uint64_t)v & 0x8000000000000000ull;
    const uint64_t a = (uint64_t)((v ^ (v >> 63)) - (v >> 63));  // |v|
    if (a == 0) return 0.0;
    const int lz = __clzll((long long)a);
    const uint64_t n = a << lz;                        // leading one at bit 63
    uint64_t mant = n >> 11;                           // 53 bits
    const uint32_t low = (uint32_t)n & 0x7ffu;         // round bit 10, sticky bits 0..9
    mant += (low >> 10) & ((low & 0x3ffu) != 0u | (uint32_t)mant) & 1u;
    const int e = 1086 - lz + T;                       // biased exponent of a * 2^T
    if (e <= 0) return __longlong_as_double((long long)sgn);
    return __longlong_as_double((long long)(sgn | (((uint64_t)(e - 1) << 52) + mant)));
}

// A wait that sleeps in hardware until the phase completes, in slices of kSleepNs; it gives up
// after kSleepSlices slices (about two seconds; setting the error flag and the block's abort flag)
// or as soon as another role has aborted.
constexpr uint32_t kSleepNs = 1000000;
constexpr uint32_t kSleepSlices = 2000;
__device__ __forceinline__ bool wait_or_abort(uint64_t* bar, uint32_t parity, volatile int* abort_flag,
                                              int* err) {
    for (uint32_t it = 0; it < kSleepSlices; ++it) {
        if (mbar_try_sleep(bar, parity, kSleepNs)) return true;
        if (*abort_flag) return false;
    }
    atomicExch(err, 1);
    *abort_flag = 1;
    return false;
}

// Digit S (0 = most significant) of the thread's 2 NA reals into an operand slot, then one arrival
// per warp on the slot's "full" barrier.
// Digits 0 and 1 of the thread's 2 NA reals into the two slots, with one wait for both stores.
template <int NA>
__device__ __forceinline__ void put_digits01(const uint64_t (&y)[2 * NA], uint32_t slot_addr, uint64_t* full,
                                             uint32_t lane) {
    uint32_t v0[NA], v1[NA];
#pragma unroll
    for (int i = 0; i < NA; ++i) {
        v0[i] = digit_pair(y[2 * i], y[2 * i + 1], 6);
        v1[i] = digit_pair(y[2 * i], y[2 * i + 1], 5);
    }
    if constexpr (NA == 16) {
        tmem_st16(slot_addr, v0);
        tmem_st16(slot_addr + 32u, v1);
    } else {
        tmem_st8(slot_addr, v0);
        tmem_st8(slot_addr + 32u, v1);
    }
    tmem_st_wait();
    tc_before_sync();
    __syncwarp();
    if (lane == 0) {
        mbar_arrive(&full[0]);
        mbar_arrive(&full[1]);
    }
}

template <int S, int NA>
__device__ __forceinline__ void put_digit(const uint64_t (&y)[2 * NA], uint32_t tmem_slot_addr, uint64_t* full,
                                          uint32_t lane) {
    uint32_t v[NA];
#pragma unroll
    for (int i = 0; i < NA; ++i) v[i] = digit_pair(y[2 * i], y[2 * i + 1], 6 - S);
    if constexpr (NA == 16) tmem_st16(tmem_slot_addr, v);
    else tmem_st8(tmem_slot_addr, v);
    tmem_st_wait();
    tc_before_sync();
    __syncwarp();
    if (lane == 0) mbar_arrive(full);
}

// Math warps: the tile in buffer b once loaded, as the thread's 2 NA biased fixed-point values y.
template <bool kInF64, int NA>
__device__ __forceinline__ bool prep_tile(const double2* tiles, uint32_t b, uint32_t& ph_tma, uint32_t mrow,
                                          const uint32_t* rp, uint64_t (&y)[2 * NA], uint32_t E, int sigma,
                                          volatile int* abort_flag, int* err, uint64_t* bar_tma, uint32_t* loads_seen) {
    if (!wait_or_abort(&bar_tma[b], (ph_tma >> b) & 1u, abort_flag, err)) return false;
    ph_tma ^= 1u << b;
    if (loads_seen) ++loads_seen[b];
    const double2* tile = tiles + (size_t)b * kTileAmps;
#pragma unroll
    for (int i = 0; i < NA; ++i) {
        const double2 a = tile[mrow | rp[i]];
        if constexpr (kInF64) {
            y[2 * i] = slice(a.x, E);
            y[2 * i + 1] = slice(a.y, E);
        } else {
            y[2 * i] = renorm(__double_as_longlong(a.x), sigma);
            y[2 * i + 1] = renorm(__double_as_longlong(a.y), sigma);
        }
    }
    return true;
}

// The level-L columns of this lane (2 NA values, loaded together).
template <int NA>
__device__ __forceinline__ void load_level(uint32_t (&v)[2 * NA], uint32_t taddr) {
#pragma unroll
    for (int part = 0; part < NA / 4; ++part) {
        uint32_t w[8];
        tmem_ld8(taddr + 8u * (uint32_t)part, w);
#pragma unroll
        for (int kk = 0; kk < 8; ++kk) v[8 * part + kk] = w[kk];
    }
}

// Read back level L (0..5) of the thread's 2 NA output reals, once digit L's products are done (the
// last to add to that level), into the output sums X' = sum_l L_l 2^(41 - 8 l):
//   levels 0, 1: V = 256 L0 + L1 (magic-number bits, one 32-bit word);
//   levels 2, 3: U = 256 L2 + L3, then acc = 2 V 2^32 + U 2^17 (64 bits);
//   levels 4, 5: acc += L4 2^9 + L5 2 (exact float-to-int conversions: |L| may reach 2^22.5).
template <int L, int NA>
__device__ __forceinline__ void read_level(uint64_t (&acc)[2 * NA], uint32_t taddr) {
    uint32_t v[2 * NA];
    load_level<NA>(v, taddr + level_col(L));
    tmem_ld_wait();
#pragma unroll
    for (int k = 0; k < 2 * NA; ++k) {
        const float f = __uint_as_float(v[k]);
        if constexpr (L == 0) {
            acc[k] = mbits(f);
        } else if constexpr (L == 1) {
            acc[k] = (uint32_t)acc[k] * 256u + mbits(f);
        } else if constexpr (L == 2) {
            acc[k] = ((uint64_t)mbits(f) << 32) | (uint32_t)acc[k];
        } else if constexpr (L == 3) {
            const uint32_t Vm = (uint32_t)acc[k];                                  // V + 257 kMagic
            const uint32_t Um = (uint32_t)(acc[k] >> 32) * 256u + mbits(f);        // U + 257 kMagic
            const int32_t V = (int32_t)(Vm - 257u * kMagic), U = (int32_t)(Um - 257u * kMagic);
            acc[k] = ((uint64_t)(uint32_t)(2 * V) << 32) + (uint64_t)((int64_t)U << 17);
        } else if constexpr (L == 4) {
            acc[k] += (uint64_t)((int64_t)__float2int_rn(f) << 9);
        } else {
            acc[k] += (uint64_t)((int64_t)__float2int_rn(f) << 1);
        }
    }
}

// Levels 6 and 7 (level 7 in level 0's columns), once the tile's last products are done:
// acc += round(L6 2^-7 + L7 2^-15): the sum taken in FP32 (|.| < 2^16, so one rounding of at most
// 2^-9), then rounded to the nearest integer by a magic-number add: within 1/2 + 2^-9 of a unit.
template <int NA>
__device__ __forceinline__ void read_levels_67(uint64_t (&acc)[2 * NA], uint32_t taddr) {
    uint32_t v6[2 * NA], v7[2 * NA];
    load_level<NA>(v6, taddr + level_col(6));
    load_level<NA>(v7, taddr + level_col(7));
    tmem_ld_wait();
#pragma unroll
    for (int k = 0; k < 2 * NA; ++k) {
        const float t = fmaf(__uint_as_float(v6[k]), 0.0078125f, __uint_as_float(v7[k]) * 3.0517578125e-05f);
        acc[k] += (uint64_t)(int64_t)(int32_t)(mbits(t) - kMagic);
    }
}

template <int kRegs, int NA, bool kInF64, bool kOutF64>
__global__ void __maxnreg__(kRegs)
    tensor64_pass_kernel(double2* __restrict__ psi, const unsigned char* __restrict__ wts,
                         const __grid_constant__ TPassParams P, int* __restrict__ err) {
    using LY = Layout<NA>;
    constexpr uint32_t kNT = LY::kNT, kMathWarps = LY::kMathWarps, kMmaWarp = LY::kMmaWarp, kTmaWarp = LY::kTmaWarp;
    extern __shared__ __align__(1024) unsigned char smem[];
    double2* tiles = reinterpret_cast<double2*>(smem);  // two tile buffers
    unsigned char* w_sm = smem + 2 * (size_t)kTileAmps * 16;
    __shared__ uint64_t seg_off[1u << (kTQ - kLowQ)];
    __shared__ uint32_t mpos[128];
    __shared__ uint32_t rpos[32];
    __shared__ __align__(8) uint64_t bar_tma[2];      // tile loaded into buffer b (TMA bytes)
    __shared__ __align__(8) uint64_t bar_written[2];  // tile results written to buffer b (math warps)
    __shared__ __align__(8) uint64_t bar_drained[2];  // a store from buffer b has read it out (copy warp)
    __shared__ __align__(8) uint64_t bar_full[2];     // operand slot holds the next digit (math warps)
    __shared__ __align__(8) uint64_t bar_mma[2];      // that digit's MMAs are done (commit)
    __shared__ __align__(8) uint64_t bar_acc;         // accumulators read back (math warps)
    __shared__ __align__(8) uint64_t bar_l0;          // level 0 read back: its columns take level 7
    __shared__ uint32_t tmem_base;
    __shared__ int s_abort;
    __shared__ uint32_t s_loads[2], s_loads_seen[2], s_commits[2], s_commits_seen[2];
    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t c = P.c;
    const uint32_t nseg = 1u << (kTQ - c);
    const uint32_t seg_amps = 1u << c;

    // the register scale this pass reads and the one it writes
    const ScaleSlot in = P.slots[P.cur];
    uint32_t E = 0;
    int sigma = 0, S_in;
    if constexpr (kInF64) {
        E = in.mag;
        S_in = 1075 - (int)E;
    } else {
        sigma = in.mag ? kTopBits - 32 - (32 - __clz((int)in.mag)) : 0;
        S_in = in.S + sigma;
    }
    if (blockIdx.x == 0 && tid == 0) {
        P.slots[(P.cur + 1) % 3].S = S_in;
        P.slots[(P.cur + 2) % 3].mag = 0;
    }

    for (uint32_t s = tid; s < nseg; s += kNT) {
        uint64_t off = 0;
        for (uint32_t j = 0; j < kTQ - c; ++j)
            if ((s >> j) & 1u) off |= 1ull << P.tq[c + j];
        seg_off[s] = off;
    }
    uint32_t bm = 0;
    for (int j = 0; j < dense::kBQ; ++j) bm |= 1u << P.bits[j];
    if (tid < 128) {
        uint32_t pos = 0, bit = 0;
        for (uint32_t p = 0; p < (uint32_t)kTQ; ++p) {
            if ((bm >> p) & 1u) continue;
            if ((tid >> bit) & 1u) pos |= 1u << p;
            ++bit;
        }
        mpos[tid] = pos;
    } else if (tid < 160) {
        const uint32_t j = tid - 128;
        uint32_t pos = 0;
        for (int b = 0; b < dense::kBQ; ++b)
            if ((j >> b) & 1u) pos |= 1u << P.bits[b];
        rpos[j] = pos;
    }
    {
        const uint4* src = reinterpret_cast<const uint4*>(wts + P.w_off);
        uint4* dst = reinterpret_cast<uint4*>(w_sm);
        for (uint32_t i = tid; i < kWBlockBytes / 16; i += kNT) dst[i] = __ldg(src + i);
        for (uint32_t i = tid; i < kWDigitBytes / 16; i += kNT) dst[kWBlockBytes / 16 + i] = __ldg(src + i);
    }
    if (warp == 0) {
        tmem_alloc(&tmem_base, 512);
        tmem_relinquish();
    }
    if (tid == 0) {
        for (int i = 0; i < 2; ++i) {
            mbar_init(&bar_tma[i], 1);
            mbar_init(&bar_written[i], kMathWarps);
            mbar_init(&bar_drained[i], 1);
            mbar_init(&bar_full[i], kMathWarps);
            mbar_init(&bar_mma[i], 1);
            s_loads[i] = s_loads_seen[i] = s_commits[i] = s_commits_seen[i] = 0;
        }
        mbar_init(&bar_acc, kMathWarps);
        mbar_init(&bar_l0, kMathWarps);
        s_abort = 0;
        fence_mbar_init();
    }
    fence_proxy_async();  // the weights written above are read by the tensor cores
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
    const uint32_t tmem = tmem_base;
    volatile int* abort_flag = &s_abort;
    const uint64_t first = blockIdx.x, stride = gridDim.x;
    const uint32_t my_tiles = first < P.ntiles ? (uint32_t)((P.ntiles - 1 - first) / stride + 1) : 0u;

    auto tile_base = [&](uint64_t t) {
        uint64_t base = t;
        for (uint32_t p = 0; p < (uint32_t)kTQ; ++p) {
            const uint32_t q = P.tq[p];
            base = ((base >> q) << (q + 1)) | (base & ((1ull << q) - 1ull));
        }
        return base;
    };

    if (warp == kTmaWarp) {
        // ---- copies: loads two tiles ahead of the math warps, stores each tile once written ----
        auto issue_load = [&](uint32_t i) {
            const uint32_t b = i & 1u;
            const uint64_t base = tile_base(first + i * stride);
            double2* dst = tiles + (size_t)b * kTileAmps;
            if (lane == 0) {
                ++s_loads[b];
                mbar_expect_tx(&bar_tma[b], kTileAmps * 16u);
            }
            __syncwarp();
            for (uint32_t s = lane; s < nseg; s += 32)
                bulk_load(dst + (size_t)s * seg_amps, psi + (base | seg_off[s]), seg_amps * 16u, &bar_tma[b]);
        };
        // Tile j is loaded into buffer j % 2 and its results are written into the other buffer (after
        // the next tile there has been sliced), so that a buffer is reloaded two tiles after its last
        // store: the load has more than a tile to land.  Buffer 0 is first free once tile 0 is sliced.
        uint32_t ph_w = 0;  // phase parity of bar_written[b] in bit b
        for (uint32_t i = 0; i < my_tiles && i < 2; ++i) issue_load(i);
        bool go = my_tiles > 2 ? wait_or_abort(&bar_written[0], 0u, abort_flag, err) : true;
        ph_w = 1u;
        if (go && my_tiles > 2) issue_load(2);
        for (uint32_t i = 0; go && i < my_tiles; ++i) {
            const uint32_t x = (i + 1u) & 1u;  // the buffer holding tile i's results
            if (!wait_or_abort(&bar_written[x], (ph_w >> x) & 1u, abort_flag, err)) break;
            ph_w ^= 1u << x;
            const uint64_t base = tile_base(first + i * stride);
            const double2* src = tiles + (size_t)x * kTileAmps;
            for (uint32_t s = lane; s < nseg; s += 32)
                bulk_store(psi + (base | seg_off[s]), src + (size_t)s * seg_amps, seg_amps * 16u);
            bulk_commit();
            bulk_wait_read();  // the buffer is free for the tile three ahead
            __syncwarp();
            if (lane == 0) mbar_arrive(&bar_drained[x]);
            if (i + 3 < my_tiles) issue_load(i + 3);
        }
        bulk_wait_all();
    } else if (warp == kMmaWarp) {
        // ---- MMA issue: digit s of a tile once its slot is full (and, for digit 0, once the
        // previous tile's accumulators have been read back; for the level-7 products, once this
        // tile's level 0 has been) ----
        const uint32_t w_addr = smem_addr(w_sm);
        uint32_t ph_full = 0, ph_acc = 0, ph_l0 = 0;  // phase parities, bit = slot
        bool ok = true;
        for (uint32_t i = 0; ok && i < my_tiles; ++i) {
#pragma unroll
            for (int s = 0; s < kDigits; ++s) {
                const uint32_t slot = (uint32_t)s & 1u;
                if (ok && s == 0 && i > 0) {
                    ok = wait_or_abort(&bar_acc, ph_acc, abort_flag, err);
                    ph_acc ^= 1u;
                }
                if (ok) ok = wait_or_abort(&bar_full[slot], (ph_full >> slot) & 1u, abort_flag, err);
                ph_full ^= 1u << slot;
                const uint32_t a_tm = tmem + kSlotCol + 32u * slot;
                // the pairs (s, t0 .. t0 + m - 1) into m adjacent levels from s + t0: one MMA of N = 64 m per
                // K step (the block's digit matrices t0 .. t0 + m - 1 are one operand of 64 m rows)
                auto issue = [&](int t0, int m, bool init) {
                    const uint32_t d_tm = tmem + level_col(s + t0);
                    const uint32_t wb = w_addr + (uint32_t)t0 * kWDigitBytes;
#pragma unroll
                    for (uint32_t ks = 0; ks < 4; ++ks)
                        mma_f16_ta(d_tm, a_tm + 8u * ks, smem_desc(wb + 256u * ks, 128u, 1024u), idesc16((uint32_t)m),
                                   (init && ks == 0) ? 0u : 1u);
                };
                if (ok && lane == 0) {
                    tc_after_sync();
                    if (s == 0) {  // levels 1..4, then 5, 6 and 0 (digit matrices 5, 6 and the copy of 0)
                        issue(1, 4, true);
                        issue(5, 3, true);
                    } else {       // levels s .. 7; for digit 1, levels 5..7 once level 0 is read and cleared
                        issue(0, min(4, 8 - s), false);
                    }
                }
                if (s == 1 && ok) {
                    ok = wait_or_abort(&bar_l0, ph_l0, abort_flag, err);
                    ph_l0 ^= 1u;
                }
                if (ok && lane == 0 && s > 0 && 8 - s > 4) {
                    tc_after_sync();
                    issue(4, 4 - s, false);
                }
                if (ok && lane == 0) {
                    mma_commit(&bar_mma[slot]);
                    ++s_commits[slot];
                }
                __syncwarp();
            }
        }
    } else {
        // ---- math warps: a row (lane quadrant) and NA of its 32 amplitudes (column group) ----
        const uint32_t quad = warp & 3u, cg = warp >> 2;
        const uint32_t row = 32u * quad + lane;
        const uint32_t lane_addr = (32u * quad) << 16;
        const uint32_t slot0 = tmem + lane_addr + kSlotCol + (uint32_t)NA * cg;
        const uint32_t* rp = rpos + (uint32_t)NA * cg;
        const uint32_t mrow = mpos[row];  // amplitude i of this thread sits at mrow | rp[i]
        const bool counter = quad == 0 && cg == 0 && lane == 0;
        uint32_t ph_tma = 0, ph_mma = 0;  // phase parities, bit = buffer / slot
        uint32_t mag = 0;                 // OR of the fixed-point outputs' high-word magnitudes
        uint64_t y[2 * NA];
        auto wait_mma = [&](uint32_t slot) -> bool {
            const bool r = wait_or_abort(&bar_mma[slot], (ph_mma >> slot) & 1u, abort_flag, err);
            ph_mma ^= 1u << slot;
            if (r && counter) ++s_commits_seen[slot];
            tc_after_sync();
            return r;
        };
        bool ok = my_tiles > 0 && prep_tile<kInF64, NA>(tiles, 0, ph_tma, mrow, rp, y, E, sigma, abort_flag, err,
                                                        bar_tma, counter ? s_loads_seen : nullptr);
        __syncwarp();
        if (ok && lane == 0) mbar_arrive(&bar_written[0]);  // buffer 0 sliced: it may take tile 2
        if (ok) put_digits01<NA>(y, slot0, bar_full, lane);
        const uint32_t acc_addr = tmem + lane_addr + 2u * NA * cg;  // this thread's columns at column 0
        for (uint32_t i = 0; ok && i < my_tiles; ++i) {
            const uint32_t b = i & 1u;
            // a slot takes digit s once the MMAs of digit s - 2 are done; level l is final once digit
            // l's are, and is read back then
            uint64_t acc[2 * NA];
            ok = wait_mma(0);
            if (ok) {
                read_level<0, NA>(acc, acc_addr);
                {  // level 0's columns, cleared, take level 7
                    uint32_t z[8] = {0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};
#pragma unroll
                    for (int part = 0; part < NA / 4; ++part) tmem_st8(acc_addr + level_col(7) + 8u * part, z);
                    tmem_st_wait();
                }
                tc_before_sync();
                __syncwarp();
                if (lane == 0) mbar_arrive(&bar_l0);
                put_digit<2, NA>(y, slot0, &bar_full[0], lane);
                ok = wait_mma(1);
            }
            if (ok) {
                read_level<1, NA>(acc, acc_addr);
                put_digit<3, NA>(y, slot0 + 32u, &bar_full[1], lane);
                ok = wait_mma(0);
            }
            if (ok) {
                read_level<2, NA>(acc, acc_addr);
                put_digit<4, NA>(y, slot0, &bar_full[0], lane);
                ok = wait_mma(1);
            }
            if (ok) {
                read_level<3, NA>(acc, acc_addr);
                put_digit<5, NA>(y, slot0 + 32u, &bar_full[1], lane);
                ok = wait_mma(0);
            }
            if (ok) {
                read_level<4, NA>(acc, acc_addr);
                put_digit<6, NA>(y, slot0, &bar_full[0], lane);
            }
            if (!ok) break;
            // levels 5, 6 and 7: the commits of digits 5 (slot 1) and 6 (slot 0), the last of this tile
            const bool done5 = wait_mma(1);
            if (done5) read_level<5, NA>(acc, acc_addr);
            const bool done6 = wait_mma(0);
            if (!(done5 && done6)) break;
            read_levels_67<NA>(acc, acc_addr);
            tc_before_sync();
            __syncwarp();
            if (lane == 0) mbar_arrive(&bar_acc);
            // the next tile (its load had the whole of this tile to land: the buffer's previous tile is
            // stored first) and its first two digits, while this tile's results are written
            const bool has_next = i + 1 < my_tiles;
            if (has_next)
                ok = prep_tile<kInF64, NA>(tiles, b ^ 1u, ph_tma, mrow, rp, y, E, sigma, abort_flag, err, bar_tma,
                                           counter ? s_loads_seen : nullptr);
            if (has_next && ok) put_digits01<NA>(y, slot0, bar_full, lane);
            // the results go to the other buffer (its tile, the next, was sliced above); after the last
            // tile, once the store from that buffer two tiles back has read it out
            if (!has_next && i >= 2 && !wait_or_abort(&bar_drained[b ^ 1u], ((i >> 1) - 1u) & 1u, abort_flag, err)) break;
            double2* tile = tiles + (size_t)(b ^ 1u) * kTileAmps;
#pragma unroll
            for (int k = 0; k < NA; ++k) {
                const int64_t v0 = (int64_t)acc[2 * k], v1 = (int64_t)acc[2 * k + 1];
                if constexpr (kOutF64) {
                    tile[mrow | rp[k]] = make_double2(scaled_to_f64(v0, -S_in), scaled_to_f64(v1, -S_in));
                } else {
                    const int32_t h0 = (int32_t)(v0 >> 32), h1 = (int32_t)(v1 >> 32);
                    mag |= (uint32_t)(h0 ^ (h0 >> 31)) | (uint32_t)(h1 ^ (h1 >> 31));
                    tile[mrow | rp[k]] = make_double2(__longlong_as_double(v0), __longlong_as_double(v1));
                }
            }
            fence_proxy_async();  // the results are read by the TMA store
            __syncwarp();
            if (lane == 0) mbar_arrive(&bar_written[b ^ 1u]);
        }
        if constexpr (!kOutF64) {
            mag = __reduce_or_sync(0xffffffffu, mag);
            if (lane == 0 && mag) atomicOr(&P.slots[(P.cur + 1) % 3].mag, mag);
        }
    }
    // teardown: after an abort, let the copies and MMAs in flight land before the memory goes away
    __syncthreads();
    if (s_abort && tid == 0) {
        for (int b = 0; b < 2; ++b) {
            uint32_t seen = s_loads_seen[b];
            while (seen < s_loads[b] && mbar_wait(&bar_tma[b], seen & 1u, kWaitLimit)) ++seen;
            seen = s_commits_seen[b];
            while (seen < s_commits[b] && mbar_wait(&bar_mma[b], seen & 1u, kWaitLimit)) ++seen;
        }
    }
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
    if (warp == 0) tmem_dealloc(tmem_base, 512);
}

// The cost of the pass's tensor-core instructions, measured in isolation: one thread per CTA issues
// `reps` rounds of 44 tcgen05.mma kind::f16 (M = 128, K = 16; A from tensor memory, B from shared
// memory) and waits for their commit; clock64 around it.  mode 0: a tile of the pass (11 MMAs of
// N = 64 m per K step, the pass's mix); 1: N = 64 only; 2: N = 256 only.  Operand values do not
// matter (shared memory holds fp16 ones, tensor memory is not initialised).
__global__ void tensor64_mma_cost_kernel(int mode, int reps, unsigned long long* out, int* err) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ uint32_t tmem_base;
    __shared__ __align__(8) uint64_t bar;
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (uint32_t i = threadIdx.x; i < (kWBlockBytes + kWDigitBytes) / 4; i += blockDim.x)
        reinterpret_cast<uint32_t*>(smem)[i] = 0x3C003C00u;
    if (warp == 0) {
        tmem_alloc(&tmem_base, 512);
        tmem_relinquish();
    }
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    fence_proxy_async();
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
    const uint32_t tmem = tmem_base, w = smem_addr(smem);
    const unsigned long long t0 = clock64();
    if (warp == 0 && lane == 0) {
        for (int it = 0; it < reps; ++it)
            for (int s = 0; s < kDigits; ++s) {
                const uint32_t a_tm = tmem + kSlotCol + 32u * (uint32_t)(s & 1);
                for (uint32_t ks = 0; ks < 4; ++ks) {
                    const uint64_t bd = smem_desc(w + 256u * ks, 128u, 1024u);
                    if (mode == 0) {  // the m of each of digit s's MMAs: 4 then 3 (s = 0, 1), 4 then 8 - s - 4, or 8 - s
                        const int first = s == 0 ? 4 : min(4, 8 - s);
                        const int second = s == 0 ? 3 : 8 - s - first;
                        mma_f16_ta(tmem, a_tm + 8u * ks, bd, idesc16((uint32_t)first), 1u);
                        if (second > 0) mma_f16_ta(tmem + 256u, a_tm + 8u * ks, bd, idesc16((uint32_t)second), 1u);
                    } else {
                        // 44 per tile: 6 or 7 per digit and K step
                        const int n = s < 4 ? 2 : 1;
                        for (int c = 0; c < n; ++c)
                            mma_f16_ta(tmem + 128u * (uint32_t)c, a_tm + 8u * ks, bd, idesc16(mode == 1 ? 1u : 4u), 1u);
                    }
                }
            }
        mma_commit(&bar);
    }
    __syncwarp();
    if (warp == 0 && !mbar_wait(&bar, 0u, 1u << 26)) atomicExch(err, 1);
    const unsigned long long t1 = clock64();
    if (threadIdx.x == 0) out[blockIdx.x] = t1 - t0;
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
    if (warp == 0) tmem_dealloc(tmem_base, 512);
}

// The largest biased f64 exponent of the register's components, into slot 0 of its scale ring (the
// ring cleared before).
__global__ void tensor64_maxexp_kernel(const double2* __restrict__ psi, uint64_t len, ScaleSlot* slots) {
    uint32_t m = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < len; i += (uint64_t)gridDim.x * blockDim.x) {
        const double2 a = psi[i];
        const uint32_t e0 = (uint32_t)((uint64_t)__double_as_longlong(a.x) >> 52) & 0x7ffu;
        const uint32_t e1 = (uint32_t)((uint64_t)__double_as_longlong(a.y) >> 52) & 0x7ffu;
        m = max(m, max(e0, e1));
    }
    m = __reduce_max_sync(0xffffffffu, m);
    if ((threadIdx.x & 31u) == 0 && m) atomicMax(&slots[0].mag, m);
}

// ---- host -----------------------------------------------------------------------------------------
uint16_t fp16_of_small_int(int d) {  // exact for |d| <= 2048
    if (d == 0) return 0;
    const uint16_t sgn = d < 0 ? 0x8000 : 0;
    uint32_t a = (uint32_t)(d < 0 ? -d : d);
    int e = 31 - __builtin_clz(a);
    const uint32_t mant = (a << (10 - e)) & 0x3ffu;
    return (uint16_t)(sgn | ((uint32_t)(e + 15) << 10) | mant);
}

// fp16 bits of the balanced digits -128 .. 128.
struct DigitTable {
    uint16_t h[257];
    DigitTable() {
        for (int d = -128; d <= 128; ++d) h[d + 128] = fp16_of_small_int(d);
    }
};

// A block's weights: the real 64 x 64 form W[2r' + c'][2r + c] = ((Re, -Im), (Im, Re)) of U[r'][r]
// (row = output real, column = input real) as the integers round(W 2^55) and their seven balanced
// base-256 digits (|digit| <= 128; digit t = 0 most significant) in fp16, in the operand layout.
// False when an entry is not finite or above 1 in magnitude (the digit bounds assume a unitary).
bool block_weights64(const dense::Block& b, unsigned char* out) {
    static const DigitTable digits;
    static thread_local double W[64][64];
    for (uint32_t rp = 0; rp < 32; ++rp)
        for (uint32_t r = 0; r < 32; ++r) {
            const dense::Cd u = b.u[rp * 32 + r];
            W[2 * rp][2 * r] = u.re;
            W[2 * rp][2 * r + 1] = -u.im;
            W[2 * rp + 1][2 * r] = u.im;
            W[2 * rp + 1][2 * r + 1] = u.re;
        }
    uint16_t* dig = reinterpret_cast<uint16_t*>(out);
    for (uint32_t n = 0; n < 64; ++n)
        for (uint32_t k = 0; k < 64; ++k) {
            const double w = W[n][k];
            if (!(std::fabs(w) <= 1.0 + 1e-9)) return false;
            int64_t rest = std::llrint(std::ldexp(w, kWScale));
            int d[kDigits];
            for (int t = kDigits - 1; t >= 1; --t) {
                d[t] = (int)((((rest + 128) % 256) + 256) % 256) - 128;
                rest = (rest - d[t]) / 256;
            }
            d[0] = (int)rest;  // |d[0]| <= 128
            for (int t = 0; t < kDigits; ++t)
                dig[(size_t)t * (kWDigitBytes / 2) + w_off16(n, k)] = digits.h[std::clamp(d[t], -128, 128) + 128];
        }
    return true;
}

// A gate goes through dense blocks when each of its dense factors (the multi-bit X/Y/Z/S/T split
// into one-qubit factors) spans at most five qubits with its controls; wider gates run as single
// passes of the plain f64 kernels.
bool blockable(const qvnt_gate& g) {
    const bool multi = g.kind == QVNT_GATE_X || g.kind == QVNT_GATE_Y || g.kind == QVNT_GATE_Z ||
                       g.kind == QVNT_GATE_S || g.kind == QVNT_GATE_T;
    if (g.kind == QVNT_GATE_ID) return true;
    if (multi) return 1 + __builtin_popcountll(g.ctrl) <= dense::kBQ;
    uint64_t tg = g.a_mask;
    if (g.kind == QVNT_GATE_H2 || g.kind == QVNT_GATE_U2) tg |= g.b_mask;
    return __builtin_popcountll(tg | g.ctrl) <= dense::kBQ;
}

int plan_blocks(const qvnt_gate* gates, size_t count, uint32_t L, std::vector<dense::Block>& blocks,
                std::vector<dense::PPlan>& passes) {
    std::vector<dense::LGate> lg;
    TRY_T(dense::lower_dense(gates, count, lg));
    dense::make_blocks(lg, L, blocks, 96);
    return dense::make_passes(blocks, L, kTQ, kLowQ, 1, passes);
}

using PassFn = void (*)(double2*, const unsigned char*, const TPassParams, int*);
// The four forms of one layout, indexed by (input f64) * 2 + (output f64).
struct PassKernel {
    PassFn fn[4] = {nullptr, nullptr, nullptr, nullptr};
    uint32_t threads = 0;
    int regs = 0;
    char why[160] = {0};
};

template <int kRegs, int NA>
PassKernel forms_of() {
    PassKernel k;
    k.fn[0] = tensor64_pass_kernel<kRegs, NA, false, false>;
    k.fn[1] = tensor64_pass_kernel<kRegs, NA, false, true>;
    k.fn[2] = tensor64_pass_kernel<kRegs, NA, true, false>;
    k.fn[3] = tensor64_pass_kernel<kRegs, NA, true, true>;
    k.threads = Layout<NA>::kNT;
    return k;
}

// The layouts in order of preference (measured on the 30-qubit circuit: 9.45 ms against 10.9 ms per
// pass): 16 math warps of 8 amplitudes with 96 registers (five of the eighteen warps share an SM
// sub-partition's 16K registers), 8 math warps of 16 amplitudes with 168 registers (three of ten);
// QVNT_T64_LAYOUT=8 or 16 picks one (amplitudes per math thread).
PassKernel pick_kernel() {
    PassKernel out;
    struct Cand {
        PassKernel k;
        int na;
    };
    const Cand cands[2] = {{forms_of<96, 8>(), 8}, {forms_of<168, 16>(), 16}};
    const char* env = std::getenv("QVNT_T64_LAYOUT");
    const int want = env ? std::atoi(env) : 0;
    for (const Cand& c : cands) {
        if (want && c.na != want) continue;
        bool good = true;
        int regs = 0;
        for (PassFn fn : c.k.fn) {
            cudaFuncAttributes a;
            if (cudaFuncGetAttributes(&a, (const void*)fn) != cudaSuccess) {
                good = false;
                break;
            }
            if (a.maxThreadsPerBlock < (int)c.k.threads) {
                snprintf(out.why, sizeof out.why, "%d registers allow %d threads per block, %u needed", a.numRegs,
                         a.maxThreadsPerBlock, c.k.threads);
                good = false;
                break;
            }
            if (cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemDyn) !=
                cudaSuccess) {
                snprintf(out.why, sizeof out.why, "shared-memory attribute refused");
                good = false;
                break;
            }
            regs = std::max(regs, a.numRegs);
        }
        if (!good) continue;
        out = c.k;
        out.regs = regs;
        return out;
    }
    cudaGetLastError();
    return out;
}

// The register's scale ring: three slots after the 64 bytes of device results.
ScaleSlot* scale_ring(qvnt_reg* r) {
    return reinterpret_cast<ScaleSlot*>(reinterpret_cast<char*>(r->d_small) + 64);
}

// One run of blockable gates: the reduction for the register's largest exponent, then one pass per
// block (f64 in for the first, f64 out for the last, 64-bit block floating point in between).
int run_blocks(qvnt_reg* r, const qvnt_gate* gates, size_t count) {
    const uint32_t L = (uint32_t)__builtin_ctzll(r->len);
    std::vector<dense::Block> blocks;
    std::vector<dense::PPlan> passes;
    TRY_T(plan_blocks(gates, count, L, blocks, passes));
    if (passes.empty()) return QVNT_OK;
    const size_t wbytes = blocks.size() * (size_t)kWBlockBytes;
    EngineBuffers& fs = r->bufs;
    TRY_T(fs.acquire(wbytes, r->stream));
    unsigned char* hw = static_cast<unsigned char*>(fs.h_buf);
    for (size_t i = 0; i < blocks.size(); ++i)
        if (!block_weights64(blocks[i], hw + i * (size_t)kWBlockBytes)) return apply_plain(r, gates, count);
    TRY_T(fs.upload(wbytes, r->stream));
    static const PassKernel kern = pick_kernel();
    if (!kern.fn[0]) return set_error(QVNT_ERR_CUDA, "tensor64 kernel: %s", kern.why);
    int* d_err = reinterpret_cast<int*>(reinterpret_cast<char*>(r->d_small) + 32);
    ScaleSlot* ring = scale_ring(r);
    QVNT_CUDA_TRY(cudaMemsetAsync(ring, 0, 3 * sizeof(ScaleSlot), r->stream));
    {
        const uint64_t grid = std::min<uint64_t>((uint64_t)r->ctx->geo.sms * 4, (r->len + 255) / 256);
        tensor64_maxexp_kernel<<<(unsigned)grid, 256, 0, r->stream>>>(r->psi, r->len, ring);
        QVNT_CUDA_TRY(cudaGetLastError());
        r->launches += 1;
    }
    for (size_t pi = 0; pi < passes.size(); ++pi) {
        const dense::PPlan& p = passes[pi];
        TPassParams P;
        memset(&P, 0, sizeof P);
        uint32_t n = 0, pos_of[64];
        for (uint32_t q = 0; q < L; ++q)
            if ((p.qmask >> q) & 1ull) {
                pos_of[q] = n;
                P.tq[n++] = q;
            }
        if (n != (uint32_t)kTQ) return set_error(QVNT_ERR_UNSUPPORTED, "tensor64 planner: tile of %u qubits", n);
        uint32_t run = 0;
        while (run < n && P.tq[run] == run) ++run;
        if (run < kLowQ) return set_error(QVNT_ERR_UNSUPPORTED, "tensor64 planner: low run of %u qubits", run);
        P.c = run;
        P.ntiles = r->len >> kTQ;
        const size_t bi = p.members[0];
        const dense::Block& blk = blocks[bi];
        uint32_t jj = 0;
        for (uint32_t q = 0; q < L; ++q)
            if ((blk.sup >> q) & 1ull) P.bits[jj++] = (uint8_t)pos_of[q];
        P.w_off = bi * (uint64_t)kWBlockBytes;
        P.slots = ring;
        P.cur = (uint32_t)(pi % 3);
        const int form = (pi == 0 ? 2 : 0) + (pi + 1 == passes.size() ? 1 : 0);
        // persistent (one CTA per SM), or one CTA per tile for registers that share the GPU
        const uint64_t grid = r->tile_grid ? P.ntiles : std::min<uint64_t>((uint64_t)r->ctx->geo.sms, P.ntiles);
        cudaEvent_t stop = nullptr;
        TRY_T(timing_begin(r, &stop));
        kern.fn[form]<<<(unsigned)grid, kern.threads, kSmemDyn, r->stream>>>(
            r->psi, static_cast<const unsigned char*>(fs.d_buf), P, d_err);
        const cudaError_t le = cudaGetLastError();
        if (le != cudaSuccess)
            return set_error(QVNT_ERR_CUDA, "tensor64 launch (%d threads, %zu B dynamic shared memory, %d registers): %s",
                             (int)kern.threads, kSmemDyn, kern.regs, cudaGetErrorString(le));
        TRY_T(timing_end(r, stop));
        r->launches += 1;
        r->passes += 1;
    }
    return QVNT_OK;
}

}  // namespace

// Registers below 12 qubits have no full tile: they run on the plain f64 kernels.
int apply_tensor64(qvnt_reg* r, const qvnt_gate* gates, size_t count) {
    const uint32_t L = (uint32_t)__builtin_ctzll(r->len);
    if (L < (uint32_t)kTQ) return apply_plain(r, gates, count);
    size_t i = 0;
    while (i < count) {
        size_t j = i;
        while (j < count && blockable(gates[j])) ++j;
        if (j > i) TRY_T(run_blocks(r, gates + i, j - i));
        if (j < count) {
            TRY_T(apply_plain(r, gates + j, 1));
            ++j;
        }
        i = j;
    }
    return QVNT_OK;
}
int tensor64_plan_info(const qvnt_gate* gates, size_t count, uint32_t L, uint64_t* passes, uint64_t* plain_gates) {
    uint64_t np = 0, pg = 0;
    if (L < (uint32_t)kTQ) {
        for (size_t k = 0; k < count; ++k) pg += gates[k].kind != QVNT_GATE_ID;
    } else {
        size_t i = 0;
        while (i < count) {
            size_t j = i;
            while (j < count && blockable(gates[j])) ++j;
            if (j > i) {
                std::vector<dense::Block> blocks;
                std::vector<dense::PPlan> ps;
                TRY_T(plan_blocks(gates + i, j - i, L, blocks, ps));
                np += ps.size();
            }
            if (j < count) {
                ++pg;
                ++j;
            }
            i = j;
        }
    }
    if (passes) *passes = np;
    if (plain_gates) *plain_gates = pg;
    return QVNT_OK;
}

int tensor64_mma_costs(int device, int sms, double* n64, double* n256, double* tile) {
    const size_t smem = kWBlockBytes + kWDigitBytes;
    QVNT_CUDA_TRY(cudaSetDevice(device));
    QVNT_CUDA_TRY(cudaFuncSetAttribute((const void*)tensor64_mma_cost_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    unsigned long long* d_out = nullptr;
    int* d_err = nullptr;
    QVNT_CUDA_TRY(cudaMalloc(&d_out, sizeof(unsigned long long) * (size_t)sms));
    QVNT_CUDA_TRY(cudaMalloc(&d_err, sizeof(int)));
    QVNT_CUDA_TRY(cudaMemset(d_err, 0, sizeof(int)));
    std::vector<unsigned long long> h((size_t)sms);
    double res[3] = {0, 0, 0};
    const int reps = 200;
    int st = QVNT_OK;
    for (int mode = 0; mode < 3 && !st; ++mode) {
        for (int rep = 0; rep < 2; ++rep) tensor64_mma_cost_kernel<<<sms, 128, smem>>>(mode, reps, d_out, d_err);
        cudaError_t e = cudaDeviceSynchronize();
        if (e == cudaSuccess) e = cudaMemcpy(h.data(), d_out, sizeof(unsigned long long) * (size_t)sms, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) {
            st = set_cuda_error(e, "mma cost kernel");
            break;
        }
        double avg = 0;
        for (unsigned long long v : h) avg += (double)v;
        avg /= (double)sms;
        res[mode] = mode == 0 ? avg / reps : avg / reps / 44.0;  // per tile, or per MMA
    }
    int h_err = 0;
    if (!st) {
        cudaMemcpy(&h_err, d_err, sizeof(int), cudaMemcpyDeviceToHost);
        if (h_err) st = set_error(QVNT_ERR_TIMEOUT, "mma cost kernel: commit wait ran out");
    }
    cudaFree(d_out);
    cudaFree(d_err);
    if (st) return st;
    *tile = res[0];
    *n64 = res[1];
    *n256 = res[2];
    return QVNT_OK;
}

int tensor64_plan_blocks(const qvnt_gate* gates, size_t count, uint32_t L, uint64_t* sups, double* mats, size_t cap,
                         size_t* nblocks) {
    std::vector<dense::LGate> lg;
    TRY_T(dense::lower_dense(gates, count, lg));
    std::vector<dense::Block> blocks;
    dense::make_blocks(lg, L, blocks, 96);
    *nblocks = blocks.size();
    if (cap < blocks.size()) return QVNT_OK;
    for (size_t i = 0; i < blocks.size(); ++i) {
        sups[i] = blocks[i].sup;
        for (int e = 0; e < dense::kBD * dense::kBD; ++e) {
            mats[2048 * i + 2 * e] = blocks[i].u[e].re;
            mats[2048 * i + 2 * e + 1] = blocks[i].u[e].im;
        }
    }
    return QVNT_OK;
}

}  // namespace qvnt
