// Tensor-core f64 engine: IEEE f64 amplitudes in HBM (qvnt's Complex<f64> layout, the PLAIN
// format), runs of gates fused into dense 5-qubit blocks (32 x 32 complex unitaries, the planner of
// dense_blocks.h) and contracted on the tcgen05 tensor cores with 53-bit operands by exact integer
// slicing (the Ozaki splitting of a matrix product into exactly representable digit products).
//
// Arithmetic.  Every operand row is scaled by a power of two to its largest element and rounded
// to a 53-bit integer (an f64 significand): the state row X (the 32 amplitudes of one block
// index group, 64 reals, scaled by the row's largest f64 exponent E) and the block matrix row W
// (64 reals of one output component, scaled by its exponent F).  Each integer is split into seven
// balanced base-256 digits in [-128, 127] (the top one in [-33, 32]), exact in fp16.  The block
// product is the sum over digit pairs (s, t) of A_s * B_t^T weighted by 256^(12 - s - t); the 28
// pairs with s + t <= 6 are issued as tcgen05.mma kind::f16 (M = 128 rows, N = 64, K = 16) into
// seven FP32 accumulators in tensor memory, one per level l = s + t.  Every partial sum is an
// integer below 2^23 in magnitude (at most l + 1 products of 64 terms of |digit| <= 128), so the
// FP32 accumulation is exact.  Levels >= 7 are dropped (below 2^-55 of the row bound).  The
// accumulators are read back (tcgen05.ld), turned into integers with a magic-number add, combined
// into one 64-bit integer and rounded to the nearest f64 with the exponent E + F - 2094: per block
// the result carries one rounding of the inputs (2^-53 of the row's power-of-two bound) and one
// rounding to f64, no FP64 instruction is issued.
//
// Kernel (one pass = one block): persistent CTAs of 512 threads, one per SM (tensor memory: all
// 512 columns).  Per tile of 4096 amplitudes (12 tile qubits: the 7 lowest, so a tile is 2 KB
// runs, plus the block's): TMA bulk loads into one of two shared-memory buffers (the next tile
// loads while this one computes); each thread takes one row (lane quadrant) and 8 of its 32
// amplitudes, finds the row exponent with its three partners, slices its 16 reals and stores the
// digits to two ping-pong operand slots in tensor memory; one thread issues each digit's MMAs and
// commits them to the slot's mbarrier, so the next digit's store waits only for the digit two
// before it.  Read-back, reconstruction and the TMA bulk store of the tile follow.
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
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
constexpr uint32_t kNT = 512;                   // 16 warps: 4 lane quadrants x 4 column groups
constexpr int kDigits = 7;                      // base-256 digits per 53-bit operand
constexpr uint32_t kWDigitBytes = 64 * 64 * 2;  // one fp16 digit matrix of a block (8 KB)
constexpr uint32_t kWBlockBytes = kDigits * kWDigitBytes + 64 * 4;  // digits + 64 row exponents
constexpr uint32_t kWaitLimit = 1u << 22;       // mbarrier polls before a wait gives up
constexpr uint32_t kSlotCol = 448;              // tensor-memory columns: levels 0..6 at 64 l, slots 448 / 480
constexpr uint64_t kBias = 0x80808080808080ull; // 128 in each of the 7 digit bytes
constexpr size_t kSmemDyn = 2 * (size_t)kTileAmps * 16 + kWBlockBytes;

// Instruction descriptor of kind::f16: FP32 accumulator, A and B fp16 and K-major, N = 64, M = 128.
constexpr uint32_t kIdesc16 = (1u << 4) | ((64u >> 3) << 17) | ((128u >> 4) << 24);

// fp16 element offset of B[row][k] (row = output real, k = input real) in the no-swizzle K-major
// operand layout: core matrices of 8 rows x 16 bytes; adjacent along K 128 B apart, 8-row groups
// 1024 B apart.
__host__ __device__ constexpr uint32_t w_off16(uint32_t row, uint32_t k) {
    return (row >> 3) * 512u + (k >> 3) * 64u + (row & 7u) * 8u + (k & 7u);
}

struct TPassParams {
    uint64_t ntiles;
    uint64_t w_off;      // byte offset of the block's weights in the weight buffer
    uint32_t c;          // tile qubits 0 .. c-1 are the register's lowest: runs of 2^c amplitudes
    uint32_t tq[kTQ];    // tile qubits, ascending
    uint8_t bits[dense::kBQ];  // tile-local bit of block bit j
};

__device__ __forceinline__ void mma_f16_ta(uint32_t d_tmem, uint32_t a_tmem, uint64_t b, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}" ::"r"(d_tmem),
        "r"(a_tmem), "l"(b), "r"(kIdesc16), "r"(accumulate)
        : "memory");
}

// 53-bit fixed point of x against the row exponent E (biased, >= x's): X = round(x * 2^(1075 - E)),
// |X| < 2^53; returns Y = X + kBias, whose byte j minus 128 is the balanced digit j of X.  Zeros and
// f64 subnormals give X = 0.
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

// Digits `byte` of two reals as a packed fp16 pair: fp16(1408 + c) has the bits 0x6580 + c for a
// byte c, and subtracting 1536 leaves c - 128 exactly.
__device__ __forceinline__ uint32_t digit_pair(uint64_t y0, uint64_t y1, int byte) {
    const uint32_t b0 = (uint32_t)(y0 >> (8 * byte)) & 0xffu;
    const uint32_t b1 = (uint32_t)(y1 >> (8 * byte)) & 0xffu;
    uint32_t h = (b0 | (b1 << 16)) + 0x65806580u;
    __half2 v = *reinterpret_cast<__half2*>(&h);
    v = __hsub2(v, __halves2half2(__ushort_as_half((unsigned short)0x6600), __ushort_as_half((unsigned short)0x6600)));
    return *reinterpret_cast<uint32_t*>(&v);
}

// Integer value of an integer-valued float: |f| < 2^22 exactly; |f| < 2^23 to the nearest even
// (f2i_even); round(f / 256).
__device__ __forceinline__ int32_t f2i(float f) { return __float_as_int(f + 12582912.0f) - 0x4B400000; }
__device__ __forceinline__ int32_t f2i_even(float f) { return (__float_as_int(f + 25165824.0f) - 0x4BC00000) * 2; }
__device__ __forceinline__ int32_t f2i_div256(float f) {
    return __float_as_int(fmaf(f, 0.00390625f, 12582912.0f)) - 0x4B400000;
}

// v * 2^T rounded to the nearest f64 (ties to even); below the normal range: signed zero.
__device__ __forceinline__ double scaled_to_f64(int64_t v, int T) {
    if (v == 0) return 0.0;
    const uint64_t sgn = (uint64_t)v & 0x8000000000000000ull;
    uint64_t a = v < 0 ? 0ull - (uint64_t)v : (uint64_t)v;
    const int lz = __clzll((long long)a);
    a <<= lz;
    uint64_t mant = a >> 11;
    const uint32_t rem = (uint32_t)a & 0x7ffu;
    mant += (uint64_t)((rem > 0x400u) | ((rem == 0x400u) & (uint32_t)(mant & 1ull)));
    const int e = 63 - lz + T + 1023;
    if (e <= 0) return __longlong_as_double((long long)sgn);
    return __longlong_as_double((long long)(sgn | (((uint64_t)(e - 1) << 52) + mant)));
}

__global__ void __launch_bounds__(kNT, 1)
    tensor64_pass_kernel(double2* __restrict__ psi, const unsigned char* __restrict__ wts,
                         const __grid_constant__ TPassParams P, int* __restrict__ err) {
    extern __shared__ __align__(1024) unsigned char smem[];
    double2* tiles = reinterpret_cast<double2*>(smem);  // two tile buffers
    unsigned char* w_sm = smem + 2 * (size_t)kTileAmps * 16;
    __shared__ uint64_t seg_off[1u << (kTQ - kLowQ)];
    __shared__ uint32_t mpos[128];
    __shared__ uint32_t rpos[32];
    __shared__ uint32_t s_exp[4][128];
    __shared__ __align__(8) uint64_t bar_tma[2];
    __shared__ __align__(8) uint64_t bar_mma[2];
    __shared__ uint32_t tmem_base;
    __shared__ int s_abort;
    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t quad = warp & 3u, cg = warp >> 2;
    const uint32_t row = 32u * quad + lane;  // operand row (lane of tensor memory)
    const uint32_t c = P.c;
    const uint32_t nseg = 1u << (kTQ - c);
    const uint32_t seg_amps = 1u << c;

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
    }
    if (warp == 0) {
        tmem_alloc(&tmem_base, 512);
        tmem_relinquish();
    }
    if (tid == 0) {
        for (int i = 0; i < 2; ++i) {
            mbar_init(&bar_tma[i], 1);
            mbar_init(&bar_mma[i], 1);
        }
        s_abort = 0;
        fence_mbar_init();
    }
    fence_proxy_async();  // the weights written above are read by the tensor cores
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
    const uint32_t tmem = tmem_base;
    const uint32_t lane_addr = (32u * quad) << 16;
    const int32_t* w_exp = reinterpret_cast<const int32_t*>(w_sm + kDigits * kWDigitBytes);
    int32_t fexp[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) fexp[i] = w_exp[16 * cg + i];
    const uint32_t w_addr = smem_addr(w_sm);
    const bool leader = warp == 0;
    uint32_t ph_tma[2] = {0, 0}, ph_mma[2] = {0, 0};

    auto tile_base = [&](uint64_t t) {
        uint64_t base = t;
        for (uint32_t p = 0; p < (uint32_t)kTQ; ++p) {
            const uint32_t q = P.tq[p];
            base = ((base >> q) << (q + 1)) | (base & ((1ull << q) - 1ull));
        }
        return base;
    };
    auto issue_load = [&](uint64_t t, uint32_t b) {  // leader warp
        const uint64_t base = tile_base(t);
        double2* dst = tiles + (size_t)b * kTileAmps;
        if (lane == 0) {
            fence_proxy_async();
            mbar_expect_tx(&bar_tma[b], kTileAmps * 16u);
        }
        __syncwarp();
        for (uint32_t s = lane; s < nseg; s += 32)
            bulk_load(dst + (size_t)s * seg_amps, psi + (base | seg_off[s]), seg_amps * 16u, &bar_tma[b]);
    };
    auto wait_bar = [&](uint64_t* bar, uint32_t& ph) {
        if (!mbar_wait(bar, ph, kWaitLimit)) {
            atomicExch(err, 1);
            s_abort = 1;
        }
        ph ^= 1u;
    };

    if (leader && (uint64_t)blockIdx.x < P.ntiles) issue_load(blockIdx.x, 0);
    uint32_t it = 0;
    for (uint64_t t = blockIdx.x; t < P.ntiles; t += gridDim.x, ++it) {
        const uint32_t b = it & 1u;
        double2* tile = tiles + (size_t)b * kTileAmps;
        wait_bar(&bar_tma[b], ph_tma[b]);
        // this thread's 8 amplitudes of its row, and the row exponent
        uint32_t pos[8];
        double2 a[8];
        uint32_t emax = 0;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            pos[i] = mpos[row] | rpos[8u * cg + i];
            a[i] = tile[pos[i]];
            const uint32_t e0 = (uint32_t)((uint64_t)__double_as_longlong(a[i].x) >> 52) & 0x7ffu;
            const uint32_t e1 = (uint32_t)((uint64_t)__double_as_longlong(a[i].y) >> 52) & 0x7ffu;
            emax = max(emax, max(e0, e1));
        }
        s_exp[cg][row] = emax;
        __syncthreads();
        if (s_abort) break;
        const uint32_t E = max(max(s_exp[0][row], s_exp[1][row]), max(s_exp[2][row], s_exp[3][row]));
        // the next tile loads into the other buffer once its last store has read it
        const uint64_t tn = t + gridDim.x;
        if (leader && tn < P.ntiles) {
            bulk_wait_read();
            issue_load(tn, b ^ 1u);
        }
        uint64_t y[16];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            y[2 * i] = slice(a[i].x, E);
            y[2 * i + 1] = slice(a[i].y, E);
        }
        // digits, most significant first, through the two operand slots
#pragma unroll
        for (int s = 0; s < kDigits; ++s) {
            const uint32_t slot = (uint32_t)s & 1u;
            if (s >= 2) {
                wait_bar(&bar_mma[slot], ph_mma[slot]);
                tc_after_sync();
            }
            uint32_t v[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) v[i] = digit_pair(y[2 * i], y[2 * i + 1], 6 - s);
            tmem_st8(tmem + lane_addr + kSlotCol + 32u * slot + 8u * cg, v);
            tmem_st_wait();
            tc_before_sync();
            __syncthreads();
            if (tid == 0 && !s_abort) {
                tc_after_sync();
                const uint32_t a_tm = tmem + kSlotCol + 32u * slot;
                for (int tt = 0; tt + s < kDigits; ++tt) {
                    const uint32_t d_tm = tmem + 64u * (uint32_t)(s + tt);
                    const uint32_t wb = w_addr + (uint32_t)tt * kWDigitBytes;
#pragma unroll
                    for (uint32_t ks = 0; ks < 4; ++ks)
                        mma_f16_ta(d_tm, a_tm + 8u * ks, smem_desc(wb + 256u * ks, 128u, 1024u),
                                   (s > 0 || ks > 0) ? 1u : 0u);
                }
                mma_commit(&bar_mma[slot]);
            }
        }
        // all 28 digit products done (the last commit of each slot)
        wait_bar(&bar_mma[0], ph_mma[0]);
        wait_bar(&bar_mma[1], ph_mma[1]);
        tc_after_sync();
        // read back the seven levels of this thread's 16 output reals and round them to f64
        int32_t hi[16];
        int64_t acc[16];
#pragma unroll
        for (int l = 0; l < kDigits; ++l) {
            uint32_t v[16];
            tmem_ld16(tmem + lane_addr + 64u * (uint32_t)l + 16u * cg, v);
            tmem_ld_wait();
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                const float f = __uint_as_float(v[i]);
                if (l == 0) hi[i] = f2i(f);
                else if (l == 1) hi[i] = hi[i] * 256 + f2i(f);
                else if (l == 2) acc[i] = (int64_t)f2i(f) << 24;
                else if (l == 3) acc[i] += (int64_t)f2i(f) << 16;
                else if (l == 4) acc[i] += (int64_t)f2i(f) << 8;
                else if (l == 5) acc[i] += (int64_t)f2i_even(f);
                else acc[i] += (int64_t)f2i_div256(f);
            }
        }
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int64_t v0 = acc[2 * i] + ((int64_t)hi[2 * i] << 32);
            const int64_t v1 = acc[2 * i + 1] + ((int64_t)hi[2 * i + 1] << 32);
            tile[pos[i]] = make_double2(scaled_to_f64(v0, (int)E + fexp[2 * i] - 2094),
                                        scaled_to_f64(v1, (int)E + fexp[2 * i + 1] - 2094));
        }
        tc_before_sync();
        fence_proxy_async();
        __syncthreads();
        if (s_abort) break;
        if (leader) {
            const uint64_t base = tile_base(t);
            for (uint32_t s = lane; s < nseg; s += 32)
                bulk_store(psi + (base | seg_off[s]), tile + (size_t)s * seg_amps, seg_amps * 16u);
            bulk_commit();
        }
    }
    if (s_abort) {  // let the copies and MMAs in flight finish before the memory goes away
        mbar_wait(&bar_tma[0], ph_tma[0], kWaitLimit);
        mbar_wait(&bar_tma[1], ph_tma[1], kWaitLimit);
        mbar_wait(&bar_mma[0], ph_mma[0], kWaitLimit);
        mbar_wait(&bar_mma[1], ph_mma[1], kWaitLimit);
    }
    if (leader) bulk_wait_all();
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
    if (warp == 0) tmem_dealloc(tmem_base, 512);
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

// A block's weights: the real 64 x 64 form W[2r' + c'][2r + c] = ((Re, -Im), (Im, Re)) of U[r'][r]
// (row = output real, column = input real); per row its largest exponent F, the 53-bit integers
// round(W * 2^(1075 - F)) and their seven balanced base-256 digits as fp16 in the operand layout
// (digit t = 0 most significant), then the 64 row exponents.
void block_weights64(const dense::Block& b, unsigned char* out) {
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
    int32_t* F = reinterpret_cast<int32_t*>(out + kDigits * kWDigitBytes);
    for (uint32_t n = 0; n < 64; ++n) {
        int fmax = 0;
        for (uint32_t k = 0; k < 64; ++k) {
            uint64_t bits;
            memcpy(&bits, &W[n][k], 8);
            fmax = std::max(fmax, (int)((bits >> 52) & 0x7ff));
        }
        F[n] = fmax;
        for (uint32_t k = 0; k < 64; ++k) {
            int64_t X = 0;
            uint64_t bits;
            memcpy(&bits, &W[n][k], 8);
            if (fmax > 0 && ((bits >> 52) & 0x7ff) != 0) X = std::llrint(std::ldexp(W[n][k], 1075 - fmax));
            const uint64_t Y = (uint64_t)X + kBias;
            for (int t = 0; t < kDigits; ++t) {
                const int d = (int)((Y >> (8 * (6 - t))) & 0xffu) - 128;
                dig[(size_t)t * (kWDigitBytes / 2) + w_off16(n, k)] = fp16_of_small_int(d);
            }
        }
    }
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
    dense::make_blocks(lg, L, blocks);
    return dense::make_passes(blocks, L, kTQ, kLowQ, 1, passes);
}

int run_blocks(qvnt_reg* r, const qvnt_gate* gates, size_t count) {
    const uint32_t L = (uint32_t)__builtin_ctzll(r->len);
    std::vector<dense::Block> blocks;
    std::vector<dense::PPlan> passes;
    TRY_T(plan_blocks(gates, count, L, blocks, passes));
    if (passes.empty()) return QVNT_OK;
    const size_t wbytes = blocks.size() * (size_t)kWBlockBytes;
    EngineBuffers& fs = r->bufs;
    if (fs.h_buf) QVNT_CUDA_TRY(cudaStreamSynchronize(r->stream));  // the last upload has left h_buf
    if (fs.d_bytes < wbytes || fs.h_bytes < wbytes) {
        fs.release();
        QVNT_CUDA_TRY(cudaMalloc(&fs.d_buf, wbytes));
        QVNT_CUDA_TRY(cudaMallocHost(&fs.h_buf, wbytes));
        fs.d_bytes = fs.h_bytes = wbytes;
    }
    unsigned char* hw = static_cast<unsigned char*>(fs.h_buf);
    for (size_t i = 0; i < blocks.size(); ++i) block_weights64(blocks[i], hw + i * (size_t)kWBlockBytes);
    QVNT_CUDA_TRY(cudaMemcpyAsync(fs.d_buf, fs.h_buf, wbytes, cudaMemcpyHostToDevice, r->stream));
    static const bool attr = [] {
        return cudaFuncSetAttribute((const void*)tensor64_pass_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)kSmemDyn) == cudaSuccess;
    }();
    if (!attr) return set_error(QVNT_ERR_CUDA, "tensor64 kernel: shared-memory attribute refused");
    int* d_err = reinterpret_cast<int*>(reinterpret_cast<char*>(r->d_small) + 32);
    for (const dense::PPlan& p : passes) {
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
        const uint64_t grid = std::min<uint64_t>((uint64_t)r->ctx->geo.sms, P.ntiles);
        cudaEvent_t stop = nullptr;
        TRY_T(timing_begin(r, &stop));
        tensor64_pass_kernel<<<(unsigned)grid, kNT, kSmemDyn, r->stream>>>(
            r->psi, static_cast<const unsigned char*>(fs.d_buf), P, d_err);
        QVNT_CUDA_TRY(cudaGetLastError());
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

}  // namespace qvnt
