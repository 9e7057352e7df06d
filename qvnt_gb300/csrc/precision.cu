// Precision engine: complex<f32> amplitudes; runs of gates fused into dense 5-qubit blocks (32 x 32
// complex unitaries) contracted on the tcgen05 tensor cores.
//
// The host lowers every qvnt gate to its dense matrix on its support (targets and controls, split
// into one-qubit factors for the multi-bit X/Y/Z/S/T of src/operator/atomic/{x,y,z,s,t}.rs), then
// greedily fuses gates into BLOCKS of at most five qubits (a gate may overtake earlier skipped
// gates only when their supports are disjoint), multiplying their matrices in double precision.
// Blocks are grouped into PASSES: a pass picks 13 tile qubits (12 for a 12-qubit register): the 7
// lowest, so a tile is a set of 1 KB runs, plus the qubits of up to kMaxPB blocks.  Each CTA,
// persistent over tiles, runs two independent pipelines (warp groups), each of which:
//   1. stages its tile (8192 amplitudes, 64 KB) into shared memory with TMA bulk copies;
//   2. per block: threads repack the tile into the MMA operand A (2 x 128 rows = the 8 other tile
//      bits, 64 columns = the block's 32 amplitudes as (re, im)), split into TF32 hi and lo parts and
//      written to tensor memory with tcgen05.st; one thread issues, per 128-row half,
//      D = A_lo W_hi^T + A_hi W_lo^T + A_hi W_hi^T as 24 tcgen05.mma (kind::tf32, M = 128, N = 64,
//      K = 8, A from tensor memory, B from shared memory) into a 128 x 64 FP32 accumulator in tensor
//      memory, where W is the block's unitary as a real 64 x 64 matrix ([[Re, -Im], [Im, Re]]
//      interleaved), kept in shared memory for the whole pass; threads read D back with tcgen05.ld
//      and scatter it into the tile;
//   3. writes the tile back with TMA bulk stores.
// The three-term TF32 split keeps each block product at ~2^-21 relative error with FP32
// accumulation.  Every kRenormEvery passes the state is rescaled in FP64 to the norm it had when
// the apply call started (gates are unitary; this removes FP32 drift and keeps qvnt's unnormalised
// states unnormalised).  Norms, probabilities and measurement run in FP64 (measure.cu).
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "atomic.cuh"
#include "dense_blocks.h"
#include "engine.h"
#include "kernels.h"
#include "tc_ptx.cuh"

#define TRY_LAUNCH(expr)        \
    do {                        \
        const int _s = (expr);  \
        if (_s) return _s;      \
    } while (0)

namespace qvnt {

namespace {

constexpr int kPT = 13;            // tile qubits (at most; 12 for a 12-qubit register)
constexpr int kBQ = dense::kBQ;    // block qubits
constexpr int kBD = dense::kBD;    // block dimension
constexpr int kNT = 512;           // threads: 16 warps, four per tensor-memory lane quadrant
constexpr int kMaxPB = 2;          // blocks per pass (their weights stay in shared memory)
constexpr int kRenormEvery = 10;   // passes between FP64 norm restorations
constexpr uint32_t kPWaitLimit = 1u << 22;
constexpr uint32_t kWFloats = 64 * 64;  // one weight matrix (hi or lo)
constexpr uint32_t kTileAmps = 1u << kPT;
constexpr uint32_t kMaxRows = 1u << (kPT - kBQ);
constexpr size_t kSmemTile = (size_t)kTileAmps * 8, kSmemW = 2 * kWFloats * 4;

// Operand layout of tcgen05 for a K-major matrix without swizzling: core matrices of 8 rows x 16
// bytes (row stride 16 B); the 16 core matrices along K (64 floats) of an 8-row group are contiguous
// (leading-dimension byte offset 128 B), and the groups follow each other (stride 2048 B).
__host__ __device__ constexpr uint32_t op_off(uint32_t row, uint32_t k) {
    return (row >> 3) * 512u + (k >> 2) * 32u + (row & 7u) * 4u + (k & 3u);
}

struct PBlockDesc {
    uint8_t bits[kBQ];  // tile-local bit of block bit j
    uint8_t pad[3];
    uint32_t w_off;     // float offset of the block's weights (hi, then lo) in the weight buffer
};

struct PPassParams {
    uint64_t ntiles;
    uint32_t k, c, nblocks, pad;
    uint32_t tq[kPT];
    PBlockDesc blocks[kMaxPB];
};

// ---- PTX helpers (tc_ptx.cuh) --------------------------------------------------------------------
using namespace tc;
// Bounded wait with this engine's poll limit.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) { return tc::mbar_wait(bar, parity, kPWaitLimit); }
// Operand descriptor: LBO = 128 B, SBO = 2048 B (64 TF32 values per row).
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) { return tc::smem_desc(addr, 128u, 2048u); }

// Instruction descriptor of kind::tf32: FP32 accumulator, A and B TF32 and K-major, N = 64, M = 128.
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((64u >> 3) << 17) | ((128u >> 4) << 24);

// D (+)= A * B^T with A in tensor memory (lane = row, one column per TF32 element) and B in shared
// memory.
__device__ __forceinline__ void mma_tf32_ta(uint32_t d_tmem, uint32_t a_tmem, uint64_t b, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n\t}" ::"r"(d_tmem),
        "r"(a_tmem), "l"(b), "r"(kIdesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ float tf32_rna(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

// One pass.  A tile holds 2^k amplitudes (k = 13, or 12 for a 12-qubit register): 2^(k-5) operand
// rows in halves of 128 (the MMA's M).  The 16 warps form two groups of 8, each an independent
// pipeline over its own tiles (tile buffer, tensor-memory columns 256 g .. + 255, mbarriers, named
// barrier 1 + g), so that one group issues while the other waits on its MMAs, copies or barriers.  Per group, tensor
// memory holds D of both 128-row halves (columns 0..127) and one operand slot, A_hi (128..191) and
// A_lo (192..255), that the halves take in turn: half 1 is repacked once half 0's MMAs are done, and
// half 0 is read back while half 1's MMAs run.
__device__ __forceinline__ void group_sync(uint32_t g) {
    asm volatile("bar.sync %0, 256;" ::"r"(1u + g) : "memory");
}

__global__ void __launch_bounds__(kNT, 1)
    precision_tc_kernel(float2* __restrict__ psi, const float* __restrict__ wts, const __grid_constant__ PPassParams P,
                         int* __restrict__ err) {
    constexpr uint32_t kCols = 512;
    extern __shared__ __align__(1024) unsigned char smem[];
    float2* tiles = reinterpret_cast<float2*>(smem);  // one tile buffer per group
    float* w_sm = reinterpret_cast<float*>(smem + 2 * kSmemTile);
    __shared__ uint64_t seg_off[1 << (kPT - kBQ)];
    __shared__ uint32_t mpos[kMaxPB][kMaxRows];
    __shared__ uint32_t rpos[kMaxPB][kBD];
    __shared__ __align__(8) uint64_t bar_tma[2];
    __shared__ __align__(8) uint64_t bar_mma[2];
    __shared__ uint32_t tmem_base;
    __shared__ int s_abort[2];
    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t g = warp >> 3;                  // pipeline group
    const uint32_t gw = warp & 7u;                 // warp within the group
    const uint32_t k = P.k, c = P.c, nb = P.nblocks;
    const uint32_t nseg = 1u << (k - c);
    const uint32_t seg_amps = 1u << c;
    const uint32_t rows = 1u << (k - kBQ);
    const uint32_t halves = rows >> 7;
    const uint32_t tile_amps = 1u << k;

    for (uint32_t s = tid; s < nseg; s += kNT) {
        uint64_t off = 0;
        for (uint32_t j = 0; j < k - c; ++j)
            if ((s >> j) & 1u) off |= 1ull << P.tq[c + j];
        seg_off[s] = off;
    }
    for (uint32_t b = 0; b < nb; ++b) {
        uint32_t bm = 0;
        for (int j = 0; j < kBQ; ++j) bm |= 1u << P.blocks[b].bits[j];
        if (tid < rows) {
            uint32_t pos = 0, bit = 0;
            for (uint32_t p = 0; p < k; ++p) {
                if ((bm >> p) & 1u) continue;
                if ((tid >> bit) & 1u) pos |= 1u << p;
                ++bit;
            }
            mpos[b][tid] = pos;
        }
        if (tid < (uint32_t)kBD) {
            uint32_t pos = 0;
            for (int j = 0; j < kBQ; ++j)
                if ((tid >> j) & 1u) pos |= 1u << P.blocks[b].bits[j];
            rpos[b][tid] = pos;
        }
        const float4* src = reinterpret_cast<const float4*>(wts + P.blocks[b].w_off);
        float4* dst = reinterpret_cast<float4*>(w_sm + (size_t)b * 2 * kWFloats);
        for (uint32_t i = tid; i < 2 * kWFloats / 4; i += kNT) dst[i] = __ldg(src + i);
    }
    if (warp == 0) {
        tmem_alloc(&tmem_base, kCols);
        tmem_relinquish();
    }
    if (tid == 0) {
        for (int i = 0; i < 2; ++i) {
            mbar_init(&bar_tma[i], 1);
            mbar_init(&bar_mma[i], 1);
            s_abort[i] = 0;
        }
        fence_mbar_init();
    }
    fence_proxy_async();  // the weights written above are read by the tensor cores
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
    const uint32_t tmem = tmem_base + 256u * g;
    const uint32_t lane_base = (32u * (gw & 3u)) << 16;  // this warp's lane quadrant
    const uint32_t grp = gw >> 2;                        // column group: amplitudes 16 grp .. + 15
    float2* tile = tiles + (size_t)g * kTileAmps;
    const bool leader = gw == 0;                         // warp issuing the copies and the MMAs
    uint32_t ph_tma = 0, ph_mma = 0;
    // per half: operand repack, and read-back of the accumulator into the tile
    auto repack = [&](uint32_t b, uint32_t h) {
        const uint32_t m = 128u * h + 32u * (gw & 3u) + lane;
        const uint32_t mp = mpos[b][m];
#pragma unroll
        for (uint32_t half = 0; half < 2; ++half) {
            uint32_t hv[16], lv[16];
#pragma unroll
            for (uint32_t j = 0; j < 8; ++j) {
                const float2 x = tile[mp + rpos[b][16u * grp + 8u * half + j]];
                const float hr = tf32_rna(x.x), hm = tf32_rna(x.y);
                hv[2 * j] = __float_as_uint(hr);
                hv[2 * j + 1] = __float_as_uint(hm);
                lv[2 * j] = __float_as_uint(x.x - hr);
                lv[2 * j + 1] = __float_as_uint(x.y - hm);
            }
            tmem_st16(tmem + lane_base + 128u + 32u * grp + 16u * half, hv);
            tmem_st16(tmem + lane_base + 192u + 32u * grp + 16u * half, lv);
        }
        tmem_st_wait();
    };
    auto readback = [&](uint32_t b, uint32_t h) {
        const uint32_t m = 128u * h + 32u * (gw & 3u) + lane;
        const uint32_t mp = mpos[b][m];
#pragma unroll
        for (uint32_t half = 0; half < 2; ++half) {
            uint32_t v[16];
            tmem_ld16(tmem + lane_base + 64u * h + 32u * grp + 16u * half, v);
            tmem_ld_wait();
#pragma unroll
            for (uint32_t j = 0; j < 8; ++j)
                tile[mp + rpos[b][16u * grp + 8u * half + j]] =
                    make_float2(__uint_as_float(v[2 * j]), __uint_as_float(v[2 * j + 1]));
        }
    };
    auto issue = [&](uint32_t b, uint32_t h) {  // leader lane 0: the half's 24 MMAs and a commit
        tc_after_sync();
        const uint32_t wh = smem_addr(w_sm + (size_t)b * 2 * kWFloats), wl = wh + kWFloats * 4;
        const uint32_t bs[3] = {wh, wl, wh};
        const uint32_t as[3] = {tmem + 192u, tmem + 128u, tmem + 128u};  // lo, hi, hi
        uint32_t acc = 0;
        for (int term = 0; term < 3; ++term)
#pragma unroll
            for (uint32_t ks = 0; ks < 8; ++ks) {
                mma_tf32_ta(tmem + 64u * h, as[term] + ks * 8u, smem_desc(bs[term] + ks * 256u), acc);
                acc = 1;
            }
        mma_commit(&bar_mma[g]);
    };
    auto wait_mma = [&]() {
        if (!mbar_wait(&bar_mma[g], ph_mma)) {
            atomicExch(err, 1);
            s_abort[g] = 1;
        }
        ph_mma ^= 1u;
        tc_after_sync();
    };
    for (uint64_t t = 2ull * blockIdx.x + g; t < P.ntiles; t += 2ull * gridDim.x) {
        uint64_t base = t;
        for (uint32_t p = 0; p < k; ++p) {
            const uint32_t q = P.tq[p];
            base = ((base >> q) << (q + 1)) | (base & ((1ull << q) - 1ull));
        }
        if (leader) {
            if (lane == 0) {
                fence_proxy_async();
                mbar_expect_tx(&bar_tma[g], tile_amps * 8u);
            }
            __syncwarp();
            for (uint32_t s = lane; s < nseg; s += 32)
                bulk_load(tile + (size_t)s * seg_amps, psi + (base | seg_off[s]), seg_amps * 8u, &bar_tma[g]);
        }
        if (!mbar_wait(&bar_tma[g], ph_tma)) {
            atomicExch(err, 1);
            s_abort[g] = 1;
        }
        ph_tma ^= 1u;
        group_sync(g);
        if (s_abort[g]) break;
        for (uint32_t b = 0; b < nb; ++b) {
            repack(b, 0);
            tc_before_sync();
            group_sync(g);
            if (leader && lane == 0) issue(b, 0);
            wait_mma();
            if (halves == 2) {
                repack(b, 1);  // the operand slot is free: half 0's MMAs are done
                tc_before_sync();
                group_sync(g);
                if (leader && lane == 0) issue(b, 1);
                readback(b, 0);  // while half 1's MMAs run
                wait_mma();
                readback(b, 1);
            } else {
                readback(b, 0);
            }
            tc_before_sync();
            group_sync(g);
            if (s_abort[g]) break;
        }
        if (s_abort[g]) break;
        fence_proxy_async();
        group_sync(g);
        if (leader) {
            for (uint32_t s = lane; s < nseg; s += 32)
                bulk_store(psi + (base | seg_off[s]), tile + (size_t)s * seg_amps, seg_amps * 8u);
            bulk_commit();
            bulk_wait_read();  // the tile buffer is reused by the next load
        }
        group_sync(g);
    }
    if (s_abort[g]) {
        mbar_wait(&bar_tma[g], ph_tma);
        mbar_wait(&bar_mma[g], ph_mma);
    }
    if (leader) bulk_wait_all();
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
    if (warp == 0) tmem_dealloc(tmem_base, kCols);
}

// ---- host: dense blocks (dense_blocks.h) and their weights -----------------------------------------
using dense::Block;
using dense::Cd;
using dense::LGate;
using dense::PPlan;

// Lowest qubits every pass keeps in its tile: 2^lowq contiguous amplitudes per TMA copy.  At most
// 12 - 5 = 7, so that a block on five other qubits still fits an empty tile of a 12-qubit register.  Longer runs cost passes
// but make each pass faster (fewer, larger copies with better DRAM locality); measured at 30 qubits,
// depth 60: lowq 5 -> 262 passes of 10.9 ms, 6 -> 310 of 7.7 ms, 7 -> 345 of 6.5 ms.
// QVNT_PRECISION_LOWQ (5..7) overrides the default of 7.
uint32_t precision_lowq() {
    static const uint32_t v = [] {
        const char* e = std::getenv("QVNT_PRECISION_LOWQ");
        const int x = e ? std::atoi(e) : 0;
        return (uint32_t)(x >= 5 && x <= 7 ? x : 7);
    }();
    return v;
}

int make_passes(const std::vector<Block>& blocks, uint32_t L, std::vector<PPlan>& passes) {
    return dense::make_passes(blocks, L, kPT, precision_lowq(), (size_t)kMaxPB, passes);
}

// TF32 rounding to nearest (ties away from zero), as cvt.rna.tf32.f32 does on the device.
float tf32_host(float x) {
    uint32_t u;
    memcpy(&u, &x, 4);
    if ((u & 0x7f800000u) != 0x7f800000u) {
        u += 0x1000u;
        u &= 0xffffe000u;
    }
    float r;
    memcpy(&r, &u, 4);
    return r;
}

// Weights of a block in the operand layout: W[2r' + c'][2r + c] = ((Re, -Im), (Im, Re)) of U[r'][r];
// hi = TF32(W), lo = W - hi.
void block_weights(const Block& b, float* hi, float* lo) {
    for (uint32_t rp = 0; rp < (uint32_t)kBD; ++rp)
        for (uint32_t r = 0; r < (uint32_t)kBD; ++r) {
            const Cd u = b.u[rp * kBD + r];
            const float w[2][2] = {{(float)u.re, (float)-u.im}, {(float)u.im, (float)u.re}};
            for (int cp = 0; cp < 2; ++cp)
                for (int cc = 0; cc < 2; ++cc) {
                    const uint32_t o = op_off(2 * rp + cp, 2 * r + cc);
                    const float h = tf32_host(w[cp][cc]);
                    hi[o] = h;
                    lo[o] = w[cp][cc] - h;
                }
        }
}

}  // namespace

int apply_precision(qvnt_reg* r, const qvnt_gate* gates, size_t count) {
    const uint32_t L = (uint32_t)__builtin_ctzll(r->len);
    if (L < 12) return set_error(QVNT_ERR_UNSUPPORTED, "the precision engine needs at least 12 qubits");
    std::vector<LGate> lg;
    int st = dense::lower_dense(gates, count, lg);
    if (st) return st;
    if (lg.empty()) return QVNT_OK;
    std::vector<Block> blocks;
    dense::make_blocks(lg, L, blocks);
    std::vector<PPlan> passes;
    st = make_passes(blocks, L, passes);
    if (st) return st;
    // weights of every block, uploaded once per apply call
    const size_t wfl = blocks.size() * 2 * kWFloats;
    EngineBuffers& fs = r->bufs;
    TRY_LAUNCH(fs.acquire(wfl * 4, r->stream));
    float* hw = static_cast<float*>(fs.h_buf);
    for (size_t i = 0; i < blocks.size(); ++i) block_weights(blocks[i], hw + i * 2 * kWFloats, hw + i * 2 * kWFloats + kWFloats);
    TRY_LAUNCH(fs.upload(wfl * 4, r->stream));
    // the norm to keep (FP64)
    double* d_norm0 = reinterpret_cast<double*>(r->d_small) + 5;
    double* d_norm = reinterpret_cast<double*>(r->d_small) + 6;
    TRY_LAUNCH(launch_norm_sqr_sum(r->psi, r->fmt, r->len, r->scratch, d_norm0, r->stream));
    static const bool attr = [] {
        return cudaFuncSetAttribute((const void*)precision_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)(2 * kSmemTile + kMaxPB * kSmemW)) == cudaSuccess;
    }();
    if (!attr) return set_error(QVNT_ERR_CUDA, "precision kernel: shared-memory attribute refused");
    int* d_err = reinterpret_cast<int*>(reinterpret_cast<char*>(r->d_small) + 32);
    PPassParams P;
    size_t since = 0;
    for (size_t pi = 0; pi < passes.size(); ++pi) {
        const PPlan& p = passes[pi];
        memset(&P, 0, sizeof P);
        uint32_t n = 0, pos_of[64];
        for (uint32_t b = 0; b < L; ++b)
            if ((p.qmask >> b) & 1ull) {
                pos_of[b] = n;
                P.tq[n++] = b;
            }
        uint32_t run = 0;
        while (run < n && P.tq[run] == run) ++run;
        P.k = n;
        P.c = run;
        P.ntiles = r->len >> n;
        P.nblocks = (uint32_t)p.members.size();
        for (size_t j = 0; j < p.members.size(); ++j) {
            const Block& b = blocks[p.members[j]];
            uint32_t jj = 0;
            for (uint32_t q = 0; q < L; ++q)
                if ((b.sup >> q) & 1ull) P.blocks[j].bits[jj++] = (uint8_t)pos_of[q];
            P.blocks[j].w_off = (uint32_t)(p.members[j] * 2 * kWFloats);
        }
        const size_t smem = 2 * kSmemTile + P.nblocks * kSmemW;
        // one CTA per SM, two tiles at a time (one per pipeline group)
        const uint64_t grid = std::min<uint64_t>((uint64_t)r->ctx->geo.sms, (P.ntiles + 1) / 2);
        cudaEvent_t stop = nullptr;
        st = timing_begin(r, &stop);
        if (st) return st;
        precision_tc_kernel<<<(unsigned)grid, kNT, smem, r->stream>>>(reinterpret_cast<float2*>(r->psi),
                                                                        static_cast<const float*>(fs.d_buf), P, d_err);
        QVNT_CUDA_TRY(cudaGetLastError());
        st = timing_end(r, stop);
        if (st) return st;
        r->launches += 1;
        r->passes += 1;
        if (++since == (size_t)kRenormEvery || pi + 1 == passes.size()) {
            since = 0;
            TRY_LAUNCH(launch_norm_sqr_sum(r->psi, r->fmt, r->len, r->scratch, d_norm, r->stream));
            TRY_LAUNCH(launch_rescale(r->psi, r->fmt, r->len, d_norm0, d_norm, r->stream));
            r->launches += 3;
        }
    }
    return QVNT_OK;
}

int precision_plan_info(const qvnt_gate* gates, size_t count, uint32_t L, uint64_t* passes, uint64_t* blocks) {
    std::vector<LGate> lg;
    int st = dense::lower_dense(gates, count, lg);
    if (st) return st;
    std::vector<Block> bl;
    dense::make_blocks(lg, L, bl);
    std::vector<PPlan> ps;
    st = make_passes(bl, L, ps);
    if (st) return st;
    *passes = ps.size();
    *blocks = bl.size();
    return QVNT_OK;
}

}  // namespace qvnt
