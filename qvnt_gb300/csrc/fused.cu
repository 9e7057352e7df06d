// Fused engine: runs of gates applied to shared-memory tiles, one HBM round trip per pass, in
// double-float arithmetic (df64.cuh) on the FP32 pipes.
//
// qvnt applies every SingleOp as a full sweep over the state (src/operator/multi/mod.rs:97-114).
// Here the host plans PASSES.  A pass picks KT tile qubits Q (12 by default), always containing the
// lowest qubits, so a tile -- the 2^KT amplitudes that share all non-Q index bits -- is a set of
// contiguous runs of at least 512 bytes.  Each CTA (persistent over tiles):
//   1. stages the tile into shared memory with TMA bulk copies (cp.async.bulk, one per run) that
//      complete on an mbarrier (bounded wait, error flag on timeout);
//   2. runs the pass's STAGES: a stage gives every thread 2^KR amplitudes in registers, spanning KR
//      "register qubits" of the tile, applies every gate of the stage there, and writes back;
//   3. writes the tile back with TMA bulk stores.
// A gate joins a pass when its target qubits lie in Q; controls may lie anywhere (outside Q they
// are a per-tile predicate, on thread bits a per-thread predicate) and diagonal gates (Z, S, T, RZ,
// RZZ) join any pass and any stage.  A gate may overtake a deferred gate only when both are diagonal
// or their qubit supports are disjoint, so the result is the in-order product up to rounding.
// Uncontrolled Hadamards run as unscaled butterflies; their 2^(-m/2) is applied once per pass.
// Runs of one-qubit gates on the same qubit (u3 = rz ry rz, rx ry rz, ...) are merged on the host
// into one 2x2 matrix when that costs fewer instructions.
// The pass descriptor (stages, gates, coefficients) is a __grid_constant__ kernel parameter.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "df64.cuh"
#include "engine.h"
#include "kernels.h"

namespace qvnt {

namespace {

constexpr int kMaxKT = 12;   // largest tile (qubits)
constexpr int kMaxKR = 4;    // largest register-qubit count
constexpr int kLowQ = 5;     // lowest qubits always in a tile (512-byte runs)
constexpr int kMaxGates = 192;
constexpr int kMaxStages = 96;
constexpr int kMaxCoef = 4096;
constexpr uint32_t kWaitLimit = 1u << 22;  // bounded mbarrier waits (iterations of try_wait)

// OP_DIAG1: a diagonal gate on ONE qubit (two table entries by that bit); its register bit, or the
// thread / out-of-tile bit it reads, is resolved per stage so that no per-amplitude select is left.
enum : uint8_t { OP_G1 = 1, OP_G2P = 2, OP_G4 = 3, OP_DIAG = 4, OP_DIAG1 = 5 };
// Exact permutation forms are compile-time specialisations: F_SWAPX [[0,1],[1,0]] (X, SWAP),
// F_PY [[0,-i],[i,0]] (Y), F_PI [[0,i],[i,0]] (iSWAP), F_PMI [[0,-i],[-i,0]] (iSWAP dagger);
// F_PERM is any other pair of powers of i.
enum : uint8_t { F_ID = 0, F_PERM = 1, F_RX = 2, F_REAL = 3, F_GEN = 4, F_HADD = 5, F_SWAPX = 6, F_PY = 7,
                 F_PI = 8, F_PMI = 9 };
enum : uint8_t { D_PAR = 0, D_POP = 1 };

struct DGate {
    uint64_t ctrl_out;  // control bits outside the tile (global mask)
    uint64_t dm_out;    // diagonal mask bits outside the tile (global mask)
    uint32_t coef;      // offset into the coefficient pool (floats)
    uint32_t codes;     // exact phase codes: F_PERM (c01 | c10 << 4); diagonal tables (4 bits per entry)
    uint16_t ctrl_thr;  // controls on thread bits (thread-index mask)
    uint16_t dm_thr;    // diagonal mask on thread bits
    uint8_t ctrl_reg;   // controls on register bits (slot mask)
    uint8_t dm_reg;     // diagonal mask on register bits
    uint8_t op, form0, form1, b0, b1, dkind;
    uint8_t exact;      // diagonal: every table entry is a power of i
    uint8_t one0;       // OP_DIAG1: table entry 0 is exactly 1 (nothing to do where the bit is 0)
    uint8_t pad[6];
};
static_assert(sizeof(DGate) == 48, "DGate layout");

struct DStage {
    uint8_t rbit[kMaxKR];   // tile-local bit of register bit b
    uint8_t tbit[kMaxKT];   // tile-local bit of thread bit i
    uint16_t gbegin, gend;
};
static_assert(sizeof(DStage) == 20, "DStage layout");

struct PassParams {
    uint64_t ntiles;
    uint32_t k;         // tile qubits of this pass
    uint32_t c;         // contiguous low run: tile-local bits 0..c-1 are qubits 0..c-1
    uint32_t nthreads;  // 2^(k - KR)
    uint32_t nstages;
    uint32_t tq[kMaxKT];  // global qubit of tile-local bit p (ascending)
    float scale_h, scale_l;  // deferred Hadamard factor 2^(-m/2) as a df pair
    uint32_t has_scale;
    uint32_t pad;
    DStage stages[kMaxStages];
    DGate gates[kMaxGates];
    float coef[kMaxCoef];
};
static_assert(sizeof(PassParams) <= 32760, "pass descriptor must fit the kernel-parameter space");

// ---- TMA / mbarrier helpers (inline PTX) ------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ void tma_load_1d(void* smem_dst, const void* gsrc, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(smem_dst)),
                 "l"(gsrc), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void tma_store_1d(void* gdst, const void* smem_src, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(gdst), "r"(smem_u32(smem_src)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read0() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait0() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// ---- register-level gate application ------------------------------------------------------------
// The gate functions read coefficients through `P.coef`: a PassParams (kernel-parameter space) for
// the single-register kernel, a GCoef (global memory) for the batch kernel.
struct GCoef {
    const float* __restrict__ coef;
};

template <class PP>
__device__ __forceinline__ df cdf(const PP& P, uint32_t o) { return df{P.coef[o], P.coef[o + 1]}; }
__device__ __forceinline__ df cdf(const GCoef& P, uint32_t o) { return df{__ldg(P.coef + o), __ldg(P.coef + o + 1)}; }

// z * i^Q for a compile-time Q: register renames and sign flips only.
template <int Q>
__device__ __forceinline__ dfc rotc(dfc z) {
    if (Q == 1) return dfc{df_neg(z.im), z.re};
    if (Q == 2) return dfc{df_neg(z.re), df_neg(z.im)};
    if (Q == 3) return dfc{z.im, df_neg(z.re)};
    return z;
}

// One 2x2 block on the pair (x0, x1): [y0; y1] = M [x0; x1]; results are left unnormalised.
template <int FORM, class PP>
__device__ __forceinline__ void pair_op(dfc& x0, dfc& x1, const PP& P, uint32_t o, uint32_t codes) {
    if (FORM == F_SWAPX) {
        const dfc t = x0;
        x0 = x1;
        x1 = t;
    } else if (FORM == F_PY || FORM == F_PI || FORM == F_PMI) {
        const dfc n0 = rotc<FORM == F_PI ? 1 : 3>(x1);
        const dfc n1 = rotc<FORM == F_PMI ? 3 : 1>(x0);
        x0 = n0;
        x1 = n1;
    } else if (FORM == F_PERM) {
        const dfc n0 = dfc_rotate(x1, codes & 3u);
        const dfc n1 = dfc_rotate(x0, (codes >> 4) & 3u);
        x0 = n0;
        x1 = n1;
    } else if (FORM == F_HADD) {
        dfc n0, n1;
        n0.re = df_add_raw(x0.re, x1.re);
        n0.im = df_add_raw(x0.im, x1.im);
        n1.re = df_sub_raw(x0.re, x1.re);
        n1.im = df_sub_raw(x0.im, x1.im);
        x0 = n0;
        x1 = n1;
    } else if (FORM == F_RX) {
        // [[a, i b], [i c, d]] with a, b, c, d real
        const df a = cdf(P, o), b = cdf(P, o + 2), c = cdf(P, o + 4), d = cdf(P, o + 6);
        dfc n0, n1;
        n0.re = df_lin2(a, x0.re, df_neg(b), x1.im);
        n0.im = df_lin2(a, x0.im, b, x1.re);
        n1.re = df_lin2(df_neg(c), x0.im, d, x1.re);
        n1.im = df_lin2(c, x0.re, d, x1.im);
        x0 = n0;
        x1 = n1;
    } else if (FORM == F_REAL) {
        const df a = cdf(P, o), b = cdf(P, o + 2), c = cdf(P, o + 4), d = cdf(P, o + 6);
        dfc n0, n1;
        n0.re = df_lin2(a, x0.re, b, x1.re);
        n0.im = df_lin2(a, x0.im, b, x1.im);
        n1.re = df_lin2(c, x0.re, d, x1.re);
        n1.im = df_lin2(c, x0.im, d, x1.im);
        x0 = n0;
        x1 = n1;
    } else if (FORM == F_GEN) {
        const df ar = cdf(P, o), ai = cdf(P, o + 2), br = cdf(P, o + 4), bi = cdf(P, o + 6);
        const df cr = cdf(P, o + 8), ci = cdf(P, o + 10), dr = cdf(P, o + 12), di = cdf(P, o + 14);
        dfc n0, n1;
        n0.re = df_lin4(ar, x0.re, df_neg(ai), x0.im, br, x1.re, df_neg(bi), x1.im);
        n0.im = df_lin4(ar, x0.im, ai, x0.re, br, x1.im, bi, x1.re);
        n1.re = df_lin4(cr, x0.re, df_neg(ci), x0.im, dr, x1.re, df_neg(di), x1.im);
        n1.im = df_lin4(cr, x0.im, ci, x0.re, dr, x1.im, di, x1.re);
        x0 = n0;
        x1 = n1;
    }
}

template <int SLOTS, int B, int FORM, class PP>
__device__ __forceinline__ void g1_form(dfc (&v)[SLOTS], const PP& P, const DGate& G) {
    const uint32_t creg = G.ctrl_reg;
    if (creg == 0) {
#pragma unroll
        for (int j = 0; j < SLOTS; ++j)
            if (!(j & (1 << B))) pair_op<FORM>(v[j], v[j | (1 << B)], P, G.coef, G.codes);
    } else {
#pragma unroll
        for (int j = 0; j < SLOTS; ++j)
            if (!(j & (1 << B)) && (j & creg) == creg) pair_op<FORM>(v[j], v[j | (1 << B)], P, G.coef, G.codes);
    }
}

template <int SLOTS, int B, class PP>
__device__ __forceinline__ void g1(dfc (&v)[SLOTS], const PP& P, const DGate& G) {
    switch (G.form0) {
    case F_SWAPX: g1_form<SLOTS, B, F_SWAPX>(v, P, G); break;
    case F_PY: g1_form<SLOTS, B, F_PY>(v, P, G); break;
    case F_PI: g1_form<SLOTS, B, F_PI>(v, P, G); break;
    case F_PMI: g1_form<SLOTS, B, F_PMI>(v, P, G); break;
    case F_HADD: g1_form<SLOTS, B, F_HADD>(v, P, G); break;
    case F_RX: g1_form<SLOTS, B, F_RX>(v, P, G); break;
    case F_REAL: g1_form<SLOTS, B, F_REAL>(v, P, G); break;
    default: g1_form<SLOTS, B, F_GEN>(v, P, G); break;
    }
}

// Two-qubit gate as 2x2 blocks on the pairs (00, 11) [block A] and (01, 10) [block B] of register
// bits B0 < B1; member order inside a pair: the one with bit B0 clear in A, set in B, first.
template <int SLOTS, int B0, int B1, int FORM, class PP>
__device__ __forceinline__ void g2p_block(dfc (&v)[SLOTS], const PP& P, const DGate& G, bool tok,
                                          bool blockA, uint32_t o, uint32_t codes) {
    constexpr int M0 = 1 << B0, M1 = 1 << B1;
    const uint32_t creg = G.ctrl_reg;
    if (creg == 0) {
#pragma unroll
        for (int j = 0; j < SLOTS; ++j) {
            if (j & (M0 | M1)) continue;
            if (blockA)
                pair_op<FORM>(v[j], v[j | M0 | M1], P, o, codes);
            else
                pair_op<FORM>(v[j | M0], v[j | M1], P, o, codes);
        }
        return;
    }
#pragma unroll
    for (int j = 0; j < SLOTS; ++j) {
        if (j & (M0 | M1)) continue;
        if ((j & creg) != creg) continue;
        if (blockA)
            pair_op<FORM>(v[j], v[j | M0 | M1], P, o, codes);
        else
            pair_op<FORM>(v[j | M0], v[j | M1], P, o, codes);
    }
}

template <int SLOTS, int B0, int B1, class PP>
__device__ __forceinline__ void g2p_any(dfc (&v)[SLOTS], const PP& P, const DGate& G, bool tok, bool blockA) {
    const uint8_t form = blockA ? G.form0 : G.form1;
    const uint32_t o = G.coef + (blockA ? 0u : 16u);
    const uint32_t codes = blockA ? (G.codes & 0xffu) : ((G.codes >> 8) & 0xffu);
    switch (form) {
    case F_ID: break;
    case F_SWAPX: g2p_block<SLOTS, B0, B1, F_SWAPX>(v, P, G, tok, blockA, o, codes); break;
    case F_PI: g2p_block<SLOTS, B0, B1, F_PI>(v, P, G, tok, blockA, o, codes); break;
    case F_PMI: g2p_block<SLOTS, B0, B1, F_PMI>(v, P, G, tok, blockA, o, codes); break;
    case F_RX: g2p_block<SLOTS, B0, B1, F_RX>(v, P, G, tok, blockA, o, codes); break;
    case F_REAL: g2p_block<SLOTS, B0, B1, F_REAL>(v, P, G, tok, blockA, o, codes); break;
    default: g2p_block<SLOTS, B0, B1, F_GEN>(v, P, G, tok, blockA, o, codes); break;
    }
}

template <int SLOTS, int B0, int B1, class PP>
__device__ __forceinline__ void g2p(dfc (&v)[SLOTS], const PP& P, const DGate& G, bool tok) {
    constexpr int M0 = 1 << B0, M1 = 1 << B1;
    if (G.form0 == F_RX && G.form1 == F_RX && G.ctrl_reg == 0) {
        // RXX / RYY: both blocks RX-shaped, one loop, both coefficient sets loaded once
        const uint32_t o = G.coef;
#pragma unroll
        for (int j = 0; j < SLOTS; ++j) {
            if (j & (M0 | M1)) continue;
            pair_op<F_RX>(v[j], v[j | M0 | M1], P, o, 0);
            pair_op<F_RX>(v[j | M0], v[j | M1], P, o + 16, 0);
        }
        return;
    }
    g2p_any<SLOTS, B0, B1>(v, P, G, tok, true);
    g2p_any<SLOTS, B0, B1>(v, P, G, tok, false);
}

// Parity diagonal: table entry parity(idx & mask) of two.  The register part of the mask has NR = 0,
// 1 or 2 bits (B0, B1): their parity per slot is a compile-time constant.  The thread and
// out-of-tile parts give one parity per thread (tpar): slots whose parity equals tpar take entry 0.
template <int SLOTS, int NR, int B0, int B1>
__device__ __forceinline__ int slot_par(int j) {
    return (NR >= 1 ? ((j >> B0) & 1) : 0) ^ (NR >= 2 ? ((j >> B1) & 1) : 0);
}

template <int SLOTS, int NR, int B0, int B1, int PAR, int Q>
__device__ __forceinline__ void rot_par(dfc (&v)[SLOTS], uint32_t creg) {
#pragma unroll
    for (int j = 0; j < SLOTS; ++j)
        if (slot_par<SLOTS, NR, B0, B1>(j) == PAR && (j & creg) == creg) v[j] = rotc<Q>(v[j]);
}

template <int SLOTS, int NR, int B0, int B1, int PAR>
__device__ __forceinline__ void rot_par_code(dfc (&v)[SLOTS], uint32_t creg, uint32_t code) {
    switch (code & 3u) {
    case 1: rot_par<SLOTS, NR, B0, B1, PAR, 1>(v, creg); break;
    case 2: rot_par<SLOTS, NR, B0, B1, PAR, 2>(v, creg); break;
    case 3: rot_par<SLOTS, NR, B0, B1, PAR, 3>(v, creg); break;
    default: break;
    }
}

template <int SLOTS, int NR, int B0, int B1, int PAR>
__device__ __forceinline__ void mul_par(dfc (&v)[SLOTS], uint32_t creg, df cr, df ci) {
    if (creg == 0) {
#pragma unroll
        for (int j = 0; j < SLOTS; ++j)
            if (slot_par<SLOTS, NR, B0, B1>(j) == PAR) v[j] = dfc_mul(cr, ci, v[j]);
        return;
    }
#pragma unroll
    for (int j = 0; j < SLOTS; ++j)
        if (slot_par<SLOTS, NR, B0, B1>(j) == PAR && (j & creg) == creg) v[j] = dfc_mul(cr, ci, v[j]);
}

template <int SLOTS, int NR, int B0, int B1, class PP>
__device__ __forceinline__ void diagp(dfc (&v)[SLOTS], const PP& P, const DGate& G, uint32_t tid,
                                      uint64_t base) {
    const uint32_t creg = G.ctrl_reg;
    const uint32_t tpar = (__popc(tid & G.dm_thr) + __popcll(base & G.dm_out)) & 1u;
    if (G.exact) {
        const uint32_t e0 = G.codes & 3u, e1 = (G.codes >> 4) & 3u;
        rot_par_code<SLOTS, NR, B0, B1, 0>(v, creg, tpar ? e1 : e0);
        rot_par_code<SLOTS, NR, B0, B1, 1>(v, creg, tpar ? e0 : e1);
        return;
    }
    const uint32_t o = G.coef;
    if (G.one0) {
        // entry 0 is 1: only the slots of odd overall parity change
        const df r1 = cdf(P, o + 4), i1 = cdf(P, o + 6);
        if (tpar) mul_par<SLOTS, NR, B0, B1, 0>(v, creg, r1, i1);
        else mul_par<SLOTS, NR, B0, B1, 1>(v, creg, r1, i1);
        return;
    }
    const uint32_t oa = o + (tpar ? 4u : 0u), ob = o + (tpar ? 0u : 4u);
    mul_par<SLOTS, NR, B0, B1, 0>(v, creg, cdf(P, oa), cdf(P, oa + 2));
    mul_par<SLOTS, NR, B0, B1, 1>(v, creg, cdf(P, ob), cdf(P, ob + 2));
}

// Dense 4x4 on register bits B0 < B1; member r = (bit B0) | (bit B1) << 1, row-major complex matrix.
template <int SLOTS, int B0, int B1, class PP>
__device__ __forceinline__ void g4(dfc (&v)[SLOTS], const PP& P, const DGate& G, bool tok) {
    constexpr int M0 = 1 << B0, M1 = 1 << B1;
    const uint32_t creg = G.ctrl_reg;
    const uint32_t o = G.coef;
#pragma unroll
    for (int j = 0; j < SLOTS; ++j) {
        if (j & (M0 | M1)) continue;
        if (!(tok && (j & creg) == creg)) continue;
        const int s[4] = {j, j | M0, j | M1, j | M0 | M1};
        dfc x[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) x[c] = v[s[c]];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            // term-by-term accumulation keeps only the running sums live
            df ar = df_mul_raw(cdf(P, o + 16 * r), x[0].re);
            df ai = df_mul_raw(cdf(P, o + 16 * r), x[0].im);
            {
                const df mi = cdf(P, o + 16 * r + 2);
                ar = df_add_raw(ar, df_mul_raw(df_neg(mi), x[0].im));
                ai = df_add_raw(ai, df_mul_raw(mi, x[0].re));
            }
#pragma unroll
            for (int c = 1; c < 4; ++c) {
                const df mr = cdf(P, o + 16 * r + 4 * c), mi = cdf(P, o + 16 * r + 4 * c + 2);
                ar = df_add_raw(ar, df_mul_raw(mr, x[c].re));
                ar = df_add_raw(ar, df_mul_raw(df_neg(mi), x[c].im));
                ai = df_add_raw(ai, df_mul_raw(mr, x[c].im));
                ai = df_add_raw(ai, df_mul_raw(mi, x[c].re));
            }
            v[s[r]].re = ar;
            v[s[r]].im = ai;
        }
    }
}

template <int SLOTS, class PP>
__device__ __forceinline__ void gdiag(dfc (&v)[SLOTS], const PP& P, const DGate& G, bool tok, uint32_t tid,
                                      uint64_t base) {
    if (!tok) return;
    const uint32_t cnt0 = __popc(tid & G.dm_thr) + __popcll(base & G.dm_out);
    const uint32_t creg = G.ctrl_reg, dreg = G.dm_reg;
    if (G.exact) {
        const uint32_t codes = G.codes;
        const uint32_t idxmask = G.dkind == D_PAR ? 1u : 7u;
#pragma unroll
        for (int j = 0; j < SLOTS; ++j) {
            if ((j & creg) != creg) continue;
            const uint32_t k = (cnt0 + __popc(j & dreg)) & idxmask;
            v[j] = dfc_rotate(v[j], (codes >> (4 * k)) & 3u);
        }
    } else if (G.dkind == D_PAR) {
        const uint32_t o = G.coef;
        const df r0 = cdf(P, o), i0 = cdf(P, o + 2), r1 = cdf(P, o + 4), i1 = cdf(P, o + 6);
#pragma unroll
        for (int j = 0; j < SLOTS; ++j) {
            if ((j & creg) != creg) continue;
            const bool odd = (cnt0 + __popc(j & dreg)) & 1u;
            v[j] = dfc_mul(odd ? r1 : r0, odd ? i1 : i0, v[j]);
        }
    } else {
#pragma unroll
        for (int j = 0; j < SLOTS; ++j) {
            if ((j & creg) != creg) continue;
            const uint32_t o = G.coef + 4u * ((cnt0 + __popc(j & dreg)) & 7u);
            v[j] = dfc_mul(cdf(P, o), cdf(P, o + 2), v[j]);
        }
    }
}

template <int KR, class PP>
__device__ __forceinline__ void apply_gate(dfc (&v)[1 << KR], const PP& P, const DGate& G, uint32_t tid,
                                           uint64_t base) {
    constexpr int S = 1 << KR;
    if ((base & G.ctrl_out) != G.ctrl_out) return;
    if ((tid & G.ctrl_thr) != G.ctrl_thr) return;
    const bool tok = true;
    switch (G.op) {
    case OP_G1:
        switch (G.b0) {
        case 0: g1<S, 0>(v, P, G); break;
        case 1: g1<S, 1>(v, P, G); break;
        case 2: g1<S, 2>(v, P, G); break;
        default:
            if constexpr (KR > 3) g1<S, 3>(v, P, G);
            break;
        }
        break;
    case OP_DIAG1: {
        // parity diagonal with at most two register bits (b0 < b1 when two)
        const int nr = __popc(G.dm_reg);
        if (nr == 0) {
            diagp<S, 0, 0, 0>(v, P, G, tid, base);
        } else if (nr == 1) {
            switch (G.b0) {
            case 0: diagp<S, 1, 0, 0>(v, P, G, tid, base); break;
            case 1: diagp<S, 1, 1, 0>(v, P, G, tid, base); break;
            case 2: diagp<S, 1, 2, 0>(v, P, G, tid, base); break;
            default:
                if constexpr (KR > 3) diagp<S, 1, 3, 0>(v, P, G, tid, base);
                break;
            }
        } else {
            switch (G.b0 * 4 + G.b1) {
            case 1: diagp<S, 2, 0, 1>(v, P, G, tid, base); break;
            case 2: diagp<S, 2, 0, 2>(v, P, G, tid, base); break;
            case 6: diagp<S, 2, 1, 2>(v, P, G, tid, base); break;
            default:
                if constexpr (KR > 3) {
                    switch (G.b0 * 4 + G.b1) {
                    case 3: diagp<S, 2, 0, 3>(v, P, G, tid, base); break;
                    case 7: diagp<S, 2, 1, 3>(v, P, G, tid, base); break;
                    default: diagp<S, 2, 2, 3>(v, P, G, tid, base); break;
                    }
                }
                break;
            }
        }
        break;
    }
    case OP_G2P:
    case OP_G4: {
        const int pr = G.b0 * 4 + G.b1;
        const bool d = G.op == OP_G4;
        switch (pr) {
        case 1: d ? g4<S, 0, 1>(v, P, G, tok) : g2p<S, 0, 1>(v, P, G, tok); break;
        case 2: d ? g4<S, 0, 2>(v, P, G, tok) : g2p<S, 0, 2>(v, P, G, tok); break;
        case 6: d ? g4<S, 1, 2>(v, P, G, tok) : g2p<S, 1, 2>(v, P, G, tok); break;
        default:
            if constexpr (KR > 3) {
                switch (pr) {
                case 3: d ? g4<S, 0, 3>(v, P, G, tok) : g2p<S, 0, 3>(v, P, G, tok); break;
                case 7: d ? g4<S, 1, 3>(v, P, G, tok) : g2p<S, 1, 3>(v, P, G, tok); break;
                default: d ? g4<S, 2, 3>(v, P, G, tok) : g2p<S, 2, 3>(v, P, G, tok); break;
                }
            }
            break;
        }
        break;
    }
    default:
        gdiag<S>(v, P, G, tok, tid, base);
        break;
    }
}

template <int KT, int KR, int MINB>
__global__ void __launch_bounds__(1 << (KT - KR), MINB)
    fused_df_kernel(float4* __restrict__ psi, const __grid_constant__ PassParams P, int* __restrict__ err) {
    constexpr int SLOTS = 1 << KR;
    constexpr int NTB = KT - KR;  // thread bits
    extern __shared__ __align__(128) float4 tile[];
    __shared__ uint64_t seg_off[1 << (kMaxKT - kLowQ)];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ int s_abort;
    const uint32_t tid = threadIdx.x;
    const uint32_t nthr = P.nthreads;
    const uint32_t nseg = 1u << (P.k - P.c);
    const uint32_t seg_amps = 1u << P.c;
    const uint32_t lanes = nthr < 32 ? nthr : 32;
    for (uint32_t s = tid; s < nseg; s += nthr) {
        uint64_t off = 0;
        for (uint32_t j = 0; j < P.k - P.c; ++j)
            if ((s >> j) & 1u) off |= 1ull << P.tq[P.c + j];
        seg_off[s] = off;
    }
    if (tid == 0) {
        mbar_init(&mbar, 1);
        fence_mbar_init();
        s_abort = 0;
    }
    __syncthreads();
    const df scale{P.scale_h, P.scale_l};
    uint32_t phase = 0;
    for (uint64_t t = blockIdx.x; t < P.ntiles; t += gridDim.x) {
        // tile base: tile index with zeros inserted at the tile qubits
        uint64_t base = t;
        for (uint32_t p = 0; p < P.k; ++p) {
            const uint32_t q = P.tq[p];
            base = ((base >> q) << (q + 1)) | (base & ((1ull << q) - 1ull));
        }
        if (tid < lanes) {
            if (tid == 0) {
                fence_proxy_async();
                mbar_arrive_expect_tx(&mbar, (1u << P.k) * 16u);
            }
            __syncwarp(lanes == 32 ? 0xffffffffu : ((1u << lanes) - 1u));
            for (uint32_t s = tid; s < nseg; s += lanes)
                tma_load_1d(tile + (size_t)s * seg_amps, psi + (base | seg_off[s]), seg_amps * 16u, &mbar);
        }
        uint32_t it = 0;
        while (!mbar_try_wait(&mbar, phase)) {
            if (++it >= kWaitLimit) {
                atomicExch(err, 1);
                s_abort = 1;
                break;
            }
        }
        phase ^= 1u;
        __syncthreads();
        if (s_abort) {
            // the copies may still land: wait for them (bounded) before leaving
            uint32_t it2 = 0;
            while (!mbar_try_wait(&mbar, phase ^ 1u) && ++it2 < kWaitLimit) {
            }
            return;
        }
        for (uint32_t si = 0; si < P.nstages; ++si) {
            const DStage& S = P.stages[si];
            uint32_t tl = 0;
#pragma unroll
            for (int i = 0; i < NTB; ++i)
                if (i < (int)(P.k - KR) && ((tid >> i) & 1u)) tl |= 1u << S.tbit[i];
            uint32_t roff[KR];
#pragma unroll
            for (int b = 0; b < KR; ++b) roff[b] = 1u << S.rbit[b];
            dfc v[SLOTS];
#pragma unroll
            for (int j = 0; j < SLOTS; ++j) {
                uint32_t l = tl;
#pragma unroll
                for (int b = 0; b < KR; ++b)
                    if (j & (1 << b)) l += roff[b];
                const float4 a = tile[l];
                v[j].re = df{a.x, a.y};
                v[j].im = df{a.z, a.w};
            }
            for (uint32_t gi = S.gbegin; gi < S.gend; ++gi) apply_gate<KR>(v, P, P.gates[gi], tid, base);
            // Intermediate stages hand unnormalised pairs to the next stage; the pass's last stage
            // applies the deferred Hadamard scale and renormalises before the tile goes to HBM.
            const bool last = si + 1 == P.nstages;
            if (last) {
                const bool scaled = P.has_scale != 0;
#pragma unroll
                for (int j = 0; j < SLOTS; ++j) {
                    uint32_t l = tl;
#pragma unroll
                    for (int b = 0; b < KR; ++b)
                        if (j & (1 << b)) l += roff[b];
                    df re = v[j].re, im = v[j].im;
                    if (scaled) {
                        re = df_mul_raw(scale, re);
                        im = df_mul_raw(scale, im);
                    }
                    re = df_renorm(re);
                    im = df_renorm(im);
                    tile[l] = make_float4(re.h, re.l, im.h, im.l);
                }
            } else {
#pragma unroll
                for (int j = 0; j < SLOTS; ++j) {
                    uint32_t l = tl;
#pragma unroll
                    for (int b = 0; b < KR; ++b)
                        if (j & (1 << b)) l += roff[b];
                    tile[l] = make_float4(v[j].re.h, v[j].re.l, v[j].im.h, v[j].im.l);
                }
            }
            __syncthreads();
        }
        fence_proxy_async();
        __syncthreads();
        if (tid < lanes) {
            for (uint32_t s = tid; s < nseg; s += lanes)
                tma_store_1d(psi + (base | seg_off[s]), tile + (size_t)s * seg_amps, seg_amps * 16u);
            bulk_commit();
            bulk_wait_read0();
        }
        __syncthreads();
    }
    if (tid < lanes) bulk_wait0();
}

// ---- batch kernel: many registers, one persistent launch ------------------------------------------
// The schedule is a queue of ITEMS (one tile of one pass of one register, or one register's
// measurement) in wave order: every register's pass p comes before any register's pass p + 1.  A CTA
// takes the next item with an atomic counter and, before it starts, waits until its register has
// completed `need` items (all tiles of the previous pass).  Those items were taken earlier by CTAs that
// are running, so every wait ends; it is bounded all the same (error flag, then the item is skipped).
// Descriptors live in global memory; states are double-float (float4 per amplitude) like the
// single-register fused engine, read and written with L2-coherent loads and stores.
constexpr uint32_t kMeasureItem = 0xffffffffu;
constexpr uint32_t kBatchWaitLimit = 1u << 22;  // iterations of a 256 ns back-off: about a second

struct BPass {
    uint64_t ntiles;
    uint32_t k, c, nthreads, nstages;
    uint32_t tq[kMaxKT];
    float scale_h, scale_l;
    uint32_t has_scale;
    uint32_t stage0, gate0, coef0;  // offsets into the schedule's stage, gate and coefficient arrays
};

struct BEntry {           // one pass (or the measurement) of one register
    uint64_t psi_off;     // float4 offset of the register's state in the arena
    uint64_t len;         // amplitudes of the register
    uint64_t mask;        // measure: mask
    double u01;           // measure: uniform draw
    uint32_t pass;        // index into the pass array, or kMeasureItem
    uint32_t reg;         // register index
    uint32_t need;        // completed items of the register required before this one starts
    uint32_t pad;
};

struct BItem {
    uint32_t entry;
    uint32_t tile;
};

struct BatchArgs {
    float4* psi;
    const BItem* items;
    uint64_t nitems;
    const BEntry* entries;
    const BPass* passes;
    const DStage* stages;
    const DGate* gates;
    const float* coef;
    const double* u01;  // per register, overrides BEntry::u01 when set
    unsigned int* done;
    unsigned long long* next;
    unsigned long long* results;
    int* err;
};

__device__ __forceinline__ unsigned int ld_acquire_u32(const unsigned int* p) {
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ double amp_nsq(float4 a) {
    const double re = df_to_double(df{a.x, a.y}), im = df_to_double(df{a.z, a.w});
    return re * re + im * im;
}

// Inclusive scan of one double per thread over a block of NT threads, in thread order.
template <int NT>
__device__ __forceinline__ double batch_block_scan(double v, double* sm, double* total) {
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const double u = __shfl_up_sync(0xffffffffu, v, o);
        if (l >= o) v += u;
    }
    __syncthreads();
    if (l == 31) sm[w] = v;
    __syncthreads();
    if (w == 0) {
        double s = (l < NT / 32) ? sm[l] : 0.0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const double u = __shfl_up_sync(0xffffffffu, s, o);
            if (l >= o) s += u;
        }
        if (l < NT / 32) sm[l] = s;
    }
    __syncthreads();
    if (w > 0) v += sm[w - 1];
    *total = sm[NT / 32 - 1];
    __syncthreads();
    return v;
}

// measure_mask of one register by one CTA (src/register/quant.rs:468-501): weights |psi_i|^2 / sum,
// WeightedIndex selection (first i with inclusive cumulative weight > u01 * total, else the last
// index), collapse without renormalisation, result idx & mask.  Thread t owns the contiguous index
// range [t * per, (t + 1) * per), so the cumulative order is the index order.
template <int NT>
__device__ void batch_measure(const BatchArgs& A, const BEntry& E, double u01) {
    __shared__ double sm[32];
    __shared__ double s_last[NT / 32];
    __shared__ unsigned long long s_idx;
    const uint32_t t = threadIdx.x;
    float4* psi = A.psi + E.psi_off;
    const uint64_t per = (E.len + NT - 1) / NT;
    const uint64_t i0 = min((uint64_t)t * per, E.len), i1 = min(i0 + per, E.len);
    double s = 0.0;
    for (uint64_t i = i0; i < i1; ++i) s += amp_nsq(__ldcg(psi + i));
    double total;
    batch_block_scan<NT>(s, sm, &total);
    const double inv = 1. / total;
    if (t == 0 && (!(total > 0.0) || !isfinite(inv))) atomicExch(A.err, QVNT_ERR_BAD_ARG);
    double p = 0.0;
    for (uint64_t i = i0; i < i1; ++i) p += amp_nsq(__ldcg(psi + i)) * inv;
    double ptotal;
    const double incl = batch_block_scan<NT>(p, sm, &ptotal);
    const double chosen = u01 * ptotal;
    // exclusive prefix of each thread = inclusive prefix of the thread before it
    const double prev = __shfl_up_sync(0xffffffffu, incl, 1);
    if ((t & 31) == 31) s_last[t >> 5] = incl;
    if (t == 0) s_idx = E.len - 1;
    __syncthreads();
    const double before = (t & 31) ? prev : (t >= 32 ? s_last[(t >> 5) - 1] : 0.0);
    // the thread whose range crosses `chosen` walks it in index order
    if (i0 < i1 && incl > chosen && !(before > chosen)) {
        double run = before;
        uint64_t pick = i1 - 1;
        for (uint64_t i = i0; i < i1; ++i) {
            run += amp_nsq(__ldcg(psi + i)) * inv;
            if (run > chosen) {
                pick = i;
                break;
            }
        }
        atomicMin(&s_idx, (unsigned long long)pick);
    }
    __syncthreads();
    const uint64_t idx = s_idx;
    for (uint64_t i = t; i < E.len; i += NT)
        if ((i ^ idx) & E.mask) __stcg(psi + i, make_float4(0.f, 0.f, 0.f, 0.f));
    if (t == 0) A.results[E.reg] = idx & E.mask;
}

template <int KT, int KR, int MINB>
__global__ void __launch_bounds__(1 << (KT - KR), MINB) batch_df_kernel(const __grid_constant__ BatchArgs A) {
    constexpr int SLOTS = 1 << KR;
    constexpr int NT = 1 << (KT - KR);
    extern __shared__ __align__(128) float4 tile[];
    __shared__ uint64_t seg_off[1 << (kMaxKT - kLowQ)];
    __shared__ unsigned long long s_item;
    __shared__ int s_skip;
    const uint32_t tid = threadIdx.x;
    while (true) {
        if (tid == 0) s_item = atomicAdd(A.next, 1ull);
        __syncthreads();
        const unsigned long long it = s_item;
        if (it >= A.nitems) break;
        const BItem item = A.items[it];
        const BEntry E = A.entries[item.entry];
        if (tid == 0) {
            int skip = 0;
            uint32_t n = 0;
            while (ld_acquire_u32(A.done + E.reg) < E.need) {
                if (++n >= kBatchWaitLimit) {
                    atomicExch(A.err, QVNT_ERR_TIMEOUT);
                    skip = 1;
                    break;
                }
                __nanosleep(256);
            }
            s_skip = skip;
        }
        __syncthreads();
        if (!s_skip) {
            if (E.pass == kMeasureItem) {
                batch_measure<NT>(A, E, A.u01 ? A.u01[E.reg] : E.u01);
            } else {
                const BPass& P = A.passes[E.pass];
                const uint32_t k = P.k, c = P.c, nthr = P.nthreads, nstages = P.nstages;
                const uint32_t nseg = 1u << (k - c);
                const uint32_t seg_mask = (1u << c) - 1u;
                for (uint32_t s = tid; s < nseg; s += NT) {
                    uint64_t off = 0;
                    for (uint32_t j = 0; j < k - c; ++j)
                        if ((s >> j) & 1u) off |= 1ull << P.tq[c + j];
                    seg_off[s] = off;
                }
                uint64_t base = item.tile;
                for (uint32_t p = 0; p < k; ++p) {
                    const uint32_t q = P.tq[p];
                    base = ((base >> q) << (q + 1)) | (base & ((1ull << q) - 1ull));
                }
                __syncthreads();
                float4* psi = A.psi + E.psi_off;
                for (uint32_t i = tid; i < (1u << k); i += NT)
                    tile[i] = __ldcg(psi + (base | seg_off[i >> c] | (i & seg_mask)));
                __syncthreads();
                const GCoef C{A.coef + P.coef0};
                const df scale{P.scale_h, P.scale_l};
                const bool scaled = P.has_scale != 0;
                for (uint32_t si = 0; si < nstages; ++si) {
                    if (tid < nthr) {
                        const DStage S = A.stages[P.stage0 + si];
                        uint32_t tl = 0;
#pragma unroll
                        for (int i = 0; i < KT - KR; ++i)
                            if (i < (int)(k - KR) && ((tid >> i) & 1u)) tl |= 1u << S.tbit[i];
                        uint32_t roff[KR];
#pragma unroll
                        for (int b = 0; b < KR; ++b) roff[b] = 1u << S.rbit[b];
                        dfc v[SLOTS];
#pragma unroll
                        for (int j = 0; j < SLOTS; ++j) {
                            uint32_t l = tl;
#pragma unroll
                            for (int b = 0; b < KR; ++b)
                                if (j & (1 << b)) l += roff[b];
                            const float4 a = tile[l];
                            v[j].re = df{a.x, a.y};
                            v[j].im = df{a.z, a.w};
                        }
                        for (uint32_t gi = S.gbegin; gi < S.gend; ++gi) {
                            const DGate G = A.gates[P.gate0 + gi];
                            apply_gate<KR>(v, C, G, tid, base);
                        }
                        const bool last = si + 1 == nstages;
#pragma unroll
                        for (int j = 0; j < SLOTS; ++j) {
                            uint32_t l = tl;
#pragma unroll
                            for (int b = 0; b < KR; ++b)
                                if (j & (1 << b)) l += roff[b];
                            df re = v[j].re, im = v[j].im;
                            if (last) {
                                if (scaled) {
                                    re = df_mul_raw(scale, re);
                                    im = df_mul_raw(scale, im);
                                }
                                re = df_renorm(re);
                                im = df_renorm(im);
                            }
                            tile[l] = make_float4(re.h, re.l, im.h, im.l);
                        }
                    }
                    __syncthreads();
                }
                for (uint32_t i = tid; i < (1u << k); i += NT)
                    __stcg(psi + (base | seg_off[i >> c] | (i & seg_mask)), tile[i]);
            }
        }
        __syncthreads();
        if (tid == 0) {
            __threadfence();
            atomicAdd(A.done + E.reg, 1u);
        }
    }
}

// Two register budgets of the batch kernel: 2 CTAs per SM (128 registers, some spills) or 1 CTA per
// SM (no spills, half the warps); the autotuner picks one per batch.
constexpr int kBatchKT = 12, kBatchKR = 4, kBatchMinB = 2;

// ---- kernel configurations ----------------------------------------------------------------------
using KernelFn = void (*)(float4*, PassParams, int*);

struct KCfg {
    int kt, kr, minb;
    KernelFn fn;
};

// The shape of the single-register kernel: 12-qubit tiles (64 KB), 256 threads x 16 amplitudes over 4
// register qubits, 2 CTAs per SM.  Measured on the 30-qubit random circuit against 11-qubit tiles,
// 8 amplitudes per thread, 512-thread CTAs and 1 or 3 CTAs per SM, this shape was the fastest.
const KCfg kCfgs[] = {
    {12, 4, 2, fused_df_kernel<12, 4, 2>},
};

void launch_cfg(size_t, unsigned grid, unsigned block, size_t smem, cudaStream_t s, float4* psi, const PassParams& P,
                int* err) {
    fused_df_kernel<12, 4, 2><<<grid, block, smem, s>>>(psi, P, err);
}

const KCfg& active_cfg() { return kCfgs[0]; }

// ---- host: lowering qvnt gates to engine gates ----------------------------------------------------
struct C2 {
    double re, im;
};

C2 cmul(C2 a, C2 b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
C2 cadd(C2 a, C2 b) { return {a.re + b.re, a.im + b.im}; }

struct EGate {
    uint8_t op = 0;
    uint8_t form0 = F_ID, form1 = F_ID;
    uint8_t dkind = D_PAR;
    bool exact = false;
    bool hadd = false;    // unscaled Hadamard butterfly: contributes 1/sqrt(2) to the pass scale
    bool one0 = false;    // diagonal: table entry 0 is exactly 1
    bool has_m2 = false;  // one-qubit gate with its 2x2 matrix in m2 (mergeable)
    int q0 = -1, q1 = -1;  // target qubits (q0 < q1 for two-qubit ops)
    uint64_t ctrl = 0;
    uint64_t dmask = 0;
    uint32_t codes = 0;
    C2 m2[4];
    std::vector<float> coef;  // df64 pairs
    int cost = 0;             // FP32 instructions per amplitude (estimate)
    bool standalone = false;
    size_t src = 0;
};

void push_df(std::vector<float>& out, double x) {
    const float h = (float)x;
    out.push_back(h);
    out.push_back((float)(x - (double)h));
}

inline unsigned popc(uint64_t x) { return (unsigned)__builtin_popcountll(x); }

const C2 kI4[4] = {{1, 0}, {0, 1}, {-1, 0}, {0, -1}};  // i^k

// i^code for the exact phases.
int exact_code(C2 z) {
    for (int k = 0; k < 4; ++k)
        if (z.re == kI4[k].re && z.im == kI4[k].im) return k;
    return -1;
}

int form_cost(uint8_t f) {
    switch (f) {
    case F_ID: return 0;
    case F_SWAPX: return 1;
    case F_PY: case F_PI: case F_PMI: return 3;
    case F_PERM: return 6;
    case F_HADD: return 18;
    case F_RX: case F_REAL: return 36;
    default: return 76;
    }
}

EGate diag_gate(uint64_t mask, uint64_t ctrl, const std::vector<C2>& table, uint8_t dkind) {
    EGate e;
    e.op = OP_DIAG;
    e.dmask = mask;
    e.ctrl = ctrl;
    e.dkind = dkind;
    bool exact = true;
    uint32_t codes = 0;
    for (size_t k = 0; k < table.size(); ++k) {
        const int c = exact_code(table[k]);
        if (c < 0) exact = false;
        else codes |= (uint32_t)c << (4 * k);
    }
    e.exact = exact;
    e.codes = codes;
    if (!exact)
        for (const C2& z : table) {
            push_df(e.coef, z.re);
            push_df(e.coef, z.im);
        }
    const bool one0 = table[0].re == 1.0 && table[0].im == 0.0;
    e.one0 = one0;
    if (popc(mask) == 1 && dkind == D_PAR) e.cost = exact ? 3 : (one0 ? 18 : 34);
    else e.cost = exact ? 8 : 38;
    if (popc(mask) == 1 && dkind == D_PAR) {
        e.has_m2 = true;
        e.q0 = __builtin_ctzll(mask);
        e.m2[0] = table[0];
        e.m2[1] = {0, 0};
        e.m2[2] = {0, 0};
        e.m2[3] = table[1];
    }
    return e;
}

// One-qubit gate with the given 2x2 matrix, in the cheapest form that represents it.
EGate g1_matrix(int q, uint64_t ctrl, const C2* m) {
    EGate e;
    e.op = OP_G1;
    e.q0 = q;
    e.ctrl = ctrl;
    e.has_m2 = true;
    for (int k = 0; k < 4; ++k) e.m2[k] = m[k];
    const bool real = m[0].im == 0 && m[1].im == 0 && m[2].im == 0 && m[3].im == 0;
    const bool rx = m[0].im == 0 && m[3].im == 0 && m[1].re == 0 && m[2].re == 0;
    const int c01 = exact_code(m[1]), c10 = exact_code(m[2]);
    const bool anti = m[0].re == 0 && m[0].im == 0 && m[3].re == 0 && m[3].im == 0;
    // exact anti-diagonal forms: [[0,1],[1,0]], [[0,-i],[i,0]], [[0,i],[i,0]], [[0,-i],[-i,0]]
    uint8_t perm_form = F_ID;
    if (anti && c01 == 0 && c10 == 0) perm_form = F_SWAPX;
    else if (anti && c01 == 3 && c10 == 1) perm_form = F_PY;
    else if (anti && c01 == 1 && c10 == 1) perm_form = F_PI;
    else if (anti && c01 == 3 && c10 == 3) perm_form = F_PMI;
    if (perm_form != F_ID) {
        e.form0 = perm_form;
        e.codes = (uint32_t)c01 | ((uint32_t)c10 << 4);
    } else if (real) {
        e.form0 = F_REAL;
        push_df(e.coef, m[0].re);
        push_df(e.coef, m[1].re);
        push_df(e.coef, m[2].re);
        push_df(e.coef, m[3].re);
    } else if (rx) {
        e.form0 = F_RX;
        push_df(e.coef, m[0].re);
        push_df(e.coef, m[1].im);
        push_df(e.coef, m[2].im);
        push_df(e.coef, m[3].re);
    } else {
        e.form0 = F_GEN;
        for (int k = 0; k < 4; ++k) {
            push_df(e.coef, m[k].re);
            push_df(e.coef, m[k].im);
        }
    }
    e.cost = form_cost(e.form0);
    return e;
}

EGate g1_hadd(int q) {
    EGate e;
    e.op = OP_G1;
    e.q0 = q;
    e.form0 = F_HADD;
    e.hadd = true;
    e.cost = form_cost(F_HADD);
    return e;
}

void push_block(EGate& e, uint8_t form, const C2* m) {  // m: row-major 2x2
    if (form == F_RX || form == F_REAL) {
        const double a = m[0].re, d = m[3].re;
        const double b = form == F_RX ? m[1].im : m[1].re, c = form == F_RX ? m[2].im : m[2].re;
        push_df(e.coef, a);
        push_df(e.coef, b);
        push_df(e.coef, c);
        push_df(e.coef, d);
        for (int k = 0; k < 8; ++k) e.coef.push_back(0.f);  // blocks are 16 floats apart
    } else {
        for (int k = 0; k < 4; ++k) {
            push_df(e.coef, m ? m[k].re : 0.0);
            push_df(e.coef, m ? m[k].im : 0.0);
        }
    }
}

// Two-qubit gate as blocks on (00, 11) and (01, 10).
EGate g2p_gate(uint64_t ab, uint64_t ctrl, uint8_t fa, const C2* ma, uint32_t codes_a, uint8_t fb, const C2* mb,
               uint32_t codes_b) {
    EGate e;
    e.op = OP_G2P;
    e.q0 = __builtin_ctzll(ab);
    e.q1 = 63 - __builtin_clzll(ab);
    e.ctrl = ctrl;
    e.form0 = fa;
    e.form1 = fb;
    e.codes = codes_a | (codes_b << 8);
    push_block(e, fa == F_RX || fa == F_REAL || fa == F_GEN ? fa : F_GEN, fa == F_RX || fa == F_REAL || fa == F_GEN ? ma : nullptr);
    push_block(e, fb == F_RX || fb == F_REAL || fb == F_GEN ? fb : F_GEN, fb == F_RX || fb == F_REAL || fb == F_GEN ? mb : nullptr);
    e.cost = (form_cost(fa) + form_cost(fb) + 1) / 2 + 2;
    return e;
}

// Lowers one validated qvnt gate (the atomic formulas of src/operator/atomic/*.rs written as the
// matrices they apply) to engine gates.
void lower(const qvnt_gate& g, size_t src, std::vector<EGate>& out) {
    const uint64_t a = g.a_mask, ctrl = g.ctrl;
    const double c = g.phase[0], s = g.phase[1];
    const double r = 0.70710678118654752440084436210484903;
    auto each_bit = [&](uint64_t m, auto&& f) {
        for (int q = 0; q < 64; ++q)
            if ((m >> q) & 1ull) f(q);
    };
    switch (g.kind) {
    case QVNT_GATE_ID:
        return;
    case QVNT_GATE_X: {  // x.rs: a product of single-bit flips (exact)
        const C2 m[4] = {{0, 0}, {1, 0}, {1, 0}, {0, 0}};
        each_bit(a, [&](int q) { out.push_back(g1_matrix(q, ctrl, m)); });
        return;
    }
    case QVNT_GATE_Y: {  // y.rs: Y(mask) = tensor product of single-qubit Y = [[0, -i], [i, 0]] (exact)
        const C2 m[4] = {{0, 0}, {0, -1}, {0, 1}, {0, 0}};
        each_bit(a, [&](int q) { out.push_back(g1_matrix(q, ctrl, m)); });
        return;
    }
    case QVNT_GATE_Z:  // z.rs: sign by parity
        if (a) out.push_back(diag_gate(a, ctrl, {{1, 0}, {-1, 0}}, D_PAR));
        return;
    case QVNT_GATE_S: {  // s.rs: i^popcount (dagger: i^-popcount) = product of i^bit over the mask
        const C2 ph = g.dagger ? C2{0, -1} : C2{0, 1};
        each_bit(a, [&](int q) { out.push_back(diag_gate(1ull << q, ctrl, {{1, 0}, ph}, D_PAR)); });
        return;
    }
    case QVNT_GATE_T: {  // t.rs: e^{i pi/4 popcount} (dagger: e^{-i pi/4 popcount}) = product over the bits
        const C2 ph = g.dagger ? C2{r, -r} : C2{r, r};
        each_bit(a, [&](int q) { out.push_back(diag_gate(1ull << q, ctrl, {{1, 0}, ph}, D_PAR)); });
        return;
    }
    case QVNT_GATE_RZ:   // rz.rs: (c, -s) where the bit is 0, (c, s) where it is 1
    case QVNT_GATE_RZZ:  // rzz.rs: (c, -s) for even parity, (c, s) for odd
        out.push_back(diag_gate(a, ctrl, {{c, -s}, {c, s}}, D_PAR));
        return;
    case QVNT_GATE_RX: {  // rx.rs: c p0 - i s p1
        const C2 m[4] = {{c, 0}, {0, -s}, {0, -s}, {c, 0}};
        out.push_back(g1_matrix(__builtin_ctzll(a), ctrl, m));
        return;
    }
    case QVNT_GATE_RY: {  // ry.rs: [[c, -s], [s, c]]
        const C2 m[4] = {{c, 0}, {-s, 0}, {s, 0}, {c, 0}};
        out.push_back(g1_matrix(__builtin_ctzll(a), ctrl, m));
        return;
    }
    case QVNT_GATE_H1:  // h1.rs
    case QVNT_GATE_H2: {  // h2.rs = H on each of the two qubits
        const C2 m[4] = {{r, 0}, {r, 0}, {r, 0}, {-r, 0}};
        const uint64_t bits = g.kind == QVNT_GATE_H2 ? (g.a_mask | g.b_mask) : a;
        each_bit(bits, [&](int q) { out.push_back(ctrl ? g1_matrix(q, ctrl, m) : g1_hadd(q)); });
        return;
    }
    case QVNT_GATE_U1: {  // u1.rs: dense 2x2
        const C2 m[4] = {{g.matrix[0], g.matrix[1]}, {g.matrix[2], g.matrix[3]},
                         {g.matrix[4], g.matrix[5]}, {g.matrix[6], g.matrix[7]}};
        out.push_back(g1_matrix(__builtin_ctzll(a), ctrl, m));
        return;
    }
    case QVNT_GATE_RXX: {  // rxx.rs: c p - i s p(partner) on both pairs
        const C2 m[4] = {{c, 0}, {0, -s}, {0, -s}, {c, 0}};
        out.push_back(g2p_gate(a, ctrl, F_RX, m, 0, F_RX, m, 0));
        return;
    }
    case QVNT_GATE_RYY: {  // ryy.rs: c p - i pi p(partner), pi = -s on (00, 11), +s on (01, 10)
        const C2 ma[4] = {{c, 0}, {0, s}, {0, s}, {c, 0}};
        const C2 mb[4] = {{c, 0}, {0, -s}, {0, -s}, {c, 0}};
        out.push_back(g2p_gate(a, ctrl, F_RX, ma, 0, F_RX, mb, 0));
        return;
    }
    case QVNT_GATE_SWAP:  // swap.rs
        out.push_back(g2p_gate(a, ctrl, F_ID, nullptr, 0, F_SWAPX, nullptr, 0));
        return;
    case QVNT_GATE_ISWAP: {  // i_swap.rs: i p(partner) (dagger: -i)
        const uint32_t code = g.dagger ? 3u : 1u;
        out.push_back(g2p_gate(a, ctrl, F_ID, nullptr, 0, g.dagger ? F_PMI : F_PI, nullptr, code | (code << 4)));
        return;
    }
    case QVNT_GATE_SQRT_SWAP: {  // sqrt_swap.rs: 0.5(1+i) p + 0.5(1-i) p(partner) (dagger: conjugate)
        const double sg = g.dagger ? -1.0 : 1.0;
        const C2 m[4] = {{0.5, 0.5 * sg}, {0.5, -0.5 * sg}, {0.5, -0.5 * sg}, {0.5, 0.5 * sg}};
        out.push_back(g2p_gate(a, ctrl, F_ID, nullptr, 0, F_GEN, m, 0));
        return;
    }
    case QVNT_GATE_SQRT_ISWAP: {  // sqrt_i_swap.rs: r p + i r p(partner) (dagger: -i r)
        const double sg = g.dagger ? -1.0 : 1.0;
        const C2 m[4] = {{r, 0}, {0, r * sg}, {0, r * sg}, {r, 0}};
        out.push_back(g2p_gate(a, ctrl, F_ID, nullptr, 0, F_RX, m, 0));
        return;
    }
    case QVNT_GATE_U2: {  // u2.rs: dense 4x4, member index (b_bit << 1) | a_bit
        EGate e;
        const DevGate d = decode_gate(g);
        if (plain_gate_needs_gather(d)) {
            e.standalone = true;
            e.src = src;
            out.push_back(e);
            return;
        }
        const int qa = __builtin_ctzll(g.a_mask), qb = __builtin_ctzll(g.b_mask);
        e.op = OP_G4;
        e.ctrl = ctrl;
        e.q0 = std::min(qa, qb);
        e.q1 = std::max(qa, qb);
        // engine member order: (bit q0) | (bit q1) << 1; swap the roles of a and b when qa > qb
        auto perm = [&](int rr) { return qa < qb ? rr : (((rr & 1) << 1) | ((rr >> 1) & 1)); };
        for (int rr = 0; rr < 4; ++rr)
            for (int cc = 0; cc < 4; ++cc) {
                const int sr = perm(rr), sc = perm(cc);
                push_df(e.coef, g.matrix[2 * (4 * sr + sc)]);
                push_df(e.coef, g.matrix[2 * (4 * sr + sc) + 1]);
            }
        e.cost = 150;
        out.push_back(e);
        return;
    }
    default:
        return;
    }
}

// Merges runs of consecutive one-qubit gates on the same qubit and control mask into one 2x2
// matrix (multiplied in double precision) when that is cheaper than running them one by one.
void merge_one_qubit_runs(std::vector<EGate>& eg) {
    std::vector<EGate> out;
    out.reserve(eg.size());
    size_t i = 0;
    while (i < eg.size()) {
        size_t j = i;
        if (eg[i].has_m2) {
            while (j + 1 < eg.size() && eg[j + 1].has_m2 && eg[j + 1].q0 == eg[i].q0 && eg[j + 1].ctrl == eg[i].ctrl) ++j;
        }
        int total = 0;
        for (size_t k = i; k <= j; ++k) total += eg[k].cost;
        if (j > i && total > form_cost(F_GEN)) {
            C2 M[4] = {eg[i].m2[0], eg[i].m2[1], eg[i].m2[2], eg[i].m2[3]};
            for (size_t k = i + 1; k <= j; ++k) {
                const C2* A = eg[k].m2;  // applied after M: M <- A M
                C2 R[4];
                R[0] = cadd(cmul(A[0], M[0]), cmul(A[1], M[2]));
                R[1] = cadd(cmul(A[0], M[1]), cmul(A[1], M[3]));
                R[2] = cadd(cmul(A[2], M[0]), cmul(A[3], M[2]));
                R[3] = cadd(cmul(A[2], M[1]), cmul(A[3], M[3]));
                for (int w = 0; w < 4; ++w) M[w] = R[w];
            }
            out.push_back(g1_matrix(eg[i].q0, eg[i].ctrl, M));
        } else {
            for (size_t k = i; k <= j; ++k) out.push_back(eg[k]);
        }
        i = j + 1;
    }
    eg.swap(out);
}

uint64_t targets_of(const EGate& e) {
    if (e.op == OP_DIAG || e.standalone) return 0;
    uint64_t t = 1ull << e.q0;
    if (e.q1 >= 0) t |= 1ull << e.q1;
    return t;
}

uint64_t touched_of(const EGate& e) {
    if (e.op == OP_DIAG) return e.dmask | e.ctrl;
    return targets_of(e) | e.ctrl;
}

struct PlannedPass {
    bool standalone = false;
    size_t src = 0;
    uint64_t qmask = 0;
    std::vector<size_t> members;  // indices into the engine gate list
};

// Pass budget in estimated FP32 instructions per amplitude (form_cost units).  One HBM round trip
// of a tile hides about 200 (32 B per amplitude at ~6.8 TB/s against ~114 FFMA/clk/SM), but on GB300
// double-float passes are compute-bound, so fewer, heavier passes win: measured on the 30-qubit
// random circuit, 200 -> 330 passes, 505 gate-passes/s; 450 -> 151, 532; 800 -> 130, 539;
// 1400 -> 121, 540.
int pass_budget() {
    static int b = [] {
        const char* e = std::getenv("QVNT_PASS_BUDGET");
        const int v = e ? std::atoi(e) : 0;
        return v > 0 ? v : 800;
    }();
    return b;
}
constexpr size_t kLookahead = 2048;

// What one pass may hold: the single-register kernel is bounded by its parameter space; the batch
// kernel reads its descriptors from global memory and, when the tile is the whole register, takes
// the entire circuit in one pass.
struct PlanLimits {
    int budget = 0;
    size_t max_gates = kMaxGates;
    size_t max_coef = kMaxCoef;
};

int plan_fused(const qvnt_gate* gates, size_t count, uint32_t L, uint32_t fusion_k, const KCfg& cfg,
               std::vector<EGate>& eg, std::vector<uint64_t>& tgt, std::vector<PlannedPass>& passes,
               uint32_t* kk_out, PlanLimits lim = PlanLimits()) {
    const uint32_t k = std::min<uint32_t>(fusion_k ? fusion_k : cfg.kt, std::min<uint32_t>(L, cfg.kt));
    const uint32_t kk = std::max<uint32_t>(k, cfg.kr);
    // At least two free tile slots, so that every two-qubit gate fits an empty pass.
    const uint32_t c0 = std::min<uint32_t>(kLowQ, kk - 2);
    const uint64_t low = (1ull << c0) - 1ull;
    const uint64_t all = (1ull << L) - 1ull;
    const int budget_max = lim.budget > 0 ? lim.budget : pass_budget();
    *kk_out = kk;

    eg.clear();
    eg.reserve(count * 2);
    for (size_t i = 0; i < count; ++i) lower(gates[i], i, eg);
    merge_one_qubit_runs(eg);
    const size_t ne = eg.size();
    std::vector<uint64_t> tch(ne);
    tgt.assign(ne, 0);
    for (size_t i = 0; i < ne; ++i) {
        tgt[i] = targets_of(eg[i]);
        // a standalone gate is an ordering barrier: nothing moves across it
        tch[i] = eg[i].standalone ? ~0ull : touched_of(eg[i]);
    }

    std::vector<char> done(ne, 0);
    passes.clear();
    size_t first = 0;
    while (true) {
        while (first < ne && done[first]) ++first;
        if (first >= ne) break;
        if (eg[first].standalone) {
            PlannedPass p;
            p.standalone = true;
            p.src = eg[first].src;
            passes.push_back(p);
            done[first] = 1;
            continue;
        }
        PlannedPass p;
        uint64_t Q = low;
        uint32_t free_slots = kk - c0;
        uint64_t block_nd = 0, block_d = 0;
        int budget = 0;
        size_t scanned = 0, ncoef = 0;
        for (size_t j = first; j < ne && scanned < kLookahead; ++j) {
            if (done[j]) continue;
            ++scanned;
            const EGate& g = eg[j];
            const bool diag = g.op == OP_DIAG;
            const bool conflict = diag ? (tch[j] & block_nd) != 0 : (tch[j] & (block_nd | block_d)) != 0;
            bool take = false;
            // an empty pass takes its first gate whatever the budget, so every gate gets placed
            if (!conflict && !g.standalone && (budget + g.cost <= budget_max || p.members.empty()) &&
                p.members.size() < lim.max_gates &&
                ncoef + g.coef.size() <= lim.max_coef) {
                const uint64_t need = tgt[j] & ~Q;
                if (popc(need) <= free_slots) {
                    Q |= need;
                    free_slots -= popc(need);
                    take = true;
                }
            }
            if (take) {
                p.members.push_back(j);
                done[j] = 1;
                budget += g.cost;
                ncoef += g.coef.size();
                continue;
            }
            if (diag) block_d |= tch[j];
            else block_nd |= tch[j];
            if ((block_nd & all) == all) break;
            if (budget >= budget_max) break;
        }
        if (p.members.empty())
            return set_error(QVNT_ERR_UNSUPPORTED, "fused planner could not place engine gate %zu", first);
        for (uint32_t b = 0; b < L && free_slots > 0; ++b)
            if (!((Q >> b) & 1ull)) {
                Q |= 1ull << b;
                --free_slots;
            }
        p.qmask = Q;
        passes.push_back(p);
    }
    return QVNT_OK;
}

// Register stages of a pass: contiguous runs of members whose targets fit kr register bits.
template <class LocalFn>
void build_stages(const PlannedPass& p, const std::vector<EGate>& eg, const std::vector<uint64_t>& tgt, int kr,
                  LocalFn&& local, std::vector<std::pair<uint32_t, std::vector<size_t>>>& stages) {
    stages.clear();
    for (size_t m : p.members) {
        const uint32_t lt = local(tgt[m]);
        if (stages.empty() || (eg[m].op != OP_DIAG && popc(stages.back().first | lt) > (unsigned)kr))
            stages.push_back({lt, {}});
        else
            stages.back().first |= lt;
        stages.back().second.push_back(m);
    }
}

// Pass descriptor in host form: header, register stages (gate ranges relative to the pass), engine
// gates (coefficient offsets relative to the pass) and the df64 coefficient pool.
struct PassHead {
    uint64_t ntiles = 0;
    uint32_t k = 0, c = 0, nthreads = 0, nstages = 0;
    uint32_t tq[kMaxKT] = {};
    float scale_h = 0.f, scale_l = 0.f;
    uint32_t has_scale = 0;
    void copy_to(PassParams& P) const {
        P.ntiles = ntiles;
        P.k = k;
        P.c = c;
        P.nthreads = nthreads;
        P.nstages = nstages;
        for (int i = 0; i < kMaxKT; ++i) P.tq[i] = tq[i];
        P.scale_h = scale_h;
        P.scale_l = scale_l;
        P.has_scale = has_scale;
    }
};

struct PassEnc {
    PassHead head;
    std::vector<DStage> stages;
    std::vector<DGate> gates;
    std::vector<float> coef;
};

void encode_pass(const PlannedPass& p, const std::vector<EGate>& eg, const std::vector<uint64_t>& tgt, int kr,
                 uint32_t L, uint64_t len, PassEnc& out);

template <class F>
int launch_passes(qvnt_reg* r, const qvnt_gate* gates, const std::vector<EGate>& eg, const std::vector<uint64_t>& tgt,
                  const std::vector<PlannedPass>& passes, uint32_t kk, const KCfg& cfg, F&& standalone_gate) {
    const uint32_t L = (uint32_t)__builtin_ctzll(r->len);
    const int kr = cfg.kr;
    PassParams* P = new PassParams;
    int* d_err = reinterpret_cast<int*>(reinterpret_cast<char*>(r->d_small) + 32);
    const size_t smem = ((size_t)1 << kk) * 16;
    // registers may be driven from several host threads (the serving loop): the attribute is set
    // once per configuration, idempotently
    static std::atomic<bool> attr_set[sizeof(kCfgs) / sizeof(kCfgs[0])] = {};
    const size_t ci = (size_t)(&cfg - kCfgs);
    if (!attr_set[ci].load(std::memory_order_acquire)) {
        QVNT_CUDA_TRY(cudaFuncSetAttribute((const void*)cfg.fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)(((size_t)1 << cfg.kt) * 16)));
        attr_set[ci].store(true, std::memory_order_release);
    }
    int per_sm = 0;
    QVNT_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void*)cfg.fn,
                                                                1 << (cfg.kt - cfg.kr), smem));
    if (per_sm < 1) per_sm = 1;
    int status = QVNT_OK;
    PassEnc enc;
    for (const PlannedPass& p : passes) {
        if (p.standalone) {
            status = standalone_gate(gates[p.src]);
            if (status) break;
            continue;
        }
        memset(P, 0, sizeof(PassParams));
        encode_pass(p, eg, tgt, kr, L, r->len, enc);
        if (enc.stages.size() > (size_t)kMaxStages || enc.gates.size() > (size_t)kMaxGates ||
            enc.coef.size() > (size_t)kMaxCoef) {
            status = set_error(QVNT_ERR_UNSUPPORTED, "pass needs %zu stages, %zu gates", enc.stages.size(),
                               enc.gates.size());
            break;
        }
        enc.head.copy_to(*P);
        std::copy(enc.stages.begin(), enc.stages.end(), P->stages);
        std::copy(enc.gates.begin(), enc.gates.end(), P->gates);
        std::copy(enc.coef.begin(), enc.coef.end(), P->coef);
        // persistent grid by default; one CTA per tile when the register shares the GPU with others
        // (CTAs then retire every tile, so other streams' higher-priority work gets SMs quickly)
        uint64_t grid = r->tile_grid ? P->ntiles : (uint64_t)r->ctx->geo.sms * per_sm;
        if (grid > P->ntiles) grid = P->ntiles;
        cudaEvent_t stop = nullptr;
        status = timing_begin(r, &stop);
        if (status) break;
        launch_cfg(ci, (unsigned)grid, P->nthreads, smem, r->stream, reinterpret_cast<float4*>(r->psi), *P, d_err);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) {
            status = set_cuda_error(e, "fused_df_kernel launch");
            break;
        }
        status = timing_end(r, stop);
        if (status) break;
        r->launches += 1;
        r->passes += 1;
    }
    delete P;
    return status;
}

void encode_pass(const PlannedPass& p, const std::vector<EGate>& eg, const std::vector<uint64_t>& tgt, int kr,
                 uint32_t L, uint64_t len, PassEnc& out) {
    PassHead& H = out.head;
    H = PassHead();
    out.gates.clear();
    out.coef.clear();
    uint32_t n = 0;
    uint32_t pos_of[64];
    for (uint32_t b = 0; b < L; ++b)
        if ((p.qmask >> b) & 1ull) {
            pos_of[b] = n;
            H.tq[n++] = b;
        }
    uint32_t run = 0;
    while (run < n && H.tq[run] == run) ++run;
    H.k = n;
    H.c = std::min<uint32_t>(run, n);
    H.nthreads = 1u << (n - kr);
    H.ntiles = len >> n;
    auto local = [&](uint64_t m) {  // global mask (within Q) -> tile-local mask
        uint32_t lm = 0;
        for (uint32_t b = 0; b < L; ++b)
            if (((m & p.qmask) >> b) & 1ull) lm |= 1u << pos_of[b];
        return lm;
    };
    std::vector<std::pair<uint32_t, std::vector<size_t>>> stages;
    build_stages(p, eg, tgt, kr, local, stages);
    out.stages.assign(stages.size(), DStage());
    // deferred Hadamard scale 2^(-m/2) of the pass, exact as a df pair
    int m_h = 0;
    for (size_t m : p.members) m_h += eg[m].hadd ? 1 : 0;
    if (m_h) {
        const double pw = std::ldexp(1.0, -(m_h / 2));
        if (m_h & 1) {
            const double rr = 0.70710678118654752440084436210484903;
            const float h = (float)rr;
            H.scale_h = (float)((double)h * pw);
            H.scale_l = (float)((rr - (double)h) * pw);
        } else {
            H.scale_h = (float)pw;
            H.scale_l = 0.f;
        }
        H.has_scale = 1;
    }
    H.nstages = (uint32_t)stages.size();
    out.gates.resize(p.members.size());
    uint32_t ng = 0;
    for (size_t si = 0; si < stages.size(); ++si) {
        uint32_t R = stages[si].first;
        // Fill the free register bits, preferring qubits that single-qubit diagonals and controls
        // of this stage read (their slot selection then folds at compile time), then the highest
        // free tile bits (keeps the lanes on low tile bits).
        auto add_pref = [&](uint32_t bits) {
            for (uint32_t b = 0; b < n && popc(R) < (unsigned)kr; ++b)
                if (((bits >> b) & 1u) && !((R >> b) & 1u)) R |= 1u << b;
        };
        for (size_t m : stages[si].second)
            if (eg[m].op == OP_DIAG && popc(eg[m].dmask) <= 2) add_pref(local(eg[m].dmask));
        for (size_t m : stages[si].second) add_pref(local(eg[m].ctrl));
        for (int b = (int)n - 1; b >= 0 && popc(R) < (unsigned)kr; --b)
            if (!((R >> b) & 1u)) R |= 1u << b;
        DStage& S = out.stages[si];
        uint32_t nb = 0, nt = 0;
        uint32_t rix[kMaxKT], tix[kMaxKT];
        for (uint32_t b = 0; b < n; ++b) {
            if ((R >> b) & 1u) {
                rix[b] = nb;
                S.rbit[nb++] = (uint8_t)b;
            } else {
                tix[b] = nt;
                S.tbit[nt++] = (uint8_t)b;
            }
        }
        S.gbegin = (uint16_t)ng;
        for (size_t m : stages[si].second) {
            const EGate& e = eg[m];
            DGate& G = out.gates[ng++];
            G.op = e.op;
            G.form0 = e.form0;
            G.form1 = e.form1;
            G.dkind = e.dkind;
            G.exact = e.exact ? 1 : 0;
            G.codes = e.codes;
            G.coef = (uint32_t)out.coef.size();
            out.coef.insert(out.coef.end(), e.coef.begin(), e.coef.end());
            const uint32_t lc = local(e.ctrl);
            G.ctrl_out = e.ctrl & ~p.qmask;
            uint32_t creg = 0, cthr = 0;
            for (uint32_t b = 0; b < n; ++b)
                if ((lc >> b) & 1u) {
                    if ((R >> b) & 1u) creg |= 1u << rix[b];
                    else cthr |= 1u << tix[b];
                }
            G.ctrl_reg = (uint8_t)creg;
            G.ctrl_thr = (uint16_t)cthr;
            if (e.op == OP_DIAG) {
                const uint32_t ld = local(e.dmask);
                G.dm_out = e.dmask & ~p.qmask;
                uint32_t dreg = 0, dthr = 0;
                for (uint32_t b = 0; b < n; ++b)
                    if ((ld >> b) & 1u) {
                        if ((R >> b) & 1u) dreg |= 1u << rix[b];
                        else dthr |= 1u << tix[b];
                    }
                G.dm_reg = (uint8_t)dreg;
                G.dm_thr = (uint16_t)dthr;
                if (e.dkind == D_PAR && popc(dreg) <= 2) {
                    // parity diagonal with at most two register bits: compile-time slot parity
                    G.op = OP_DIAG1;
                    G.one0 = e.one0 ? 1 : 0;
                    if (dreg) G.b0 = (uint8_t)__builtin_ctz(dreg);
                    if (popc(dreg) == 2) G.b1 = (uint8_t)(31 - __builtin_clz(dreg));
                }
            } else {
                G.b0 = (uint8_t)rix[pos_of[e.q0]];
                if (e.q1 >= 0) G.b1 = (uint8_t)rix[pos_of[e.q1]];
            }
        }
        S.gend = (uint16_t)ng;
    }
}

// ---- batch schedule ---------------------------------------------------------------------------------
struct BatchRegSpec {
    uint32_t L = 0;          // log2 of the amplitude count
    uint64_t off = 0;        // float4 offset in the arena
    uint64_t mask = 0;       // measure mask (0: no measurement)
    const qvnt_gate* gates = nullptr;
    size_t ngates = 0;
};

struct BatchSchedule {
    std::vector<BItem> items;
    std::vector<BEntry> entries;
    std::vector<BPass> passes;
    std::vector<DStage> stages;
    std::vector<DGate> gates;
    std::vector<float> coef;
};

// Plans every register of `subset` with tile width fusion_k (the whole register when it is not wider)
// and orders the items in waves.  Registers that fit one tile take their entire circuit in one pass.
int build_batch_schedule(const std::vector<BatchRegSpec>& regs, const std::vector<uint32_t>& subset,
                         uint32_t fusion_k, int budget, BatchSchedule& out) {
    out = BatchSchedule();
    const KCfg cfg{kBatchKT, kBatchKR, kBatchMinB, nullptr};
    std::vector<std::vector<uint32_t>> reg_passes(regs.size());
    std::vector<uint64_t> reg_tiles(regs.size(), 1);
    std::vector<EGate> eg;
    std::vector<uint64_t> tgt;
    std::vector<PlannedPass> pl;
    PassEnc enc;
    size_t maxp = 0;
    for (uint32_t R : subset) {
        const BatchRegSpec& s = regs[R];
        const uint32_t k = std::min<uint32_t>(fusion_k, kBatchKT);
        PlanLimits lim;
        lim.max_gates = 60000;  // DStage gate ranges are 16-bit
        lim.max_coef = ~(size_t)0 >> 1;
        lim.budget = s.L <= k ? (1 << 28) : budget;
        uint32_t kk = 0;
        int st = plan_fused(s.gates, s.ngates, s.L, k, cfg, eg, tgt, pl, &kk, lim);
        if (st) return st;
        reg_tiles[R] = (1ull << s.L) >> kk;
        for (const PlannedPass& p : pl) {
            if (p.standalone)
                return set_error(QVNT_ERR_UNSUPPORTED, "register %u: gate %zu needs a standalone pass, which the batch "
                                                       "kernel does not run", R, p.src);
            encode_pass(p, eg, tgt, kBatchKR, s.L, 1ull << s.L, enc);
            BPass bp{};
            bp.ntiles = enc.head.ntiles;
            bp.k = enc.head.k;
            bp.c = enc.head.c;
            bp.nthreads = enc.head.nthreads;
            bp.nstages = enc.head.nstages;
            for (int i = 0; i < kMaxKT; ++i) bp.tq[i] = enc.head.tq[i];
            bp.scale_h = enc.head.scale_h;
            bp.scale_l = enc.head.scale_l;
            bp.has_scale = enc.head.has_scale;
            bp.stage0 = (uint32_t)out.stages.size();
            bp.gate0 = (uint32_t)out.gates.size();
            bp.coef0 = (uint32_t)out.coef.size();
            if (out.coef.size() + enc.coef.size() > 0xffffffffull || out.gates.size() + enc.gates.size() > 0xffffffffull)
                return set_error(QVNT_ERR_UNSUPPORTED, "batch schedule too large");
            out.stages.insert(out.stages.end(), enc.stages.begin(), enc.stages.end());
            out.gates.insert(out.gates.end(), enc.gates.begin(), enc.gates.end());
            out.coef.insert(out.coef.end(), enc.coef.begin(), enc.coef.end());
            reg_passes[R].push_back((uint32_t)out.passes.size());
            out.passes.push_back(bp);
        }
        maxp = std::max(maxp, reg_passes[R].size());
    }
    // wave order; inside a wave the widest registers first
    std::vector<uint32_t> order(subset);
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return regs[a].L > regs[b].L; });
    for (size_t w = 0; w <= maxp; ++w) {
        for (uint32_t R : order) {
            const BatchRegSpec& s = regs[R];
            const size_t np = reg_passes[R].size();
            BEntry e{};
            e.psi_off = s.off;
            e.len = 1ull << s.L;
            e.mask = s.mask;
            e.reg = R;
            if (w < np) {
                e.pass = reg_passes[R][w];
                e.need = (uint32_t)(w * reg_tiles[R]);
                const uint32_t ei = (uint32_t)out.entries.size();
                out.entries.push_back(e);
                for (uint64_t t = 0; t < reg_tiles[R]; ++t) out.items.push_back(BItem{ei, (uint32_t)t});
            } else if (w == np && s.mask) {
                e.pass = kMeasureItem;
                e.need = (uint32_t)(np * reg_tiles[R]);
                out.items.push_back(BItem{(uint32_t)out.entries.size(), 0});
                out.entries.push_back(e);
            }
        }
    }
    return QVNT_OK;
}

__global__ void batch_basis_kernel(float4* __restrict__ psi, const uint64_t* __restrict__ idx, uint32_t count) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) psi[idx[i]] = make_float4(1.f, 0.f, 0.f, 0.f);
}

}  // namespace

void EngineBuffers::release() {
    if (d_buf) cudaFree(d_buf);
    if (h_buf) cudaFreeHost(h_buf);
    for (void* p : retired) cudaFreeHost(p);
    retired.clear();
    if (uploaded) cudaEventDestroy(uploaded);
    d_buf = nullptr;
    h_buf = nullptr;
    uploaded = nullptr;
    d_bytes = h_bytes = 0;
}

int EngineBuffers::acquire(size_t bytes, cudaStream_t stream) {
    if (uploaded) QVNT_CUDA_TRY(cudaEventSynchronize(uploaded));  // the last upload from h_buf is done
    size_t cap = (size_t)1 << 20;
    while (cap < bytes) cap <<= 1;
    if (d_bytes < bytes) {
        // stream-ordered: the old buffer is freed after the passes queued before this call read it
        if (d_buf) QVNT_CUDA_TRY(cudaFreeAsync(d_buf, stream));
        d_buf = nullptr;
        d_bytes = 0;
        QVNT_CUDA_TRY(cudaMallocAsync(&d_buf, cap, stream));
        d_bytes = cap;
    }
    if (h_bytes < bytes) {
        if (h_buf) retired.push_back(h_buf);
        h_buf = nullptr;
        h_bytes = 0;
        QVNT_CUDA_TRY(cudaMallocHost(&h_buf, cap));
        h_bytes = cap;
    }
    return QVNT_OK;
}

int EngineBuffers::upload(size_t bytes, cudaStream_t stream) {
    QVNT_CUDA_TRY(cudaMemcpyAsync(d_buf, h_buf, bytes, cudaMemcpyHostToDevice, stream));
    if (!uploaded) QVNT_CUDA_TRY(cudaEventCreateWithFlags(&uploaded, cudaEventDisableTiming));
    QVNT_CUDA_TRY(cudaEventRecord(uploaded, stream));
    return QVNT_OK;
}

int apply_fused(qvnt_reg* r, const qvnt_gate* gates, size_t count) {
    const uint32_t L = (uint32_t)__builtin_ctzll(r->len);
    const int fmt = FMT_DF64;
    const KCfg& cfg = active_cfg();
    // Gates the tiles do not take, and every gate of registers smaller than a register stage, run
    // as per-gate passes on the double-float storage.
    auto standalone_gate = [&](const qvnt_gate& g) -> int {
        DevGate d = decode_gate(g);
        if (plain_gate_is_identity(d)) return QVNT_OK;
        int st;
        if (plain_gate_needs_gather(d)) {
            st = reg_ensure_alt(r);
            if (st) return st;
            st = launch_gather_gate(r->psi, r->alt, fmt, r->len, d, r->stream, r->ctx->geo);
            std::swap(r->psi, r->alt);
        } else {
            st = launch_plain_gate(r->psi, fmt, r->len, d, r->stream, r->ctx->geo);
        }
        r->launches += 1;
        r->passes += 1;
        return st;
    };
    if (L < (uint32_t)cfg.kr) {
        for (size_t i = 0; i < count; ++i) {
            int st = standalone_gate(gates[i]);
            if (st) return st;
        }
        return QVNT_OK;
    }
    std::vector<EGate> eg;
    std::vector<uint64_t> tgt;
    std::vector<PlannedPass> passes;
    uint32_t kk = 0;
    int status = plan_fused(gates, count, L, r->fusion_k, cfg, eg, tgt, passes, &kk);
    if (status) return status;
    return launch_passes(r, gates, eg, tgt, passes, kk, cfg, standalone_gate);
}

}  // namespace qvnt

using namespace qvnt;

extern "C" int qvnt_plan_info(const qvnt_gate* gates, size_t count, uint32_t q_num, uint32_t fusion_k,
                              uint64_t* passes, uint64_t* stages, uint64_t* engine_gates) {
    if (!gates && count) return set_error(QVNT_ERR_BAD_ARG, "null gate list");
    if (q_num > 40) return set_error(QVNT_ERR_BAD_ARG, "q_num %u > 40", q_num);
    const uint64_t len = q_num < 3 ? 8 : (1ull << q_num);
    for (size_t k = 0; k < count; ++k) {
        int st = validate_gate(gates[k], len);
        if (st) return set_error(st, "gate %zu: %s", k, qvnt_last_error());
    }
    const uint32_t L = (uint32_t)__builtin_ctzll(len);
    const KCfg& cfg = active_cfg();
    uint64_t np = 0, ns = 0, nq = 0;
    if (L < (uint32_t)cfg.kr) {
        np = count;
    } else {
        std::vector<EGate> eg;
        std::vector<uint64_t> tgt;
        std::vector<PlannedPass> pl;
        uint32_t kk = 0;
        int st = plan_fused(gates, count, L, fusion_k, cfg, eg, tgt, pl, &kk);
        if (st) return st;
        np = pl.size();
        nq = eg.size();
        std::vector<std::pair<uint32_t, std::vector<size_t>>> stg;
        for (const PlannedPass& p : pl) {
            if (p.standalone) continue;
            auto local = [&](uint64_t m) {  // global mask within the tile -> tile-local mask
                uint32_t lm = 0, n = 0;
                for (uint32_t b = 0; b < L; ++b)
                    if ((p.qmask >> b) & 1ull) {
                        if ((m >> b) & 1ull) lm |= 1u << n;
                        ++n;
                    }
                return lm;
            };
            build_stages(p, eg, tgt, cfg.kr, local, stg);
            ns += stg.size();
        }
    }
    if (passes) *passes = np;
    if (stages) *stages = ns;
    if (engine_gates) *engine_gates = nq;
    return QVNT_OK;
}

// ---- batching form: C ABI ------------------------------------------------------------------------
struct qvnt_batch {
    uint32_t magic = 0;
    qvnt_ctx* ctx = nullptr;
    cudaStream_t stream = nullptr;
    std::vector<BatchRegSpec> regs;
    std::vector<std::vector<qvnt_gate>> circuits;
    std::vector<uint64_t> basis;  // float4 index of each register's initial basis state
    uint64_t arena_amps = 0;
    float4* psi = nullptr;
    // per-register device arrays: done counters, results, draws, basis indices; error flag, queue head
    void* d_reg = nullptr;
    unsigned int* d_done = nullptr;
    unsigned long long* d_results = nullptr;
    double* d_u01 = nullptr;
    uint64_t* d_basis = nullptr;
    unsigned long long* d_next = nullptr;
    int* d_err = nullptr;
    void* h_pinned = nullptr;  // u01 | results | err
    double* h_u01 = nullptr;
    unsigned long long* h_results = nullptr;
    int* h_err = nullptr;
    // schedule
    void* d_sched = nullptr;
    BatchArgs args{};
    uint64_t nitems = 0, npasses = 0;
    uint32_t fusion_k = kBatchKT;
    int budget = 0;
    int minb = kBatchMinB;  // kernel variant: CTAs per SM
    bool has_measure = false;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    double last_ms = 0.0;
};

namespace {

constexpr uint32_t kMagicBatch = 0x51424154u;
constexpr uint32_t kBatchMaxQubits = 26;

bool batch_ok(const qvnt_batch* b) { return b && b->magic == kMagicBatch; }

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Uploads a schedule into one device buffer and fills the kernel arguments.
int batch_upload(qvnt_batch* b, const BatchSchedule& s, void** d_buf, BatchArgs* a) {
    const size_t o_items = 0;
    const size_t o_entries = align256(o_items + s.items.size() * sizeof(BItem));
    const size_t o_passes = align256(o_entries + s.entries.size() * sizeof(BEntry));
    const size_t o_stages = align256(o_passes + s.passes.size() * sizeof(BPass));
    const size_t o_gates = align256(o_stages + s.stages.size() * sizeof(DStage));
    const size_t o_coef = align256(o_gates + s.gates.size() * sizeof(DGate));
    const size_t total = align256(o_coef + s.coef.size() * sizeof(float)) + 256;
    std::vector<char> h(total, 0);
    auto put = [&](size_t off, const void* src, size_t bytes) {
        if (bytes) memcpy(h.data() + off, src, bytes);
    };
    put(o_items, s.items.data(), s.items.size() * sizeof(BItem));
    put(o_entries, s.entries.data(), s.entries.size() * sizeof(BEntry));
    put(o_passes, s.passes.data(), s.passes.size() * sizeof(BPass));
    put(o_stages, s.stages.data(), s.stages.size() * sizeof(DStage));
    put(o_gates, s.gates.data(), s.gates.size() * sizeof(DGate));
    put(o_coef, s.coef.data(), s.coef.size() * sizeof(float));
    char* d = nullptr;
    cudaError_t e = cudaMalloc(&d, total);
    if (e != cudaSuccess) return set_cuda_error(e, "cudaMalloc(batch schedule)");
    e = cudaMemcpy(d, h.data(), total, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(d);
        return set_cuda_error(e, "batch schedule upload");
    }
    *d_buf = d;
    BatchArgs& A = *a;
    A.psi = b->psi;
    A.items = reinterpret_cast<const BItem*>(d + o_items);
    A.nitems = s.items.size();
    A.entries = reinterpret_cast<const BEntry*>(d + o_entries);
    A.passes = reinterpret_cast<const BPass*>(d + o_passes);
    A.stages = reinterpret_cast<const DStage*>(d + o_stages);
    A.gates = reinterpret_cast<const DGate*>(d + o_gates);
    A.coef = reinterpret_cast<const float*>(d + o_coef);
    A.u01 = b->d_u01;
    A.done = b->d_done;
    A.next = b->d_next;
    A.results = b->d_results;
    A.err = b->d_err;
    return QVNT_OK;
}

using BatchFn = void (*)(BatchArgs);

BatchFn batch_fn(int minb) {
    return minb == 1 ? batch_df_kernel<kBatchKT, kBatchKR, 1> : batch_df_kernel<kBatchKT, kBatchKR, kBatchMinB>;
}

int batch_grid(qvnt_batch* b, int minb, unsigned* grid) {
    constexpr size_t smem = ((size_t)1 << kBatchKT) * 16;
    static std::atomic<bool> attr[3] = {};
    const BatchFn fn = batch_fn(minb);
    if (!attr[minb].load(std::memory_order_acquire)) {
        QVNT_CUDA_TRY(cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr[minb].store(true, std::memory_order_release);
    }
    int per_sm = 0;
    QVNT_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void*)fn, 1 << (kBatchKT - kBatchKR),
                                                                smem));
    if (per_sm < 1) per_sm = 1;
    *grid = (unsigned)(b->ctx->geo.sms * per_sm);
    return QVNT_OK;
}

// Enqueues one run: draws in, counters and states reset, the persistent kernel, results out.  No
// call here may synchronise: the sequence is captured into the batch's CUDA graph.
int batch_enqueue(qvnt_batch* b, const BatchArgs& A, unsigned grid, int minb, cudaStream_t s) {
    const uint32_t n = (uint32_t)b->regs.size();
    QVNT_CUDA_TRY(cudaMemcpyAsync(b->d_u01, b->h_u01, n * sizeof(double), cudaMemcpyHostToDevice, s));
    QVNT_CUDA_TRY(cudaMemsetAsync(b->d_done, 0, n * sizeof(unsigned int), s));
    QVNT_CUDA_TRY(cudaMemsetAsync(b->d_next, 0, sizeof(unsigned long long) + sizeof(int) * 2, s));
    QVNT_CUDA_TRY(cudaMemsetAsync(b->psi, 0, b->arena_amps * sizeof(float4), s));
    batch_basis_kernel<<<(n + 255) / 256, 256, 0, s>>>(b->psi, b->d_basis, n);
    QVNT_CUDA_TRY(cudaGetLastError());
    if (A.nitems) {
        if (minb == 1)
            batch_df_kernel<kBatchKT, kBatchKR, 1><<<grid, 1 << (kBatchKT - kBatchKR), ((size_t)1 << kBatchKT) * 16, s>>>(A);
        else
            batch_df_kernel<kBatchKT, kBatchKR, kBatchMinB>
                <<<grid, 1 << (kBatchKT - kBatchKR), ((size_t)1 << kBatchKT) * 16, s>>>(A);
        QVNT_CUDA_TRY(cudaGetLastError());
    }
    QVNT_CUDA_TRY(cudaMemcpyAsync(b->h_results, b->d_results, n * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    QVNT_CUDA_TRY(cudaMemcpyAsync(b->h_err, b->d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
    return QVNT_OK;
}

void batch_drop_schedule(qvnt_batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->d_sched) cudaFree(b->d_sched);
    b->exec = nullptr;
    b->graph = nullptr;
    b->d_sched = nullptr;
}

// Plans all registers with (fusion_k, budget), uploads, and captures the run as a CUDA graph.
int batch_plan(qvnt_batch* b, uint32_t fusion_k, int budget, int minb) {
    std::vector<uint32_t> all(b->regs.size());
    for (uint32_t i = 0; i < all.size(); ++i) all[i] = i;
    BatchSchedule s;
    int st = build_batch_schedule(b->regs, all, fusion_k, budget, s);
    if (st) return st;
    batch_drop_schedule(b);
    BatchArgs A{};
    st = batch_upload(b, s, &b->d_sched, &A);
    if (st) return st;
    b->args = A;
    b->nitems = s.items.size();
    b->npasses = s.passes.size();
    b->fusion_k = fusion_k;
    b->budget = budget;
    b->minb = minb;
    unsigned grid = 0;
    st = batch_grid(b, minb, &grid);
    if (st) return st;
    QVNT_CUDA_TRY(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    st = batch_enqueue(b, b->args, grid, minb, b->stream);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(b->stream, &g);
    if (st) {
        if (g) cudaGraphDestroy(g);
        return st;
    }
    if (e != cudaSuccess) return set_cuda_error(e, "batch graph capture");
    b->graph = g;
    QVNT_CUDA_TRY(cudaGraphInstantiate(&b->exec, g, 0));
    return QVNT_OK;
}

int batch_check_err(qvnt_batch* b) {
    const int e = *b->h_err;
    if (e == QVNT_ERR_TIMEOUT) return set_error(QVNT_ERR_TIMEOUT, "batch kernel: a dependency wait timed out");
    if (e) return set_error(e, "batch kernel: zero or non-finite norm in a measured register");
    return QVNT_OK;
}

void batch_free(qvnt_batch* b) {
    cudaSetDevice(b->ctx->device);
    batch_drop_schedule(b);
    if (b->psi) cudaFree(b->psi);
    if (b->d_reg) cudaFree(b->d_reg);
    if (b->h_pinned) cudaFreeHost(b->h_pinned);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->stream) cudaStreamDestroy(b->stream);
    b->magic = 0;
    delete b;
}

}  // namespace

#define CHECK_BATCH(b) \
    if (!batch_ok(b)) return set_error(QVNT_ERR_BAD_HANDLE, "invalid batch handle")

extern "C" int qvnt_batch_create(qvnt_ctx* ctx, uint32_t count, const uint32_t* q_nums, const uint64_t* states,
                                 const qvnt_gate* gates, const uint64_t* gate_offsets,
                                 const uint64_t* measure_masks, qvnt_batch** out) {
    if (!ctx_valid(ctx)) return set_error(QVNT_ERR_BAD_HANDLE, "invalid context handle");
    if (!out || !q_nums || !gate_offsets || (count && !states)) return set_error(QVNT_ERR_BAD_ARG, "null argument");
    if (count == 0) return set_error(QVNT_ERR_BAD_ARG, "empty batch");
    if (gate_offsets[0] != 0) return set_error(QVNT_ERR_BAD_ARG, "gate_offsets[0] must be 0");
    if (gate_offsets[count] && !gates) return set_error(QVNT_ERR_BAD_ARG, "null gate list");
    qvnt_batch* b = new qvnt_batch();
    b->ctx = ctx;
    b->regs.resize(count);
    b->circuits.resize(count);
    b->basis.resize(count);
    uint64_t off = 0;
    for (uint32_t i = 0; i < count; ++i) {
        const uint32_t n = q_nums[i];
        if (n < (uint32_t)kBatchKR || n > kBatchMaxQubits) {
            delete b;
            return set_error(QVNT_ERR_UNSUPPORTED, "register %u: %u qubits outside the batch range [%d, %u]", i, n,
                             kBatchKR, kBatchMaxQubits);
        }
        const uint64_t len = 1ull << n;
        if (states[i] >= len) {
            delete b;
            return set_error(QVNT_ERR_BAD_MASK, "register %u: state %llu out of range", i,
                             (unsigned long long)states[i]);
        }
        const uint64_t m = measure_masks ? measure_masks[i] : 0;
        if (m & ~(len - 1)) {
            delete b;
            return set_error(QVNT_ERR_BAD_MASK, "register %u: measure mask outside the register", i);
        }
        if (gate_offsets[i + 1] < gate_offsets[i]) {
            delete b;
            return set_error(QVNT_ERR_BAD_ARG, "gate_offsets must be non-decreasing");
        }
        for (uint64_t g = gate_offsets[i]; g < gate_offsets[i + 1]; ++g) {
            const int st = validate_gate(gates[g], len);
            if (st) {
                delete b;
                return set_error(st, "register %u, gate %llu: %s", i, (unsigned long long)(g - gate_offsets[i]),
                                 qvnt_last_error());
            }
        }
        b->circuits[i].assign(gates + gate_offsets[i], gates + gate_offsets[i + 1]);
        BatchRegSpec& s = b->regs[i];
        s.L = n;
        s.off = off;
        s.mask = m;
        s.gates = b->circuits[i].data();
        s.ngates = b->circuits[i].size();
        b->basis[i] = off + states[i];
        b->has_measure |= m != 0;
        off += (len + 15) & ~15ull;  // 256-byte aligned registers
    }
    b->arena_amps = off;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&b->psi, off * sizeof(float4));
    const size_t o_done = 0, o_res = align256(count * sizeof(unsigned int));
    const size_t o_u01 = align256(o_res + count * sizeof(unsigned long long));
    const size_t o_basis = align256(o_u01 + count * sizeof(double));
    const size_t o_next = align256(o_basis + count * sizeof(uint64_t));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_reg, o_next + 64);
    if (e == cudaSuccess) e = cudaMallocHost(&b->h_pinned, align256(count * 8) * 2 + 64);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev1);
    if (e != cudaSuccess) {
        const int st = set_cuda_error(e, "batch allocation");
        batch_free(b);
        return e == cudaErrorMemoryAllocation ? set_error(QVNT_ERR_OOM, "batch allocation: %s", qvnt_last_error()) : st;
    }
    char* d = static_cast<char*>(b->d_reg);
    b->d_done = reinterpret_cast<unsigned int*>(d + o_done);
    b->d_results = reinterpret_cast<unsigned long long*>(d + o_res);
    b->d_u01 = reinterpret_cast<double*>(d + o_u01);
    b->d_basis = reinterpret_cast<uint64_t*>(d + o_basis);
    b->d_next = reinterpret_cast<unsigned long long*>(d + o_next);
    b->d_err = reinterpret_cast<int*>(d + o_next + 8);
    char* h = static_cast<char*>(b->h_pinned);
    b->h_u01 = reinterpret_cast<double*>(h);
    b->h_results = reinterpret_cast<unsigned long long*>(h + align256(count * 8));
    b->h_err = reinterpret_cast<int*>(h + 2 * align256(count * 8));
    for (uint32_t i = 0; i < count; ++i) b->h_u01[i] = 0.5;
    e = cudaMemcpy(b->d_basis, b->basis.data(), count * sizeof(uint64_t), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        const int st = set_cuda_error(e, "batch upload");
        batch_free(b);
        return st;
    }
    b->magic = kMagicBatch;
    const int st = batch_plan(b, kBatchKT, 0, kBatchMinB);
    if (st) {
        batch_free(b);
        return st;
    }
    *out = b;
    return QVNT_OK;
}

extern "C" int qvnt_batch_destroy(qvnt_batch* b) {
    CHECK_BATCH(b);
    batch_free(b);
    return QVNT_OK;
}

extern "C" int qvnt_batch_set_fusion(qvnt_batch* b, uint32_t fusion_k, uint32_t pass_budget) {
    CHECK_BATCH(b);
    if (fusion_k < kFusedMinK || fusion_k > (uint32_t)kBatchKT)
        return set_error(QVNT_ERR_BAD_ARG, "fusion width %u outside [%u, %d]", fusion_k, kFusedMinK, kBatchKT);
    if (pass_budget > (1u << 20)) return set_error(QVNT_ERR_BAD_ARG, "pass budget %u too large", pass_budget);
    QVNT_CUDA_TRY(cudaSetDevice(b->ctx->device));
    return batch_plan(b, fusion_k, (int)pass_budget, b->minb);
}

extern "C" int qvnt_batch_run(qvnt_batch* b, const double* u01, uint64_t* measured) {
    CHECK_BATCH(b);
    if (b->has_measure && !u01) return set_error(QVNT_ERR_BAD_ARG, "the batch measures: u01 draws are required");
    const uint32_t n = (uint32_t)b->regs.size();
    for (uint32_t i = 0; i < n; ++i) {
        const double u = u01 ? u01[i] : 0.5;
        if (!(u >= 0.0 && u < 1.0)) return set_error(QVNT_ERR_BAD_ARG, "u01[%u] outside [0, 1)", i);
        b->h_u01[i] = u;
    }
    QVNT_CUDA_TRY(cudaSetDevice(b->ctx->device));
    QVNT_CUDA_TRY(cudaEventRecord(b->ev0, b->stream));
    QVNT_CUDA_TRY(cudaGraphLaunch(b->exec, b->stream));
    QVNT_CUDA_TRY(cudaEventRecord(b->ev1, b->stream));
    QVNT_CUDA_TRY(cudaStreamSynchronize(b->stream));
    float ms = 0.f;
    QVNT_CUDA_TRY(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
    b->last_ms = ms;
    const int st = batch_check_err(b);
    if (st) return st;
    if (measured)
        for (uint32_t i = 0; i < n; ++i) measured[i] = b->h_results[i];
    return QVNT_OK;
}

// Picks the fusion width and pass budget by timing the schedule of every `stride`-th register
// (a stratified sample: registers are usually generated in no particular size order) under each
// candidate, then re-plans the whole batch with the fastest.
extern "C" int qvnt_batch_autotune(qvnt_batch* b, uint32_t stride, uint32_t* fusion_k, uint32_t* pass_budget,
                                   double* best_ms) {
    CHECK_BATCH(b);
    if (stride == 0) stride = 1;
    QVNT_CUDA_TRY(cudaSetDevice(b->ctx->device));
    std::vector<uint32_t> sub;
    for (uint32_t i = 0; i < b->regs.size(); i += stride) sub.push_back(i);
    struct Cand {
        uint32_t k;
        int budget, minb;
    };
    const Cand cands[] = {{12, 200, 2}, {12, 400, 2}, {12, 800, 2}, {12, 1600, 2},
                          {12, 400, 1}, {12, 800, 1}, {12, 1600, 1}, {11, 800, 2}};
    double best = 1e300;
    uint32_t bk = kBatchKT;
    int bb = 0, bm = kBatchMinB;
    for (const Cand& cd : cands) {
        const uint32_t k = cd.k;
        const int bud = cd.budget;
        unsigned grid = 0;
        int gst = batch_grid(b, cd.minb, &grid);
        if (gst) return gst;
        BatchSchedule s;
        int st = build_batch_schedule(b->regs, sub, k, bud, s);
        if (st) return st;
        void* d = nullptr;
        BatchArgs A{};
        st = batch_upload(b, s, &d, &A);
        if (st) return st;
        float ms = 0.f;
        st = batch_enqueue(b, A, grid, cd.minb, b->stream);  // warm-up (first touch of the schedule)
        if (!st) {
            cudaEventRecord(b->ev0, b->stream);
            st = batch_enqueue(b, A, grid, cd.minb, b->stream);
            cudaEventRecord(b->ev1, b->stream);
        }
        cudaError_t e = cudaStreamSynchronize(b->stream);
        cudaFree(d);
        if (st) return st;
        if (e != cudaSuccess) return set_cuda_error(e, "batch autotune run");
        st = batch_check_err(b);
        if (st) return st;
        QVNT_CUDA_TRY(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
        if (ms < best) {
            best = ms;
            bk = k;
            bb = bud;
            bm = cd.minb;
        }
    }
    const int st = batch_plan(b, bk, bb, bm);
    if (st) return st;
    if (fusion_k) *fusion_k = bk;
    if (pass_budget) *pass_budget = (uint32_t)bb;
    if (best_ms) *best_ms = best;
    return QVNT_OK;
}

extern "C" int qvnt_batch_get_amplitudes(qvnt_batch* b, uint32_t index, double* out) {
    CHECK_BATCH(b);
    if (!out) return set_error(QVNT_ERR_BAD_ARG, "null output");
    if (index >= b->regs.size()) return set_error(QVNT_ERR_BAD_ARG, "register %u out of range", index);
    const BatchRegSpec& s = b->regs[index];
    const uint64_t len = 1ull << s.L;
    std::vector<float4> h(len);
    QVNT_CUDA_TRY(cudaSetDevice(b->ctx->device));
    QVNT_CUDA_TRY(cudaMemcpyAsync(h.data(), b->psi + s.off, len * sizeof(float4), cudaMemcpyDeviceToHost, b->stream));
    QVNT_CUDA_TRY(cudaStreamSynchronize(b->stream));
    for (uint64_t i = 0; i < len; ++i) {
        out[2 * i] = (double)h[i].x + (double)h[i].y;
        out[2 * i + 1] = (double)h[i].z + (double)h[i].w;
    }
    return QVNT_OK;
}

extern "C" int qvnt_batch_info(const qvnt_batch* b, uint64_t* items, uint64_t* passes, uint64_t* state_bytes,
                               uint32_t* fusion_k, uint32_t* budget_out, double* last_ms) {
    CHECK_BATCH(b);
    if (items) *items = b->nitems;
    if (passes) *passes = b->npasses;
    if (state_bytes) *state_bytes = b->arena_amps * sizeof(float4);
    if (fusion_k) *fusion_k = b->fusion_k;
    if (budget_out) *budget_out = (uint32_t)(b->budget > 0 ? b->budget : pass_budget());
    if (last_ms) *last_ms = b->last_ms;
    return QVNT_OK;
}
