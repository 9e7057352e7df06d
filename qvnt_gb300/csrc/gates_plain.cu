// Plain engine: one in-place FP64 pass per SingleOp (the plain f64 GPU path).
//
// qvnt computes every output amplitude by a gather over the input (`AtomicOp::for_each`,
// src/operator/atomic/dispatch.rs:32-67) into a second buffer.  Here each thread owns one ORBIT of
// the gate -- the 1, 2 or 4 amplitudes that only read each other -- loads it once, evaluates the
// same `atomic_op` expression for every member and stores the results in place.  Orbits are
// enumerated by bit insertion: the target bits are inserted as 0 and the control bits as 1 into a
// dense counter, so a gate with c controls touches only 2^(n-c) amplitudes.  Built with
// --fmad=false: on IEEE f64 storage the results are bit-identical to qvnt's non-fast-math
// arithmetic.  Gates whose targets all lie in the five lowest qubits (and whose controls do not)
// run with one amplitude per thread and the orbit partners taken from other lanes by warp shuffles
// (plain_shfl_kernel); the others read an orbit's members from the two (or four) strided halves of
// the state, each a coalesced 16-byte load per thread.  The same kernels serve double-float
// registers for gates the fused engine does not tile (AccDF64 converts on load and store).
#include <algorithm>
#include <vector>

#include "atomic.cuh"
#include "df64.cuh"
#include "kernels.h"

namespace qvnt {

namespace {

// Orbits in flight per thread: four one-amplitude orbits (diagonal gates), two of the others.
template <int SHAPE>
constexpr int unroll_of() { return SHAPE == 1 ? 4 : 2; }
constexpr int kUnroll = 2;  // grid sizing

template <int SHAPE, class Acc>
__global__ void __launch_bounds__(256) plain_gate_kernel(double2* __restrict__ psi, const DevGate g, const Enum e,
                                                         const uint64_t pmask) {
    constexpr int kU = unroll_of<SHAPE>();
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t j0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j0 < e.count; j0 += stride * kU) {
        amp_t v[kU][SHAPE];
        uint64_t base[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            const uint64_t j = j0 + u * stride;
            if (j < e.count) {
                base[u] = enum_index(e, j);
                if (SHAPE == 1) {
                    v[u][0] = Acc::load(psi, base[u]);
                } else if (SHAPE == 2) {
                    v[u][0] = Acc::load(psi, base[u]);
                    v[u][1] = Acc::load(psi, base[u] ^ pmask);
                } else {
                    v[u][0] = Acc::load(psi, base[u]);
                    v[u][1] = Acc::load(psi, base[u] | g.a);
                    v[u][2] = Acc::load(psi, base[u] | g.b);
                    v[u][3] = Acc::load(psi, base[u] | g.a | g.b);
                }
            }
        }
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            const uint64_t j = j0 + u * stride;
            if (j >= e.count) continue;
            const uint64_t i0 = base[u];
            if (SHAPE == 1) {
                const amp_t x = v[u][0];
                Acc::store(psi, i0, atomic_op(g, i0, [&](uint64_t) { return x; }));
            } else if (SHAPE == 2) {
                const amp_t x0 = v[u][0], x1 = v[u][1];
                const uint64_t i1 = i0 ^ pmask;
                auto f = [&](uint64_t k) { return k == i0 ? x0 : x1; };
                const amp_t o0 = atomic_op(g, i0, f);
                const amp_t o1 = atomic_op(g, i1, f);
                Acc::store(psi, i0, o0);
                Acc::store(psi, i1, o1);
            } else {
                const amp_t x0 = v[u][0], x1 = v[u][1], x2 = v[u][2], x3 = v[u][3];
                const uint64_t a = g.a, b = g.b;
                auto f = [&](uint64_t k) {
                    const int s = ((k & a) ? 1 : 0) | ((k & b) ? 2 : 0);
                    return s == 0 ? x0 : (s == 1 ? x1 : (s == 2 ? x2 : x3));
                };
                const amp_t o0 = atomic_op(g, i0, f);
                const amp_t o1 = atomic_op(g, i0 | a, f);
                const amp_t o2 = atomic_op(g, i0 | b, f);
                const amp_t o3 = atomic_op(g, i0 | a | b, f);
                Acc::store(psi, i0, o0);
                Acc::store(psi, i0 | a, o1);
                Acc::store(psi, i0 | b, o2);
                Acc::store(psi, i0 | a | b, o3);
            }
        }
    }
}

// Orbits inside a warp: when every target bit of the gate is below 5 and no control bit is, lane l
// holds amplitude (warp base + l) and the orbit partners of an amplitude sit in lanes l ^ m.  Each
// thread loads its one amplitude (a warp reads 512 contiguous bytes), takes the partners' values
// from their lanes (__shfl_xor_sync), evaluates qvnt's atomic_op for its own index and stores it.
// NP = 1: pairs (i, i ^ m1); NP = 3: quads (i, i ^ m1, i ^ m2, i ^ m1 ^ m2).  e.count is a multiple
// of 32, so a warp is either wholly inside the enumeration or wholly past it.
__device__ __forceinline__ double2 shfl_xor_amp(double2 v, uint32_t m) {
    return make_double2(__shfl_xor_sync(0xffffffffu, v.x, (int)m), __shfl_xor_sync(0xffffffffu, v.y, (int)m));
}

template <int NP, class Acc>
__global__ void __launch_bounds__(256) plain_shfl_kernel(double2* __restrict__ psi, const DevGate g, const Enum e,
                                                         const uint32_t m1, const uint32_t m2) {
    constexpr int U = 4;  // amplitudes in flight per thread
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t j0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j0 < e.count; j0 += stride * U) {
        uint64_t idx[U];
        amp_t x[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint64_t j = j0 + u * stride;
            if (j < e.count) {  // the same for every lane of the warp
                idx[u] = enum_index(e, j);
                x[u] = Acc::load(psi, idx[u]);
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (j0 + u * stride >= e.count) break;
            const uint64_t i = idx[u];
            const amp_t xi = x[u];
            const amp_t y1 = shfl_xor_amp(xi, m1);
            amp_t out;
            if (NP == 1) {
                out = atomic_op(g, i, [&](uint64_t k) { return k == i ? xi : y1; });
            } else {
                const amp_t y2 = shfl_xor_amp(xi, m2);
                const amp_t y3 = shfl_xor_amp(xi, m1 ^ m2);
                out = atomic_op(g, i, [&](uint64_t k) {
                    const uint64_t d = k ^ i;
                    return d == 0 ? xi : (d == m1 ? y1 : (d == m2 ? y2 : y3));
                });
            }
            Acc::store(psi, i, out);
        }
    }
}

// qvnt's own out-of-place gather, for gates whose orbits are not closed (a U2 controlled on its
// own b qubit, which qvnt allows because u2 `acts_on` omits b_mask, u2.rs:70-72).
template <class Acc>
__global__ void __launch_bounds__(256) gather_gate_kernel(const double2* __restrict__ in, double2* __restrict__ out,
                                                          const DevGate g, const uint64_t len) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < len; idx += stride) {
        if ((~idx & g.ctrl) == 0)
            Acc::store(out, idx, atomic_op(g, idx, [&](uint64_t k) { return Acc::load(in, k); }));
        else
            Acc::store(out, idx, Acc::load(in, idx));
    }
}

inline int high_bit(uint64_t m) { return 63 - __builtin_clzll(m); }
inline int low_bit(uint64_t m) { return __builtin_ctzll(m); }

Enum make_enum(uint64_t len, uint64_t inserted, uint64_t ones) {
    Enum e{};
    std::vector<uint32_t> pos;
    for (int p = 0; p < 64; ++p)
        if ((inserted >> p) & 1ull) pos.push_back((uint32_t)p);
    e.nins = (uint32_t)pos.size();
    for (size_t k = 0; k < pos.size(); ++k) e.ins[k] = pos[k];
    e.ones = ones;
    e.count = len >> pos.size();
    return e;
}

unsigned grid_for(uint64_t work, const Geometry& geo, int threads) {
    uint64_t want = (work + (uint64_t)threads * kUnroll - 1) / ((uint64_t)threads * kUnroll);
    uint64_t cap = (uint64_t)geo.sms * geo.blocks_per_sm;
    if (want > cap) want = cap;
    if (want < 1) want = 1;
    return (unsigned)want;
}

template <int NP>
void launch_shfl(int fmt, unsigned grid, cudaStream_t stream, double2* psi, const DevGate& g, const Enum& e, uint32_t m1,
                 uint32_t m2) {
    if (fmt == FMT_DF64)
        plain_shfl_kernel<NP, AccDF64><<<grid, 256, 0, stream>>>(psi, g, e, m1, m2);
    else
        plain_shfl_kernel<NP, AccF64><<<grid, 256, 0, stream>>>(psi, g, e, m1, m2);
}

// The in-warp form applies when the orbit's masks stay inside a lane's five low index bits, the
// controls do not (lane = index bits 0..4), and the enumeration covers whole warps.
bool shfl_fits(uint64_t targets, uint64_t ctrl, uint64_t count) {
    return targets != 0 && targets < 32 && (ctrl & 31ull) == 0 && count >= 32 && (count & 31ull) == 0;
}

template <int SHAPE>
void launch_shape(int fmt, unsigned grid, cudaStream_t stream, double2* psi, const DevGate& g, const Enum& e,
                  uint64_t pmask) {
    if (fmt == FMT_DF64)
        plain_gate_kernel<SHAPE, AccDF64><<<grid, 256, 0, stream>>>(psi, g, e, pmask);
    else
        plain_gate_kernel<SHAPE, AccF64><<<grid, 256, 0, stream>>>(psi, g, e, pmask);
}

}  // namespace

bool plain_gate_is_identity(const DevGate& g) {
    switch (g.kind) {
    case QVNT_GATE_ID:
        return true;
    case QVNT_GATE_X: case QVNT_GATE_Y: case QVNT_GATE_Z: case QVNT_GATE_S: case QVNT_GATE_T:
        return g.a == 0;  // popcount(idx & 0) = 0 everywhere: every output equals its input
    default:
        return false;
    }
}

bool plain_gate_needs_gather(const DevGate& g) { return g.kind == QVNT_GATE_U2 && (g.ctrl & g.b) != 0; }

int launch_plain_gate(double2* psi, int fmt, uint64_t len, const DevGate& g, cudaStream_t stream,
                      const Geometry& geo) {
    const int threads = 256;
    const uint64_t ctrl = g.ctrl;
    switch (g.kind) {
    case QVNT_GATE_Z: case QVNT_GATE_S: case QVNT_GATE_T: case QVNT_GATE_RZ: case QVNT_GATE_RZZ: {
        Enum e = make_enum(len, ctrl, ctrl);
        launch_shape<1>(fmt, grid_for(e.count, geo, threads), stream, psi, g, e, 0);
        break;
    }
    case QVNT_GATE_X: case QVNT_GATE_Y: case QVNT_GATE_RX: case QVNT_GATE_RY: case QVNT_GATE_H1:
    case QVNT_GATE_U1: case QVNT_GATE_RXX: case QVNT_GATE_RYY: {
        const Enum all = make_enum(len, ctrl, ctrl);
        if (shfl_fits(g.a, ctrl, all.count)) {  // pairs (i, i ^ a) inside a warp
            launch_shfl<1>(fmt, grid_for(all.count, geo, threads), stream, psi, g, all, (uint32_t)g.a, 0);
            break;
        }
        const uint64_t pivot = 1ull << high_bit(g.a);
        Enum e = make_enum(len, ctrl | pivot, ctrl);
        launch_shape<2>(fmt, grid_for(e.count, geo, threads), stream, psi, g, e, g.a);
        break;
    }
    case QVNT_GATE_SWAP: case QVNT_GATE_ISWAP: case QVNT_GATE_SQRT_SWAP: case QVNT_GATE_SQRT_ISWAP: {
        // Only members with odd parity of idx & ab change (swap.rs:17): pair (01) <-> (10).
        const uint64_t lo = 1ull << low_bit(g.a);
        Enum e = make_enum(len, ctrl | g.a, ctrl | lo);
        launch_shape<2>(fmt, grid_for(e.count, geo, threads), stream, psi, g, e, g.a);
        break;
    }
    case QVNT_GATE_H2: case QVNT_GATE_U2: {
        const Enum all = make_enum(len, ctrl, ctrl);
        if (shfl_fits(g.a | g.b, ctrl, all.count)) {  // quads (i, i ^ a, i ^ b, i ^ a ^ b) inside a warp
            launch_shfl<3>(fmt, grid_for(all.count, geo, threads), stream, psi, g, all, (uint32_t)g.a, (uint32_t)g.b);
            break;
        }
        Enum e = make_enum(len, ctrl | g.a | g.b, ctrl);
        launch_shape<4>(fmt, grid_for(e.count, geo, threads), stream, psi, g, e, 0);
        break;
    }
    default:
        return QVNT_OK;
    }
    QVNT_CUDA_TRY(cudaGetLastError());
    return QVNT_OK;
}

int launch_gather_gate(const double2* in, double2* out, int fmt, uint64_t len, const DevGate& g, cudaStream_t stream,
                       const Geometry& geo) {
    const int threads = 256;
    if (fmt == FMT_DF64)
        gather_gate_kernel<AccDF64><<<grid_for(len, geo, threads), threads, 0, stream>>>(in, out, g, len);
    else
        gather_gate_kernel<AccF64><<<grid_for(len, geo, threads), threads, 0, stream>>>(in, out, g, len);
    QVNT_CUDA_TRY(cudaGetLastError());
    return QVNT_OK;
}

}  // namespace qvnt
