// Fused engine: runs of gates applied to shared-memory tiles, one HBM round trip per pass.
//
// qvnt applies every SingleOp as a full sweep over the state (src/operator/multi/mod.rs:97-114).
// Here a host planner groups consecutive gates into PASSES.  A pass picks a set Q of k tile qubits
// (always containing the lowest qubits, so each tile is read as contiguous runs); a tile is the
// 2^k amplitudes that share all non-Q index bits.  Every CTA loads a tile into shared memory,
// applies the pass's gates there, and writes it back once.  A gate joins a pass when its target
// qubits lie in Q; its controls may lie anywhere (a control outside Q is a per-tile predicate),
// and diagonal gates (Z, S, T, RZ, RZZ) join any pass, their phase taking the non-Q index bits
// from the tile base.  Gates may move ahead of deferred gates only when both are diagonal or their
// qubit supports are disjoint, so the result equals the in-order product up to rounding.
#include <algorithm>
#include <cstring>
#include <vector>

#include "atomic.cuh"
#include "engine.h"
#include "kernels.h"

namespace qvnt {

namespace {

constexpr int kFusedThreads = 512;
constexpr uint32_t kDefaultK = 12;
constexpr size_t kLookahead = 4096;

struct LGate {
    DevGate g;        // masks in virtual-local coordinates (tile bit j = local bit j)
    Enum e;           // orbit enumeration inside the tile
    uint64_t gctrl;   // control bits outside the tile: gate applies where base & gctrl == gctrl
    uint64_t a_nl;    // diagonal gates: bits of a outside the tile
    uint64_t pmask;   // pair partner mask (shape 2)
    uint32_t shape;   // 1 diagonal, 2 pair, 4 quad
    uint32_t pad;
};

struct TileGeom {
    uint32_t k;         // tile qubits
    uint32_t c;         // length of the contiguous low run (tile qubits 0..c-1 are qubits 0..c-1)
    uint32_t nhigh;     // k - c
    uint32_t pad;
    uint32_t high[kFusedMaxK];  // global positions of tile bits c..k-1
    uint32_t qpos[kFusedMaxK];  // global positions of all k tile bits
    Enum tiles;         // tile t -> base index (tile qubits inserted as 0)
};

__device__ __forceinline__ void apply_local(amp_t* __restrict__ tile, const LGate& G, uint64_t extra) {
    const uint64_t count = G.e.count;
    if (G.shape == 1) {
        for (uint64_t j = threadIdx.x; j < count; j += kFusedThreads) {
            const uint64_t l = enum_index(G.e, j);
            const amp_t x = tile[l];
            tile[l] = atomic_op(G.g, l | extra, [&](uint64_t) { return x; });
        }
    } else if (G.shape == 2) {
        const uint64_t pm = G.pmask;
        for (uint64_t j = threadIdx.x; j < count; j += kFusedThreads) {
            const uint64_t l0 = enum_index(G.e, j), l1 = l0 ^ pm;
            const amp_t x0 = tile[l0], x1 = tile[l1];
            auto f = [&](uint64_t q) { return q == l0 ? x0 : x1; };
            const amp_t o0 = atomic_op(G.g, l0, f);
            const amp_t o1 = atomic_op(G.g, l1, f);
            tile[l0] = o0;
            tile[l1] = o1;
        }
    } else {
        const uint64_t a = G.g.a, b = G.g.b;
        for (uint64_t j = threadIdx.x; j < count; j += kFusedThreads) {
            const uint64_t l0 = enum_index(G.e, j);
            const amp_t x0 = tile[l0], x1 = tile[l0 | a], x2 = tile[l0 | b], x3 = tile[l0 | a | b];
            auto f = [&](uint64_t q) {
                const int s = ((q & a) ? 1 : 0) | ((q & b) ? 2 : 0);
                return s == 0 ? x0 : (s == 1 ? x1 : (s == 2 ? x2 : x3));
            };
            const amp_t o0 = atomic_op(G.g, l0, f);
            const amp_t o1 = atomic_op(G.g, l0 | a, f);
            const amp_t o2 = atomic_op(G.g, l0 | b, f);
            const amp_t o3 = atomic_op(G.g, l0 | a | b, f);
            tile[l0] = o0;
            tile[l0 | a] = o1;
            tile[l0 | b] = o2;
            tile[l0 | a | b] = o3;
        }
    }
}

__global__ void __launch_bounds__(kFusedThreads) fused_pass_kernel(amp_t* __restrict__ psi,
                                                                   const LGate* __restrict__ gates,
                                                                   uint32_t ngates, const TileGeom tg) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    amp_t* tile = reinterpret_cast<amp_t*>(smem_raw);
    const uint32_t T = 1u << tg.k;
    uint64_t* seg = reinterpret_cast<uint64_t*>(tile + T);
    const uint32_t nseg = 1u << tg.nhigh;
    const uint32_t cmask = (1u << tg.c) - 1u;
    for (uint32_t s = threadIdx.x; s < nseg; s += kFusedThreads) {
        uint64_t off = 0;
        for (uint32_t j = 0; j < tg.nhigh; ++j)
            if ((s >> j) & 1u) off |= 1ull << tg.high[j];
        seg[s] = off;
    }
    __syncthreads();
    for (uint64_t t = blockIdx.x; t < tg.tiles.count; t += gridDim.x) {
        const uint64_t base = enum_index(tg.tiles, t);
        for (uint32_t l = threadIdx.x; l < T; l += kFusedThreads)
            tile[l] = psi[base | seg[l >> tg.c] | (l & cmask)];
        __syncthreads();
        for (uint32_t gi = 0; gi < ngates; ++gi) {
            const LGate& G = gates[gi];
            if ((base & G.gctrl) != G.gctrl) continue;
            const uint64_t extra = G.a_nl ? (((1ull << __popcll(base & G.a_nl)) - 1ull) << tg.k) : 0ull;
            apply_local(tile, G, extra);
            __syncthreads();
        }
        for (uint32_t l = threadIdx.x; l < T; l += kFusedThreads)
            psi[base | seg[l >> tg.c] | (l & cmask)] = tile[l];
        __syncthreads();
    }
}

inline unsigned popc(uint64_t x) { return (unsigned)__builtin_popcountll(x); }

bool is_diag(uint32_t kind) {
    return kind == QVNT_GATE_Z || kind == QVNT_GATE_S || kind == QVNT_GATE_T || kind == QVNT_GATE_RZ ||
           kind == QVNT_GATE_RZZ;
}

struct GInfo {
    uint64_t targets = 0;
    uint64_t touched = 0;
    bool diag = false;
    bool skip = false;
    bool standalone = false;
};

GInfo classify(const qvnt_gate& g, uint32_t k, uint32_t c) {
    GInfo r;
    const DevGate d = decode_gate(g);
    if (plain_gate_is_identity(d)) {
        r.skip = true;
        return r;
    }
    r.diag = is_diag(g.kind);
    if (!r.diag) r.targets = (g.kind == QVNT_GATE_H2 || g.kind == QVNT_GATE_U2) ? (g.a_mask | g.b_mask) : g.a_mask;
    r.touched = r.targets | g.ctrl | (r.diag ? g.a_mask : 0);
    if (plain_gate_needs_gather(d)) r.standalone = true;
    const uint64_t low = (1ull << c) - 1ull;
    if (popc(r.targets & ~low) > k - c) r.standalone = true;
    return r;
}

// Maps global index bits to tile-local positions through `qpos`.
uint64_t compress(uint64_t m, const uint32_t* qpos, uint32_t k) {
    uint64_t r = 0;
    for (uint32_t j = 0; j < k; ++j)
        if ((m >> qpos[j]) & 1ull) r |= 1ull << j;
    return r;
}

Enum local_enum(uint32_t k, uint64_t inserted, uint64_t ones) {
    Enum e{};
    uint32_t n = 0;
    for (uint32_t p = 0; p < k; ++p)
        if ((inserted >> p) & 1ull) e.ins[n++] = p;
    e.nins = n;
    e.ones = ones;
    e.count = (1ull << k) >> n;
    return e;
}

LGate lower_gate(const qvnt_gate& g, const uint32_t* qpos, uint32_t k, uint64_t qmask) {
    LGate L;
    memset(&L, 0, sizeof L);
    DevGate d = decode_gate(g);
    const uint64_t ctrl_l = compress(g.ctrl & qmask, qpos, k);
    L.gctrl = g.ctrl & ~qmask;
    d.ctrl = ctrl_l;
    if (is_diag(g.kind)) {
        const uint64_t a_l = compress(g.a_mask & qmask, qpos, k);
        L.a_nl = g.a_mask & ~qmask;
        // Non-tile bits of a become popcount(a_nl) virtual bits above the tile (set per tile).
        d.a = a_l | (((1ull << popc(L.a_nl)) - 1ull) << k);
        L.shape = 1;
        L.e = local_enum(k, ctrl_l, ctrl_l);
    } else {
        d.a = compress(g.a_mask, qpos, k);
        d.b = compress(d.b, qpos, k);
        switch (g.kind) {
        case QVNT_GATE_SWAP: case QVNT_GATE_ISWAP: case QVNT_GATE_SQRT_SWAP: case QVNT_GATE_SQRT_ISWAP: {
            const uint64_t lo = d.a & (~d.a + 1ull);
            L.shape = 2;
            L.pmask = d.a;
            L.e = local_enum(k, ctrl_l | d.a, ctrl_l | lo);
            break;
        }
        case QVNT_GATE_H2: case QVNT_GATE_U2:
            L.shape = 4;
            L.e = local_enum(k, ctrl_l | d.a | d.b, ctrl_l);
            break;
        default: {
            const uint64_t pivot = 1ull << (63 - __builtin_clzll(d.a));
            L.shape = 2;
            L.pmask = d.a;
            L.e = local_enum(k, ctrl_l | pivot, ctrl_l);
            break;
        }
        }
    }
    L.g = d;
    return L;
}

struct Pass {
    bool standalone = false;
    size_t gate = 0;  // standalone: index into the caller's list
    uint64_t qmask = 0;
    std::vector<size_t> members;
};

uint32_t index_bits(uint64_t len) { return (uint32_t)__builtin_ctzll(len); }

}  // namespace

void FusedState::release() {
    if (d_buf) cudaFree(d_buf);
    if (h_buf) cudaFreeHost(h_buf);
    d_buf = nullptr;
    h_buf = nullptr;
    d_bytes = h_bytes = 0;
}

int apply_fused(qvnt_reg* r, const qvnt_gate* gates, size_t count) {
    const uint32_t L = index_bits(r->len);
    uint32_t k = r->fusion_k ? r->fusion_k : kDefaultK;
    if (k > L) k = L;
    uint32_t c = k >= 10 ? 4 : (k >= 4 ? 2 : k);
    if (c > k) c = k;
    const uint64_t low = (1ull << c) - 1ull;
    const uint64_t all = (L >= 64) ? ~0ull : ((1ull << L) - 1ull);

    // ---- plan ----
    std::vector<GInfo> info(count);
    for (size_t i = 0; i < count; ++i) info[i] = classify(gates[i], k, c);
    std::vector<char> done(count, 0);
    std::vector<Pass> passes;
    size_t first = 0;
    while (true) {
        while (first < count && (done[first] || info[first].skip)) ++first;
        if (first >= count) break;
        if (info[first].standalone) {
            Pass p;
            p.standalone = true;
            p.gate = first;
            passes.push_back(p);
            done[first] = 1;
            continue;
        }
        Pass p;
        uint64_t Q = low;
        uint32_t free_slots = k - c;
        uint64_t block_nd = 0, block_d = 0;
        size_t scanned = 0;
        for (size_t j = first; j < count && scanned < kLookahead; ++j) {
            if (done[j] || info[j].skip) continue;
            ++scanned;
            const GInfo& g = info[j];
            const bool conflict = g.diag ? (g.touched & block_nd) != 0 : (g.touched & (block_nd | block_d)) != 0;
            if (!conflict && !g.standalone) {
                const uint64_t need = g.targets & ~Q;
                if (popc(need) <= free_slots) {
                    Q |= need;
                    free_slots -= popc(need);
                    p.members.push_back(j);
                    done[j] = 1;
                    continue;
                }
            }
            if (g.diag) block_d |= g.touched;
            else block_nd |= g.touched;
            if ((block_nd & all) == all) break;
        }
        // Fill unused tile slots with the lowest free qubits: longer contiguous runs per tile.
        for (uint32_t b = 0; b < L && free_slots > 0; ++b)
            if (!((Q >> b) & 1ull)) {
                Q |= 1ull << b;
                --free_slots;
            }
        p.qmask = Q;
        passes.push_back(p);
    }
    if (passes.empty()) return QVNT_OK;

    // ---- lower and upload ----
    size_t nl = 0;
    for (const Pass& p : passes) nl += p.members.size();
    const size_t bytes = std::max<size_t>(nl, 1) * sizeof(LGate);
    if (r->fused.h_buf && r->fused.h_bytes < bytes) {
        cudaStreamSynchronize(r->stream);
        cudaFreeHost(r->fused.h_buf);
        r->fused.h_buf = nullptr;
    }
    if (!r->fused.h_buf) {
        QVNT_CUDA_TRY(cudaMallocHost(&r->fused.h_buf, bytes));
        r->fused.h_bytes = bytes;
    } else {
        // The previous upload from this pinned buffer must have completed before it is rewritten.
        QVNT_CUDA_TRY(cudaStreamSynchronize(r->stream));
    }
    if (r->fused.d_bytes < bytes) {
        QVNT_CUDA_TRY(cudaStreamSynchronize(r->stream));
        if (r->fused.d_buf) cudaFree(r->fused.d_buf);
        r->fused.d_buf = nullptr;
        cudaError_t e = cudaMalloc(&r->fused.d_buf, bytes);
        if (e != cudaSuccess) return set_cuda_error(e, "cudaMalloc(pass descriptors)");
        r->fused.d_bytes = bytes;
    }
    LGate* hl = reinterpret_cast<LGate*>(r->fused.h_buf);
    std::vector<TileGeom> geoms(passes.size());
    std::vector<size_t> offs(passes.size());
    size_t at = 0;
    for (size_t pi = 0; pi < passes.size(); ++pi) {
        const Pass& p = passes[pi];
        if (p.standalone) continue;
        TileGeom tg;
        memset(&tg, 0, sizeof tg);
        uint32_t n = 0;
        for (uint32_t b = 0; b < L; ++b)
            if ((p.qmask >> b) & 1ull) tg.qpos[n++] = b;
        tg.k = n;
        uint32_t run = 0;
        while (run < n && tg.qpos[run] == run) ++run;
        tg.c = run;
        tg.nhigh = n - run;
        for (uint32_t j = 0; j < tg.nhigh; ++j) tg.high[j] = tg.qpos[run + j];
        Enum te{};
        te.nins = n;
        for (uint32_t j = 0; j < n; ++j) te.ins[j] = tg.qpos[j];
        te.ones = 0;
        te.count = r->len >> n;
        tg.tiles = te;
        geoms[pi] = tg;
        offs[pi] = at;
        for (size_t m : p.members) hl[at++] = lower_gate(gates[m], tg.qpos, n, p.qmask);
    }
    if (at) QVNT_CUDA_TRY(cudaMemcpyAsync(r->fused.d_buf, hl, at * sizeof(LGate), cudaMemcpyHostToDevice, r->stream));

    // ---- launch ----
    const LGate* dl = reinterpret_cast<const LGate*>(r->fused.d_buf);
    for (size_t pi = 0; pi < passes.size(); ++pi) {
        const Pass& p = passes[pi];
        cudaEvent_t stop = nullptr;  // timing covers the fused-pass kernel only
        int st = QVNT_OK;
        if (p.standalone) {
            DevGate d = decode_gate(gates[p.gate]);
            if (plain_gate_needs_gather(d)) {
                st = reg_ensure_alt(r);
                if (st) return st;
                st = launch_gather_gate(r->psi, r->alt, r->len, d, r->stream, r->ctx->geo);
                std::swap(r->psi, r->alt);
            } else {
                st = launch_plain_gate(r->psi, r->len, d, r->stream, r->ctx->geo);
            }
            if (st) return st;
        } else {
            const TileGeom& tg = geoms[pi];
            const size_t smem = ((size_t)1 << tg.k) * sizeof(amp_t) + ((size_t)1 << tg.nhigh) * sizeof(uint64_t);
            if (smem > 48 * 1024)
                QVNT_CUDA_TRY(cudaFuncSetAttribute(fused_pass_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   (int)smem));
            const int per_sm = std::max(1, (int)((size_t)(r->ctx->smem_optin ? r->ctx->smem_optin : 48 * 1024) / smem));
            uint64_t grid = (uint64_t)r->ctx->geo.sms * std::min(per_sm, 4);
            if (grid > tg.tiles.count) grid = tg.tiles.count;
            st = timing_begin(r, &stop);
            if (st) return st;
            fused_pass_kernel<<<(unsigned)grid, kFusedThreads, smem, r->stream>>>(r->psi, dl + offs[pi],
                                                                                 (uint32_t)p.members.size(), tg);
            QVNT_CUDA_TRY(cudaGetLastError());
        }
        st = timing_end(r, stop);
        if (st) return st;
        r->launches += 1;
        r->passes += 1;
    }
    return QVNT_OK;
}

}  // namespace qvnt
