// Host planner of the dense-block engines (precision.cu, tensor64.cu): every qvnt gate lowered to
// its dense matrix on its support (targets and controls), evaluated with qvnt's own atomic formulas
// (atomic.cuh) and the control rule of src/operator/atomic/dispatch.rs:32-47; runs of gates fused
// greedily into BLOCKS of five qubits (a gate may overtake earlier skipped gates only when their
// supports are disjoint), their matrices multiplied in double precision; blocks grouped into PASSES
// over tiles of tile_q qubits (the lowq lowest always among them, so a tile is a set of contiguous
// runs of 2^lowq amplitudes).
#pragma once

#include <algorithm>
#include <cstdint>
#include <vector>

#include "atomic.cuh"
#include "engine.h"

namespace qvnt {
namespace dense {

constexpr int kBQ = 5;         // block qubits
constexpr int kBD = 1 << kBQ;  // block dimension

struct Cd {
    double re, im;
};
inline Cd cmul(Cd a, Cd b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
inline Cd cadd(Cd a, Cd b) { return {a.re + b.re, a.im + b.im}; }

inline uint64_t compress(uint64_t x, const std::vector<int>& sup) {  // global mask -> local bits
    uint64_t r = 0;
    for (size_t j = 0; j < sup.size(); ++j)
        if ((x >> sup[j]) & 1ull) r |= 1ull << j;
    return r;
}

struct LGate {
    uint64_t sup = 0;     // global support mask (<= 5 bits)
    std::vector<Cd> m;    // dense matrix over the support's local basis, row-major
    bool diag = false;    // m is diagonal (such gates commute with each other)
};

// The dense matrix of one gate on its support, from qvnt's own atomic formulas (atomic.cuh) and the
// control rule of dispatch.rs:32-47 (out[i] = f(psi, i) where i has every control bit, else psi[i]).
inline int dense_gate(const qvnt_gate& g, LGate& out) {
    uint64_t tg = g.a_mask;
    if (g.kind == QVNT_GATE_H2 || g.kind == QVNT_GATE_U2) tg |= g.b_mask;
    out.sup = tg | g.ctrl;
    std::vector<int> sup;
    for (int q = 0; q < 64; ++q)
        if ((out.sup >> q) & 1ull) sup.push_back(q);
    if (sup.size() > (size_t)kBQ)
        return set_error(QVNT_ERR_UNSUPPORTED, "gate acts on %zu qubits (targets and controls); dense blocks "
                                               "span at most %d", sup.size(), kBQ);
    qvnt_gate lg = g;
    lg.a_mask = compress(g.a_mask, sup);
    lg.b_mask = compress(g.b_mask, sup);
    lg.ctrl = compress(g.ctrl, sup);
    const DevGate d = decode_gate(lg);
    const uint64_t dim = 1ull << sup.size();
    out.m.assign(dim * dim, Cd{0, 0});
    std::vector<double2> col(dim);
    for (uint64_t cidx = 0; cidx < dim; ++cidx) {
        for (uint64_t i = 0; i < dim; ++i) col[i] = make_double2(i == cidx ? 1.0 : 0.0, 0.0);
        auto psi = [&](uint64_t j) { return col[j]; };
        for (uint64_t r = 0; r < dim; ++r) {
            const double2 v = ((r & lg.ctrl) == lg.ctrl) ? atomic_op(d, r, psi) : col[r];
            out.m[r * dim + cidx] = Cd{v.x, v.y};
        }
    }
    out.diag = true;
    for (uint64_t r = 0; r < dim && out.diag; ++r)
        for (uint64_t cidx = 0; cidx < dim; ++cidx)
            if (r != cidx && (out.m[r * dim + cidx].re != 0.0 || out.m[r * dim + cidx].im != 0.0)) {
                out.diag = false;
                break;
            }
    return QVNT_OK;
}

// Gates as dense factors: the multi-bit X/Y/Z/S/T split into one-qubit factors (they commute), each
// with the gate's controls.
inline int lower_dense(const qvnt_gate* gates, size_t count, std::vector<LGate>& out) {
    out.clear();
    for (size_t i = 0; i < count; ++i) {
        const qvnt_gate& g = gates[i];
        if (g.kind == QVNT_GATE_ID) continue;
        const bool multi = g.kind == QVNT_GATE_X || g.kind == QVNT_GATE_Y || g.kind == QVNT_GATE_Z ||
                           g.kind == QVNT_GATE_S || g.kind == QVNT_GATE_T;
        if (multi && __builtin_popcountll(g.a_mask) > 1) {
            for (int q = 0; q < 64; ++q)
                if ((g.a_mask >> q) & 1ull) {
                    qvnt_gate f = g;
                    f.a_mask = 1ull << q;
                    LGate lg;
                    const int st = dense_gate(f, lg);
                    if (st) return set_error(st, "gate %zu: %s", i, qvnt_last_error());
                    out.push_back(std::move(lg));
                }
            continue;
        }
        LGate lg;
        const int st = dense_gate(g, lg);
        if (st) return set_error(st, "gate %zu: %s", i, qvnt_last_error());
        out.push_back(std::move(lg));
    }
    return QVNT_OK;
}

struct Block {
    uint64_t sup = 0;        // exactly kBQ qubits
    std::vector<Cd> u;       // 32 x 32, row-major, local bit j = j-th qubit of sup (ascending)
};

// U <- (M on the sub-support) * U, for a gate whose support lies inside the block's.
inline void block_apply(Block& b, const LGate& g) {
    std::vector<int> bq;
    for (int q = 0; q < 64; ++q)
        if ((b.sup >> q) & 1ull) bq.push_back(q);
    std::vector<uint32_t> pos;  // local block bit of each gate-support qubit
    for (int q = 0; q < 64; ++q)
        if ((g.sup >> q) & 1ull) pos.push_back((uint32_t)(std::find(bq.begin(), bq.end(), q) - bq.begin()));
    const uint32_t s = (uint32_t)pos.size(), dim = 1u << s;
    uint32_t gm = 0;
    for (uint32_t p : pos) gm |= 1u << p;
    std::vector<uint32_t> dep(dim);
    for (uint32_t x = 0; x < dim; ++x) {
        uint32_t v = 0;
        for (uint32_t j = 0; j < s; ++j)
            if ((x >> j) & 1u) v |= 1u << pos[j];
        dep[x] = v;
    }
    std::vector<Cd> tmp(dim);
    for (uint32_t col = 0; col < (uint32_t)kBD; ++col)
        for (uint32_t rest = 0; rest < (uint32_t)kBD; ++rest) {
            if (rest & gm) continue;
            for (uint32_t r = 0; r < dim; ++r) {
                Cd acc{0, 0};
                for (uint32_t cc = 0; cc < dim; ++cc)
                    acc = cadd(acc, cmul(g.m[r * dim + cc], b.u[(rest | dep[cc]) * kBD + col]));
                tmp[r] = acc;
            }
            for (uint32_t r = 0; r < dim; ++r) b.u[(rest | dep[r]) * kBD + col] = tmp[r];
        }
}

// One candidate block seeded by gate `seed` (its support starts the block's qubit set): scanning the
// unplaced gates in order from `first`, a gate joins when its support fits the five qubits and it
// commutes with each gate skipped so far (their supports are disjoint, or both are diagonal).  Empty
// when the seed itself cannot join (it does not commute with a gate skipped before it).
inline std::vector<size_t> block_trial(const std::vector<LGate>& lg, const std::vector<char>& done, size_t first,
                                       size_t seed, uint64_t all) {
    std::vector<size_t> members;
    uint64_t S = lg[seed].sup, skipped_nd = 0, skipped_d = 0;  // skipped supports: non-diagonal, diagonal
    size_t scanned = 0;
    for (size_t j = first; j < lg.size() && scanned < 512; ++j) {
        if (done[j]) continue;
        ++scanned;
        const uint64_t G = lg[j].sup;
        const uint64_t must_miss = lg[j].diag ? skipped_nd : (skipped_nd | skipped_d);
        if (!(G & must_miss) && __builtin_popcountll(S | G) <= kBQ) {
            S |= G;
            members.push_back(j);
        } else {
            if (j == seed) return {};
            (lg[j].diag ? skipped_d : skipped_nd) |= G;
            if ((skipped_nd & all) == all && j > seed) break;  // nothing later can pass the skipped gates
        }
    }
    return members;
}

// Blocks: each is the largest of the candidate blocks seeded by the first `seeds` unplaced gates (the
// tensor engine takes 96, which plans QFT-heavy circuits into fewer blocks; the precision engine 48,
// whose passes pair blocks and pair the blocks of the smaller search better).
inline void make_blocks(const std::vector<LGate>& lg, uint32_t L, std::vector<Block>& blocks, size_t seeds = 48) {
    const size_t kSeeds = seeds;
    blocks.clear();
    const size_t n = lg.size();
    std::vector<char> done(n, 0);
    size_t first = 0;
    const uint64_t all = L >= 64 ? ~0ull : ((1ull << L) - 1ull);
    while (true) {
        while (first < n && done[first]) ++first;
        if (first >= n) break;
        std::vector<size_t> members;
        size_t tried = 0;
        for (size_t seed = first; seed < n && tried < kSeeds; ++seed) {
            if (done[seed]) continue;
            ++tried;
            std::vector<size_t> m = block_trial(lg, done, first, seed, all);
            if (m.size() > members.size()) members.swap(m);
        }
        uint64_t S = 0;
        for (size_t j : members) {
            S |= lg[j].sup;
            done[j] = 1;
        }
        for (int q = 0; q < (int)L && __builtin_popcountll(S) < kBQ; ++q) S |= 1ull << q;  // pad to 5 qubits
        Block b;
        b.sup = S;
        b.u.assign(kBD * kBD, Cd{0, 0});
        for (int i = 0; i < kBD; ++i) b.u[i * kBD + i] = Cd{1, 0};
        for (size_t j : members) block_apply(b, lg[j]);
        blocks.push_back(std::move(b));
    }
}

struct PPlan {
    uint64_t qmask;
    std::vector<size_t> members;  // block indices
};

// Passes: each holds up to max_per_pass blocks whose supports fit the tile's free qubits.
inline int make_passes(const std::vector<Block>& blocks, uint32_t L, int tile_q, uint32_t lowq, size_t max_per_pass,
                       std::vector<PPlan>& passes) {
    passes.clear();
    const int kt = std::min<int>(tile_q, (int)L);  // tile qubits
    const size_t n = blocks.size();
    std::vector<char> done(n, 0);
    size_t first = 0;
    const uint64_t low = (1ull << lowq) - 1ull;
    while (true) {
        while (first < n && done[first]) ++first;
        if (first >= n) break;
        PPlan p;
        uint64_t Q = low & ((L >= 64) ? ~0ull : ((1ull << L) - 1ull)), blocked = 0;
        size_t scanned = 0;
        for (size_t j = first; j < n && scanned < 64 && p.members.size() < max_per_pass; ++j) {
            if (done[j]) continue;
            ++scanned;
            const uint64_t S = blocks[j].sup;
            if (!(S & blocked) && __builtin_popcountll(Q | S) <= kt) {
                Q |= S;
                p.members.push_back(j);
                done[j] = 1;
            } else {
                blocked |= S;
            }
        }
        if (p.members.empty())  // cannot happen with lowq <= tile_q - 5: a block always fits an empty tile
            return set_error(QVNT_ERR_UNSUPPORTED, "dense-block planner could not place block %zu", first);
        for (uint32_t q = 0; q < L && __builtin_popcountll(Q) < kt; ++q) Q |= 1ull << q;
        p.qmask = Q;
        passes.push_back(std::move(p));
    }
    return QVNT_OK;
}


}  // namespace dense
}  // namespace qvnt
