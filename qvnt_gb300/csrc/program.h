// The QASM runner's loop, qvnt's `Sym::finish` (src/qasm/sym.rs:40-74), over any register backend.
//
// A program is qvnt's interpreted form `int::Op(VecDeque<(MultiOp, Sep)>, MultiOp)`
// (src/qasm/int/ext_op.rs:6-16): blocks of gates, each followed by a separator, then a trailing
// gate list.  Per block, in order:
//   NOP            apply the gates
//   MEASURE(q, c)  apply, measure_mask(q), then for the k-th set bit of q and the k-th set bit of c
//                  (zipped, the shorter list ends it) set -- or xor -- classical bit c from the
//                  measured bit q (sym.rs:49-61, `CReg::set` / `CReg::xor`, register/class.rs:89-101)
//   IF(c, v)       apply only when the classical bits under c, packed low to high, equal v
//                  (`CReg::get_by_mask`, class.rs:115-125)
//   RESET(q)       apply, then reset_by_mask(q)
// and the trailing gates last.  Measurements take the caller's uniform draws in order.
//
// Backend: int apply(const qvnt_gate*, size_t); int measure(uint64_t mask, double u01, uint64_t* v);
// int reset_by_mask(uint64_t mask); int validate(const qvnt_gate*, size_t).  Everything is checked
// before the first gate runs, so a rejected program leaves the register and the classical bits as
// they were.
#pragma once

#include <cstdint>

#include "../../include/qvnt_gb300.h"

namespace qvnt {

int set_error(int status, const char* fmt, ...);

// `CReg::get_by_mask` (class.rs:115-125): the bits of value under mask & q_mask, packed.
inline uint64_t creg_get_by_mask(uint64_t value, uint64_t mask, uint32_t c_num) {
    const uint64_t q_mask = c_num >= 64 ? ~0ull : ((1ull << c_num) - 1);
    uint64_t m = mask & q_mask, out = 0;
    for (int idx = 0; m; ++idx, m &= m - 1)
        if (value & (m & (~m + 1))) out |= 1ull << idx;
    return out;
}

// sym.rs:49-61: the k-th set bit of q_arg feeds the k-th set bit of c_arg.
inline uint64_t creg_after_measure(uint64_t value, uint64_t measured, uint64_t q_arg, uint64_t c_arg, int measure_op) {
    uint64_t q = q_arg, c = c_arg;
    while (q && c) {
        const uint64_t qb = q & (~q + 1), cb = c & (~c + 1);
        const bool bit = (measured & qb) != 0;
        if (measure_op == QVNT_MEASURE_XOR) {
            if (bit) value ^= cb;
        } else {
            value = bit ? (value | cb) : (value & ~cb);
        }
        q &= q - 1;
        c &= c - 1;
    }
    return value;
}

template <class Reg>
int run_program(Reg& reg, uint32_t c_num, int measure_op, const qvnt_gate* gates, const qvnt_block* blocks,
                uint32_t nblocks, uint64_t trailing_gates, const double* u01, uint32_t nu01, uint64_t* creg,
                uint32_t* draws_used) {
    if (!creg) return set_error(QVNT_ERR_BAD_ARG, "null classical register");
    if (nblocks && !blocks) return set_error(QVNT_ERR_BAD_ARG, "null block list");
    if (c_num > 64) return set_error(QVNT_ERR_BAD_ARG, "c_num %u > 64", c_num);
    if (measure_op != QVNT_MEASURE_SET && measure_op != QVNT_MEASURE_XOR)
        return set_error(QVNT_ERR_BAD_ARG, "unknown measure op %d", measure_op);
    uint64_t ng = trailing_gates;
    uint32_t nmeasure = 0;
    for (uint32_t b = 0; b < nblocks; ++b) {
        const qvnt_block& k = blocks[b];
        if (k.reserved) return set_error(QVNT_ERR_BAD_ARG, "block %u: reserved field is not zero", b);
        if (k.sep > QVNT_SEP_RESET) return set_error(QVNT_ERR_BAD_ARG, "block %u: unknown separator %u", b, k.sep);
        if (k.gate_count > ~0ull - ng) return set_error(QVNT_ERR_BAD_ARG, "block %u: gate count overflows", b);
        ng += k.gate_count;
        if (k.sep == QVNT_SEP_MEASURE) {
            if (nmeasure >= nu01 || !u01)
                return set_error(QVNT_ERR_BAD_ARG, "block %u: measurement %u has no draw (%u given)", b, nmeasure, nu01);
            if (!(u01[nmeasure] >= 0.0 && u01[nmeasure] < 1.0))
                return set_error(QVNT_ERR_BAD_ARG, "block %u: draw %u is outside [0, 1)", b, nmeasure);
            ++nmeasure;
        }
    }
    if (ng && !gates) return set_error(QVNT_ERR_BAD_ARG, "null gate list");
    if (ng > (uint64_t)SIZE_MAX) return set_error(QVNT_ERR_BAD_ARG, "gate list too long");
    int st = reg.validate(gates, (size_t)ng);
    if (st) return st;

    uint64_t c = *creg, g0 = 0;
    uint32_t d = 0;
    for (uint32_t b = 0; b < nblocks; ++b) {
        const qvnt_block& k = blocks[b];
        const qvnt_gate* op = gates + g0;
        g0 += k.gate_count;
        if (k.sep == QVNT_SEP_IF && creg_get_by_mask(c, k.a, c_num) != k.b) continue;
        if (k.gate_count && (st = reg.apply(op, (size_t)k.gate_count))) break;
        if (k.sep == QVNT_SEP_MEASURE) {
            uint64_t v = 0;
            if ((st = reg.measure(k.a, u01[d++], &v))) break;
            c = creg_after_measure(c, v, k.a, k.b, measure_op);
        } else if (k.sep == QVNT_SEP_RESET) {
            if ((st = reg.reset_by_mask(k.a))) break;
        }
    }
    if (!st && trailing_gates) st = reg.apply(gates + g0, (size_t)trailing_gates);
    *creg = c;
    if (draws_used) *draws_used = d;
    return st;
}

}  // namespace qvnt
