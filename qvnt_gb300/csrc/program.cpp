// qvnt_program_run: the QASM runner's loop (program.h) on a device register.
#include "program.h"

namespace qvnt {
int validate_gate(const qvnt_gate& g, uint64_t len);
}  // namespace qvnt

namespace {

struct DeviceReg {
    qvnt_reg* reg;
    uint64_t len;
    int validate(const qvnt_gate* g, size_t n) {
        for (size_t k = 0; k < n; ++k) {
            const int st = qvnt::validate_gate(g[k], len);
            if (st) return qvnt::set_error(st, "gate %zu: %s", k, qvnt_last_error());
        }
        return QVNT_OK;
    }
    int apply(const qvnt_gate* g, size_t n) { return qvnt_reg_apply(reg, g, n); }
    int measure(uint64_t mask, double u01, uint64_t* v) { return qvnt_reg_measure_mask(reg, mask, u01, v); }
    int reset_by_mask(uint64_t mask) { return qvnt_reg_reset_by_mask(reg, mask); }
};

}  // namespace

extern "C" int qvnt_program_run(qvnt_reg* reg, uint32_t c_num, int measure_op, const qvnt_gate* gates,
                                const qvnt_block* blocks, uint32_t nblocks, uint64_t trailing_gates,
                                const double* u01, uint32_t nu01, uint64_t* creg, uint32_t* draws_used) {
    DeviceReg d{reg, 0};
    const int st = qvnt_reg_len(reg, &d.len);
    if (st) return st;
    return qvnt::run_program(d, c_num, measure_op, gates, blocks, nblocks, trailing_gates, u01, nu01, creg,
                             draws_used);
}
