// TEST INFRASTRUCTURE ONLY: the runner loop of qvnt_gb300/csrc/program.h (the code that
// qvnt_program_run executes) instantiated on the CPU oracle's register, so that its control flow --
// block order, IF conditions, classical-bit updates, resets, draw order, the up-front checks -- is
// checked without a GPU.  tests/test_program_cpu.py builds and drives it.
//
// usage: program_oracle <input> <output>
//   input  (host byte order): u32 q_num, u32 c_num, i32 measure_op, u32 nblocks, u64 state,
//          u64 creg, u64 ngates, u64 trailing, u32 ndraws, u32 zero; qvnt_gate[ngates],
//          qvnt_block[nblocks], f64[ndraws]
//   output: i32 status, u32 draws_used, u64 creg, u64 len, len interleaved complex doubles
#include <cstdarg>
#include <cstdio>
#include <vector>

#include "../oracle/qvnt_oracle.h"
#include "../qvnt_gb300/csrc/program.h"

namespace qvnt {
int set_error(int status, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vfprintf(stderr, fmt, ap);
    fputc('\n', stderr);
    va_end(ap);
    return status;
}
}  // namespace qvnt

namespace {

struct OracleReg {
    uint32_t n;
    uint64_t len;
    std::vector<oc_t> psi, scratch;
    int validate(const qvnt_gate*, size_t) { return QVNT_OK; }
    int apply(const qvnt_gate* g, size_t k) {
        oracle_apply(g, k, psi.data(), scratch.data(), len, 1);
        return QVNT_OK;
    }
    int measure(uint64_t mask, double u01, uint64_t* v) {
        uint64_t idx = 0;
        *v = oracle_measure_mask(psi.data(), len, n, mask, u01, &idx);
        return QVNT_OK;
    }
    int reset_by_mask(uint64_t mask) {
        oracle_reset_by_mask(psi.data(), len, n, mask);
        return QVNT_OK;
    }
};

template <class T>
bool get(FILE* f, T* p, size_t n = 1) {
    return n == 0 || fread(p, sizeof(T), n, f) == n;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc != 3) return 2;
    FILE* in = fopen(argv[1], "rb");
    if (!in) return 3;
    uint32_t q_num, c_num, nblocks, ndraws, zero;
    int32_t measure_op;
    uint64_t state, creg, ngates, trailing;
    if (!get(in, &q_num) || !get(in, &c_num) || !get(in, &measure_op) || !get(in, &nblocks) || !get(in, &state) ||
        !get(in, &creg) || !get(in, &ngates) || !get(in, &trailing) || !get(in, &ndraws) || !get(in, &zero))
        return 4;
    if (q_num > 24) return 5;
    std::vector<qvnt_gate> gates(ngates + 1);
    std::vector<qvnt_block> blocks(nblocks + 1);
    std::vector<double> draws(ndraws + 1);
    if (!get(in, gates.data(), ngates) || !get(in, blocks.data(), nblocks) || !get(in, draws.data(), ndraws)) return 6;
    fclose(in);

    OracleReg reg;
    reg.n = q_num;
    reg.len = oracle_reg_len(q_num);
    reg.psi.resize(reg.len);
    reg.scratch.resize(reg.len);
    oracle_reg_init(q_num, state, reg.psi.data());
    uint32_t used = 0;
    const int32_t st = qvnt::run_program(reg, c_num, measure_op, ngates ? gates.data() : nullptr,
                                         nblocks ? blocks.data() : nullptr, nblocks, trailing,
                                         ndraws ? draws.data() : nullptr, ndraws, &creg, &used);
    FILE* out = fopen(argv[2], "wb");
    if (!out) return 7;
    fwrite(&st, 4, 1, out);
    fwrite(&used, 4, 1, out);
    fwrite(&creg, 8, 1, out);
    fwrite(&reg.len, 8, 1, out);
    fwrite(reg.psi.data(), sizeof(oc_t), reg.len, out);
    fclose(out);
    return 0;
}
