// Gate builders and names: qvnt's `op::` constructors for hosts that do not run qvnt's Rust code.
//
// A Rust host keeps qvnt's own `op::`/`MultiOp` and lowers `SingleOp`s itself; C, C++ and Python
// callers build the same gate lists here.  Each builder follows the reference function it names.
#include <charconv>
#include <cmath>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "../../include/qvnt_gb300.h"

namespace qvnt {
int set_error(int status, const char* fmt, ...);
uint64_t gate_acts_on(const qvnt_gate& g);
int gate_check_masks(const qvnt_gate& g);
}  // namespace qvnt

using namespace qvnt;

namespace {

inline unsigned popc(uint64_t x) { return (unsigned)__builtin_popcountll(x); }

bool is_rotation(uint32_t k) {
    return k == QVNT_GATE_RX || k == QVNT_GATE_RY || k == QVNT_GATE_RZ || k == QVNT_GATE_RXX || k == QVNT_GATE_RYY ||
           k == QVNT_GATE_RZZ;
}

// float-cmp 0.8 `approx_eq!(f64, x, y, ulps = 2)` (src/math/approx_cmp.rs:5-10).
bool approx_eq_real(double x, double y) {
    if (x == y) return true;
    if (std::fabs(x - y) <= 2.220446049250313e-16) return true;
    if ((x < 0) != (y < 0)) return false;
    int64_t bx, by;
    memcpy(&bx, &x, 8);
    memcpy(&by, &y, 8);
    int64_t d = bx - by;
    return (d < 0 ? -d : d) <= 2;
}

struct Cx {
    double re, im;
};
Cx cmul(Cx a, Cx b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
Cx cadd(Cx a, Cx b) { return {a.re + b.re, a.im + b.im}; }
Cx cconj(Cx a) { return {a.re, -a.im}; }
double nsq(Cx a) { return a.re * a.re + a.im * a.im; }

// `is_unitary_m1` (src/math/matrix.rs:24-30).
bool is_unitary_m1(const double* m) {
    Cx u[4];
    for (int k = 0; k < 4; ++k) u[k] = {m[2 * k], m[2 * k + 1]};
    const double e00 = nsq(u[0]) + nsq(u[1]);
    const double e11 = nsq(u[2]) + nsq(u[3]);
    const Cx e01 = cadd(cmul(u[0], cconj(u[2])), cmul(u[1], cconj(u[3])));
    return approx_eq_real(e00, 1.0) && approx_eq_real(e11, 1.0) && approx_eq_real(e01.re + e01.im, 0.0);
}

// `hermitian_mul` / `is_unitary_m2` (src/math/matrix.rs:37-73).
Cx herm_mul(int i, int j, const Cx* u) {
    i = (i << 2) & 0xf;
    j = (j << 2) & 0xf;
    if (i == j) return {(nsq(u[0 | i]) + nsq(u[1 | i])) + (nsq(u[2 | i]) + nsq(u[3 | i])), 0.0};
    return cadd(cadd(cmul(u[0 | i], cconj(u[0 | j])), cmul(u[1 | i], cconj(u[1 | j]))),
                cadd(cmul(u[2 | i], cconj(u[2 | j])), cmul(u[3 | i], cconj(u[3 | j]))));
}

bool is_unitary_m2(const double* m) {
    Cx u[16];
    for (int k = 0; k < 16; ++k) u[k] = {m[2 * k], m[2 * k + 1]};
    for (int d = 0; d < 4; ++d)
        if (!approx_eq_real(herm_mul(d, d, u).re, 1.0)) return false;
    for (int a = 0; a < 4; ++a)
        for (int b = a + 1; b < 4; ++b) {
            Cx e = herm_mul(a, b, u);
            if (!approx_eq_real(e.re + e.im, 0.0)) return false;
        }
    return true;
}

// Rust `{}` of f64: shortest round-trip digits, never an exponent.
std::string rust_display(double x) {
    if (std::isnan(x)) return "NaN";
    if (std::isinf(x)) return x > 0 ? "inf" : "-inf";
    char buf[512];
    auto res = std::to_chars(buf, buf + sizeof buf, x, std::chars_format::fixed);
    return std::string(buf, res.ptr);
}

// Rust `{:?}` of f64: like Display with a forced ".0", exponent form outside [1e-4, 1e16).
std::string rust_debug(double x) {
    if (std::isnan(x)) return "NaN";
    if (std::isinf(x)) return x > 0 ? "inf" : "-inf";
    const double ax = std::fabs(x);
    char buf[512];
    if (ax != 0.0 && (ax < 1e-4 || ax >= 1e16)) {
        auto res = std::to_chars(buf, buf + sizeof buf, x, std::chars_format::scientific);
        std::string s(buf, res.ptr);
        size_t e = s.find('e');
        std::string mant = s.substr(0, e), ex = s.substr(e + 1);
        bool neg = !ex.empty() && ex[0] == '-';
        size_t p = (ex[0] == '+' || ex[0] == '-') ? 1 : 0;
        while (p + 1 < ex.size() && ex[p] == '0') ++p;
        return mant + "e" + (neg ? "-" : "") + ex.substr(p);
    }
    auto res = std::to_chars(buf, buf + sizeof buf, x, std::chars_format::fixed);
    std::string s(buf, res.ptr);
    if (s.find('.') == std::string::npos) s += ".0";
    return s;
}

std::string cx_debug(double re, double im) {
    return "Complex { re: " + rust_debug(re) + ", im: " + rust_debug(im) + " }";
}

std::string atomic_name(const qvnt_gate& g) {
    const std::string a = std::to_string(g.a_mask);
    auto rot = [&](const char* n) {
        // `format!("RX{}({})", a_mask, 2.0 * self.phase.arg())` (rx.rs:26-28)
        return std::string(n) + a + "(" + rust_display(2.0 * std::atan2(g.phase[1], g.phase[0])) + ")";
    };
    switch (g.kind) {
    case QVNT_GATE_ID: return "Id";
    case QVNT_GATE_X: return "X" + a;
    case QVNT_GATE_Y: return "Y" + a;
    case QVNT_GATE_Z: return "Z" + a;
    case QVNT_GATE_S: return "S" + a;
    case QVNT_GATE_T: return "T" + a;
    case QVNT_GATE_RX: return rot("RX");
    case QVNT_GATE_RY: return rot("RY");
    case QVNT_GATE_RZ: return rot("RZ");
    case QVNT_GATE_RXX: return rot("RXX");
    case QVNT_GATE_RYY: return rot("RYY");
    case QVNT_GATE_RZZ: return rot("RZZ");
    case QVNT_GATE_H1: return "H" + a;
    case QVNT_GATE_H2: return "H" + std::to_string(g.a_mask | g.b_mask);
    case QVNT_GATE_SWAP: return "SWAP" + a;
    case QVNT_GATE_ISWAP: return "iSWAP" + a;
    case QVNT_GATE_SQRT_SWAP: return "sqrt(SWAP" + a + ")";
    case QVNT_GATE_SQRT_ISWAP: return "sqrt(iSWAP" + a + ")";
    case QVNT_GATE_U1: {  // u1.rs:27-33
        std::string s = "U" + a + "[[";
        for (int r = 0; r < 2; ++r) {
            if (r) s += "], [";
            for (int c = 0; c < 2; ++c) {
                if (c) s += ", ";
                s += cx_debug(g.matrix[2 * (2 * r + c)], g.matrix[2 * (2 * r + c) + 1]);
            }
        }
        return s + "]]";
    }
    case QVNT_GATE_U2: {  // u2.rs:51-62
        std::string s = "U" + std::to_string(g.a_mask | g.b_mask) + "[[";
        for (int r = 0; r < 4; ++r) {
            if (r) s += "], [";
            for (int c = 0; c < 4; ++c) {
                if (c) s += ", ";
                s += cx_debug(g.matrix[2 * (4 * r + c)], g.matrix[2 * (4 * r + c) + 1]);
            }
        }
        return s + "]]";
    }
    default: return "?";
    }
}

struct GateList {
    qvnt_gate* out;
    size_t cap;
    size_t n = 0;
    void push(const qvnt_gate& g) {
        if (out && n < cap) out[n] = g;
        ++n;
    }
};

int make(uint32_t kind, uint64_t a, uint64_t b, double angle, const double* m, qvnt_gate* out) {
    return qvnt_gate_make(kind, a, b, angle, m, out);
}

void build_h(uint64_t mask, GateList& gl) {  // src/operator/multi/h.rs:14-45
    qvnt_gate g;
    const unsigned count = popc(mask);
    if (count == 0) return;
    if (count == 1) {
        make(QVNT_GATE_H1, mask, 0, 0, nullptr, &g);
        gl.push(g);
        return;
    }
    uint64_t i0 = 1, i1 = 0;
    bool is_first = true;
    while (i0 != 0 && i0 <= mask) {
        if (i0 & mask) {
            if (is_first) {
                i1 = i0;
                is_first = false;
            } else {
                make(QVNT_GATE_H2, i0, i1, 0, nullptr, &g);
                gl.push(g);
                is_first = true;
            }
        }
        i0 <<= 1;
    }
    if (!is_first) {
        make(QVNT_GATE_H1, i1, 0, 0, nullptr, &g);
        gl.push(g);
    }
}

void build_qft(uint64_t mask, GateList& gl) {  // src/operator/multi/qft.rs:4-33
    const unsigned count = popc(mask);
    if (count == 0) return;
    if (count == 1) {
        build_h(mask, gl);
        return;
    }
    std::vector<uint64_t> vec;
    for (int i = 0; i < 64; ++i)
        if ((1ull << i) & mask) vec.push_back(1ull << i);
    qvnt_gate g;
    for (unsigned i = 0; i + 1 < count; ++i) {
        build_h(vec[i], gl);
        for (unsigned j = 1; j < count - i; ++j) {
            // rz(vec[i + j], PI * 0.5f64.powi(j)).c(vec[i])
            make(QVNT_GATE_RZ, vec[i + j], 0, M_PI * std::ldexp(1.0, -(int)j), nullptr, &g);
            g.ctrl = vec[i];
            gl.push(g);
        }
    }
    build_h(vec[count - 1], gl);
}

}  // namespace

extern "C" {

int qvnt_gate_make(uint32_t kind, uint64_t a_mask, uint64_t b_mask, double angle, const double* matrix,
                   qvnt_gate* out) {
    if (!out) return set_error(QVNT_ERR_BAD_ARG, "null output pointer");
    if (kind >= QVNT_GATE_KIND_COUNT) return set_error(QVNT_ERR_BAD_ARG, "unknown gate kind %u", kind);
    qvnt_gate g;
    memset(&g, 0, sizeof g);
    g.kind = kind;
    g.a_mask = a_mask;
    if (kind == QVNT_GATE_H2 || kind == QVNT_GATE_U2) g.b_mask = b_mask;
    if (is_rotation(kind)) {
        double ph = angle;
        ph /= 2.;  // rx.rs:11 (`phase *= 0.5` in rxx.rs:12 rounds identically)
        g.phase[0] = std::cos(ph);
        g.phase[1] = std::sin(ph);
    }
    if (kind == QVNT_GATE_U1 || kind == QVNT_GATE_U2) {
        if (!matrix) return set_error(QVNT_ERR_BAD_ARG, "U1/U2 need a matrix");
        memcpy(g.matrix, matrix, (kind == QVNT_GATE_U1 ? 8 : 32) * sizeof(double));
    }
    int st = gate_check_masks(g);
    if (st) return st;
    if (kind == QVNT_GATE_U1 && !is_unitary_m1(g.matrix)) return set_error(QVNT_ERR_BAD_ARG, "matrix is not unitary");
    if (kind == QVNT_GATE_U2 && !is_unitary_m2(g.matrix)) return set_error(QVNT_ERR_BAD_ARG, "matrix is not unitary");
    *out = g;
    return QVNT_OK;
}

int qvnt_gate_dgr(qvnt_gate* g) {
    if (!g) return set_error(QVNT_ERR_BAD_ARG, "null gate");
    switch (g->kind) {
    case QVNT_GATE_S: case QVNT_GATE_T: case QVNT_GATE_ISWAP: case QVNT_GATE_SQRT_SWAP: case QVNT_GATE_SQRT_ISWAP:
        g->dagger = !g->dagger;  // s.rs:39-44, t.rs:49-54, i_swap.rs:55-60, ...
        break;
    case QVNT_GATE_RX: case QVNT_GATE_RY: case QVNT_GATE_RZ: case QVNT_GATE_RXX: case QVNT_GATE_RYY:
    case QVNT_GATE_RZZ:
        g->phase[0] = -g->phase[0];  // rx.rs:42-47: `phase: -self.phase`
        g->phase[1] = -g->phase[1];
        break;
    case QVNT_GATE_U1: {  // matrix.rs `inverse_unitary_m1`: conjugate transpose
        double m[8];
        memcpy(m, g->matrix, sizeof m);
        for (int r = 0; r < 2; ++r)
            for (int c = 0; c < 2; ++c) {
                g->matrix[2 * (2 * r + c)] = m[2 * (2 * c + r)];
                g->matrix[2 * (2 * r + c) + 1] = -m[2 * (2 * c + r) + 1];
            }
        break;
    }
    case QVNT_GATE_U2: {  // matrix.rs `inverse_unitary_m2`
        double m[32];
        memcpy(m, g->matrix, sizeof m);
        for (int r = 0; r < 4; ++r)
            for (int c = 0; c < 4; ++c) {
                g->matrix[2 * (4 * r + c)] = m[2 * (4 * c + r)];
                g->matrix[2 * (4 * r + c) + 1] = -m[2 * (4 * c + r) + 1];
            }
        break;
    }
    default:
        break;
    }
    return QVNT_OK;
}

int qvnt_gate_c(qvnt_gate* g, uint64_t c_mask) {
    if (!g) return set_error(QVNT_ERR_BAD_ARG, "null gate");
    if ((gate_acts_on(*g) | g->ctrl) & c_mask)
        return set_error(QVNT_ERR_BAD_MASK, "control mask %llu overlaps %llu", (unsigned long long)c_mask,
                         (unsigned long long)(gate_acts_on(*g) | g->ctrl));
    g->ctrl |= c_mask;
    return QVNT_OK;
}

uint64_t qvnt_gate_act_on(const qvnt_gate* g) { return g ? (gate_acts_on(*g) | g->ctrl) : 0; }

int qvnt_gate_name(const qvnt_gate* g, char* buf, size_t cap, size_t* needed) {
    if (!g) return set_error(QVNT_ERR_BAD_ARG, "null gate");
    std::string s = atomic_name(*g);
    if (g->ctrl) s = "C" + std::to_string(g->ctrl) + "_" + s;  // single/mod.rs:72-78
    if (needed) *needed = s.size();
    if (buf && cap) {
        size_t n = s.size() < cap - 1 ? s.size() : cap - 1;
        memcpy(buf, s.data(), n);
        buf[n] = 0;
    }
    return QVNT_OK;
}

int qvnt_op_h(uint64_t mask, qvnt_gate* out, size_t cap, size_t* count) {
    GateList gl{out, cap};
    build_h(mask, gl);
    if (count) *count = gl.n;
    return QVNT_OK;
}

int qvnt_op_qft(uint64_t mask, qvnt_gate* out, size_t cap, size_t* count) {
    GateList gl{out, cap};
    build_qft(mask, gl);
    if (count) *count = gl.n;
    return QVNT_OK;
}

int qvnt_op_qft_swapped(uint64_t mask, qvnt_gate* out, size_t cap, size_t* count) {  // qft.rs:35-52
    GateList gl{out, cap};
    build_qft(mask, gl);
    std::vector<uint64_t> vec;
    for (uint64_t i = 1; i != 0 && i <= mask; i <<= 1)
        if (i & mask) vec.push_back(i);
    const size_t len = vec.size();
    qvnt_gate g;
    for (size_t i = 0; i < (len >> 1); ++i) {
        make(QVNT_GATE_SWAP, vec[i] | vec[len - i - 1], 0, 0, nullptr, &g);
        gl.push(g);
    }
    if (count) *count = gl.n;
    return QVNT_OK;
}

int qvnt_op_u3(double the, double phi, double lam, uint64_t mask, qvnt_gate* out, size_t cap, size_t* count) {
    if (popc(mask) != 1) return set_error(QVNT_ERR_BAD_MASK, "Mask should contain 1 bit!");
    GateList gl{out, cap};
    qvnt_gate g;
    make(QVNT_GATE_RZ, mask, 0, lam, nullptr, &g);  // operator/mod.rs:499-501
    gl.push(g);
    make(QVNT_GATE_RY, mask, 0, the, nullptr, &g);
    gl.push(g);
    make(QVNT_GATE_RZ, mask, 0, phi, nullptr, &g);
    gl.push(g);
    if (count) *count = gl.n;
    return QVNT_OK;
}

int qvnt_op_u2(double phi, double lam, uint64_t mask, qvnt_gate* out, size_t cap, size_t* count) {
    return qvnt_op_u3(M_PI_2, phi, lam, mask, out, cap, count);  // operator/mod.rs:480-482
}

int qvnt_ops_dgr(qvnt_gate* gates, size_t count) {  // multi/mod.rs:120-123
    if (!gates && count) return set_error(QVNT_ERR_BAD_ARG, "null gate list");
    for (size_t i = 0; i < count / 2; ++i) std::swap(gates[i], gates[count - 1 - i]);
    for (size_t i = 0; i < count; ++i) qvnt_gate_dgr(&gates[i]);
    return QVNT_OK;
}

// Seeded synthetic layers (the generator of qvnt_gb300/circuits.py `random_layers`, here for the
// batch and serving workloads that need thousands of circuits): per layer one gate from
// {h, s, t, u3(th, phi, lam)} on every qubit, 15 two-qubit gates from {rxx, ryy, rzz, swap, i_swap,
// sqrt_i_swap} on random distinct pairs, 3 Toffolis x(t).c(c1 | c2).  The SplitMix64 state is
// advanced in place, also when `out` is too small (the gates are then counted, not written).
int qvnt_workload_random_layers(uint32_t n, uint32_t depth, uint64_t* rng_state, qvnt_gate* out, size_t cap,
                                size_t* count) {
    if (!rng_state) return set_error(QVNT_ERR_BAD_ARG, "null rng state");
    if (n < 3 || n > 63) return set_error(QVNT_ERR_BAD_ARG, "n = %u: the layer generator needs 3..63 qubits", n);
    uint64_t& st = *rng_state;
    auto next = [&]() {
        st += 0x9E3779B97F4A7C15ull;
        uint64_t z = st;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    };
    auto uniform = [&]() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); };
    auto below = [&](uint64_t m) { return next() % m; };
    const double two_pi = 2.0 * M_PI;
    GateList gl{out, cap};
    qvnt_gate g;
    for (uint32_t layer = 0; layer < depth; ++layer) {
        for (uint32_t q = 0; q < n; ++q) {
            const uint64_t m = 1ull << q;
            switch (below(4)) {
            case 0: build_h(m, gl); break;
            case 1: make(QVNT_GATE_S, m, 0, 0, nullptr, &g); gl.push(g); break;
            case 2: make(QVNT_GATE_T, m, 0, 0, nullptr, &g); gl.push(g); break;
            default: {
                const double th = two_pi * uniform(), ph = two_pi * uniform(), la = two_pi * uniform();
                make(QVNT_GATE_RZ, m, 0, la, nullptr, &g);  // u3 = rz(la) ry(th) rz(ph), mod.rs:499-501
                gl.push(g);
                make(QVNT_GATE_RY, m, 0, th, nullptr, &g);
                gl.push(g);
                make(QVNT_GATE_RZ, m, 0, ph, nullptr, &g);
                gl.push(g);
            }
            }
        }
        for (int i = 0; i < 15; ++i) {
            const uint64_t a = below(n);
            uint64_t b = below(n - 1);
            if (b >= a) ++b;
            const uint64_t ab = (1ull << a) | (1ull << b);
            const uint64_t kind = below(6);
            if (kind < 3) {
                const uint32_t kinds[3] = {QVNT_GATE_RXX, QVNT_GATE_RYY, QVNT_GATE_RZZ};
                make(kinds[kind], ab, 0, two_pi * uniform(), nullptr, &g);
            } else {
                const uint32_t kinds[3] = {QVNT_GATE_SWAP, QVNT_GATE_ISWAP, QVNT_GATE_SQRT_ISWAP};
                make(kinds[kind - 3], ab, 0, 0, nullptr, &g);
            }
            gl.push(g);
        }
        for (int i = 0; i < 3; ++i) {
            const uint64_t t = below(n);
            uint64_t c1 = below(n - 1);
            if (c1 >= t) ++c1;
            uint64_t c2 = below(n);
            while (c2 == t || c2 == c1) c2 = below(n);
            make(QVNT_GATE_X, 1ull << t, 0, 0, nullptr, &g);
            g.ctrl = (1ull << c1) | (1ull << c2);
            gl.push(g);
        }
    }
    if (count) *count = gl.n;
    return QVNT_OK;
}

int qvnt_ops_c(qvnt_gate* gates, size_t count, uint64_t c_mask) {  // multi/mod.rs:125-132
    if (!gates && count) return set_error(QVNT_ERR_BAD_ARG, "null gate list");
    uint64_t act = 0;
    for (size_t i = 0; i < count; ++i) act |= gate_acts_on(gates[i]) | gates[i].ctrl;
    if (act & c_mask)
        return set_error(QVNT_ERR_BAD_MASK, "control mask %llu overlaps %llu", (unsigned long long)c_mask,
                         (unsigned long long)act);
    for (size_t i = 0; i < count; ++i) gates[i].ctrl |= c_mask;
    return QVNT_OK;
}

}  // extern "C"
