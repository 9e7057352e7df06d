// Gate-list wire formats: qvnt's operator names as text, and a lossless binary stream.
//
// Text: `MultiOp`'s `{:?}` (src/operator/multi/mod.rs:90-94, a debug list of `SingleOp::name`,
// src/operator/single/mod.rs:72-78), e.g. "[C4_X123, RX1(1.23456), sqrt(iSWAP3)]".  The names are
// what a qvnt program prints or logs; they do not carry everything a gate holds (see qvnt_ops_parse).
//
// Binary: every field of every qvnt_gate, bit for bit, for moving gate lists and whole serving
// requests between processes and hosts.  Layout (all integers little-endian whatever the host):
//
//   "QVNW"  u8 version (1)  u8 type (1 gate list, 2 request)  u16 zero
//   varint ngates
//   type 2 only: varint q_num, varint state, varint submit flags, varint ncalls
//   ngates gate records:
//     u8 kind, u8 fields (bit 0 dagger, 1 b_mask follows, 2 ctrl follows, 3 phase follows,
//                         4 matrix[0..8) follows, 5 matrix[8..32) follows; other bits zero)
//     varint a_mask, [varint b_mask], [varint ctrl], [2 f64], [8 f64], [24 f64]
//     (an absent field is all zero; an f64 is its IEEE bits as a u64)
//   type 2 only, ncalls call records: u8 op, varint gate_count, varint mask, f64 u01
//   u32 CRC-32 of every byte before it
//
// varint: LEB128, 7 bits per byte, low group first, at most 10 bytes.  CRC-32: the reflected
// polynomial 0xEDB88320 with initial value and final xor 0xFFFFFFFF (ISO-HDLC / zlib's crc32).
#include <charconv>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/qvnt_gb300.h"

namespace qvnt {
int set_error(int status, const char* fmt, ...);
}  // namespace qvnt

using qvnt::set_error;

namespace {

constexpr uint8_t kVersion = 1;
constexpr uint8_t kTypeGates = 1;
constexpr uint8_t kTypeRequest = 2;
constexpr uint8_t kFieldDagger = 1, kFieldB = 2, kFieldCtrl = 4, kFieldPhase = 8, kFieldM0 = 16, kFieldM1 = 32;

// ------------------------------------------------------------------------------------- CRC-32

struct CrcTable {
    uint32_t t[256];
    CrcTable() {
        for (uint32_t i = 0; i < 256; ++i) {
            uint32_t c = i;
            for (int k = 0; k < 8; ++k) c = (c & 1) ? (0xEDB88320u ^ (c >> 1)) : (c >> 1);
            t[i] = c;
        }
    }
};

uint32_t crc32(const uint8_t* p, size_t n) {
    static const CrcTable tab;
    uint32_t c = 0xFFFFFFFFu;
    for (size_t i = 0; i < n; ++i) c = tab.t[(c ^ p[i]) & 0xFF] ^ (c >> 8);
    return c ^ 0xFFFFFFFFu;
}

// ------------------------------------------------------------------------------------- encoder

struct Out {
    std::vector<uint8_t> b;
    void u8(uint8_t v) { b.push_back(v); }
    void u32(uint32_t v) {
        for (int i = 0; i < 4; ++i) b.push_back((uint8_t)(v >> (8 * i)));
    }
    void u64(uint64_t v) {
        for (int i = 0; i < 8; ++i) b.push_back((uint8_t)(v >> (8 * i)));
    }
    void var(uint64_t v) {
        while (v >= 0x80) {
            b.push_back((uint8_t)(v | 0x80));
            v >>= 7;
        }
        b.push_back((uint8_t)v);
    }
    void f64(double x) {
        uint64_t u;
        memcpy(&u, &x, 8);
        u64(u);
    }
};

bool any_bits(const double* p, int n) {
    for (int i = 0; i < n; ++i) {
        uint64_t u;
        memcpy(&u, p + i, 8);
        if (u) return true;
    }
    return false;
}

int put_gates(Out& o, const qvnt_gate* g, uint64_t n) {
    for (uint64_t i = 0; i < n; ++i) {
        if (g[i].kind >= QVNT_GATE_KIND_COUNT) return set_error(QVNT_ERR_BAD_ARG, "gate %llu: kind %u", (unsigned long long)i, g[i].kind);
        if (g[i].dagger > 1) return set_error(QVNT_ERR_BAD_ARG, "gate %llu: dagger %u", (unsigned long long)i, g[i].dagger);
        uint8_t f = 0;
        if (g[i].dagger) f |= kFieldDagger;
        if (g[i].b_mask) f |= kFieldB;
        if (g[i].ctrl) f |= kFieldCtrl;
        if (any_bits(g[i].phase, 2)) f |= kFieldPhase;
        if (any_bits(g[i].matrix, 8)) f |= kFieldM0;
        if (any_bits(g[i].matrix + 8, 24)) f |= kFieldM1;
        o.u8((uint8_t)g[i].kind);
        o.u8(f);
        o.var(g[i].a_mask);
        if (f & kFieldB) o.var(g[i].b_mask);
        if (f & kFieldCtrl) o.var(g[i].ctrl);
        if (f & kFieldPhase) {
            o.f64(g[i].phase[0]);
            o.f64(g[i].phase[1]);
        }
        if (f & kFieldM0)
            for (int k = 0; k < 8; ++k) o.f64(g[i].matrix[k]);
        if (f & kFieldM1)
            for (int k = 8; k < 32; ++k) o.f64(g[i].matrix[k]);
    }
    return QVNT_OK;
}

void header(Out& o, uint8_t type) {
    o.u8('Q');
    o.u8('V');
    o.u8('N');
    o.u8('W');
    o.u8(kVersion);
    o.u8(type);
    o.u8(0);
    o.u8(0);
}

int finish(Out& o, uint8_t* buf, size_t cap, size_t* len) {
    o.u32(crc32(o.b.data(), o.b.size()));
    *len = o.b.size();
    if (buf && cap >= o.b.size()) memcpy(buf, o.b.data(), o.b.size());
    return QVNT_OK;
}

// ------------------------------------------------------------------------------------- decoder

struct In {
    const uint8_t* p;
    size_t n, at = 0;
    bool fail = false;
    const char* why = nullptr;
    bool need(size_t k) {
        if (fail) return false;
        if (n - at < k) {
            fail = true;
            why = "truncated";
            return false;
        }
        return true;
    }
    uint8_t u8() { return need(1) ? p[at++] : 0; }
    uint64_t u64() {
        if (!need(8)) return 0;
        uint64_t v = 0;
        for (int i = 0; i < 8; ++i) v |= (uint64_t)p[at + i] << (8 * i);
        at += 8;
        return v;
    }
    uint64_t var() {
        uint64_t v = 0;
        for (int i = 0; i < 10; ++i) {
            if (!need(1)) return 0;
            const uint8_t c = p[at++];
            if (i == 9 && c > 1) break;  // more than 64 bits
            v |= (uint64_t)(c & 0x7F) << (7 * i);
            if (!(c & 0x80)) return v;
        }
        fail = true;
        why = "varint longer than 64 bits";
        return 0;
    }
    double f64() {
        const uint64_t u = u64();
        double x;
        memcpy(&x, &u, 8);
        return x;
    }
};

// Checks the frame (magic, version, type, CRC) and leaves `in` after the 8-byte header, with the
// CRC bytes excluded from its length.
int open_frame(In& in, uint8_t type) {
    if (!in.p && in.n) return set_error(QVNT_ERR_BAD_ARG, "null buffer");
    if (in.n < 12) return set_error(QVNT_ERR_BAD_ARG, "wire stream of %zu bytes is too short", in.n);
    if (memcmp(in.p, "QVNW", 4) != 0) return set_error(QVNT_ERR_BAD_ARG, "not a gate wire stream (magic)");
    if (in.p[4] != kVersion) return set_error(QVNT_ERR_BAD_ARG, "wire version %u (this library reads %u)", in.p[4], kVersion);
    if (in.p[5] != type)
        return set_error(QVNT_ERR_BAD_ARG, "wire stream type %u, expected %u", in.p[5], type);
    if (in.p[6] || in.p[7]) return set_error(QVNT_ERR_BAD_ARG, "wire header reserved bytes are not zero");
    uint32_t stored = 0;
    for (int i = 0; i < 4; ++i) stored |= (uint32_t)in.p[in.n - 4 + i] << (8 * i);
    if (crc32(in.p, in.n - 4) != stored) return set_error(QVNT_ERR_BAD_ARG, "wire stream CRC mismatch");
    in.n -= 4;
    in.at = 8;
    return QVNT_OK;
}

// Decodes ngates records; writes the first `cap` of them to out (when out is not null).
int get_gates(In& in, uint64_t ngates, qvnt_gate* out, size_t cap) {
    for (uint64_t i = 0; i < ngates; ++i) {
        qvnt_gate g;
        memset(&g, 0, sizeof g);
        g.kind = in.u8();
        const uint8_t f = in.u8();
        if (in.fail) break;
        if (g.kind >= QVNT_GATE_KIND_COUNT) return set_error(QVNT_ERR_BAD_ARG, "gate %llu: kind %u", (unsigned long long)i, g.kind);
        if (f & ~0x3F) return set_error(QVNT_ERR_BAD_ARG, "gate %llu: unknown field bits 0x%x", (unsigned long long)i, f);
        g.dagger = (f & kFieldDagger) ? 1 : 0;
        g.a_mask = in.var();
        if (f & kFieldB) g.b_mask = in.var();
        if (f & kFieldCtrl) g.ctrl = in.var();
        if (f & kFieldPhase) {
            g.phase[0] = in.f64();
            g.phase[1] = in.f64();
        }
        if (f & kFieldM0)
            for (int k = 0; k < 8; ++k) g.matrix[k] = in.f64();
        if (f & kFieldM1)
            for (int k = 8; k < 32; ++k) g.matrix[k] = in.f64();
        if (in.fail) break;
        if (out && i < cap) out[i] = g;
    }
    if (in.fail) return set_error(QVNT_ERR_BAD_ARG, "wire stream: %s at byte %zu", in.why, in.at);
    return QVNT_OK;
}

// ------------------------------------------------------------------------------------- text parser

struct Text {
    const char* s;
    size_t n, at = 0;
    const char* why = nullptr;
    size_t why_at = 0;

    bool error(const char* w) {
        if (!why) {
            why = w;
            why_at = at;
        }
        return false;
    }
    void ws() {
        while (at < n && (s[at] == ' ' || s[at] == '\t' || s[at] == '\n' || s[at] == '\r')) ++at;
    }
    bool peek(const char* lit) const {
        const size_t k = strlen(lit);
        return n - at >= k && memcmp(s + at, lit, k) == 0;
    }
    bool eat(const char* lit) {
        if (!peek(lit)) return false;
        at += strlen(lit);
        return true;
    }
    bool expect(const char* lit) {
        ws();
        return eat(lit) || error("unexpected character");
    }
    bool uint(uint64_t* v) {
        const char* b = s + at;
        auto r = std::from_chars(b, s + n, *v, 10);
        if (r.ptr == b) return error("expected a mask (decimal integer)");
        if (r.ec == std::errc::result_out_of_range) return error("mask does not fit 64 bits");
        at += (size_t)(r.ptr - b);
        return true;
    }
    // A Rust `{}` or `{:?}` f64: "-1.5", "0.0000001", "1e-7", "1.2e16"; NaN and infinities are
    // rejected (no valid gate holds them).
    bool real(double* x) {
        ws();
        const char* b = s + at;
        size_t k = 0;
        if (k < n - at && b[k] == '-') ++k;
        if (k >= n - at || b[k] < '0' || b[k] > '9') return error("expected a finite number");
        auto r = std::from_chars(b, s + n, *x, std::chars_format::general);
        if (r.ptr == b || r.ec != std::errc()) return error("expected a finite number");
        at += (size_t)(r.ptr - b);
        return true;
    }
    bool complex(double* re, double* im) {
        return expect("Complex") && expect("{") && expect("re") && expect(":") && real(re) && expect(",") &&
               expect("im") && expect(":") && real(im) && expect("}");
    }
    // `[[a, b], [c, d]]` or the 4x4 form; *dim gets 2 or 4.  Row-major, as u1.rs:27-33 and
    // u2.rs:51-62 print them.
    bool matrix(double* m, int* dim) {
        if (!expect("[")) return false;
        int rows = 0, cols = -1;
        for (;;) {
            if (!expect("[")) return false;
            int c = 0;
            for (;;) {
                if (rows >= 4 || c >= 4) return error("matrix larger than 4x4");
                double re, im;
                if (!complex(&re, &im)) return false;
                m[2 * (rows * 4 + c)] = re;
                m[2 * (rows * 4 + c) + 1] = im;
                ++c;
                ws();
                if (eat("]")) break;
                if (!expect(",")) return false;
            }
            if (cols >= 0 && c != cols) return error("ragged matrix");
            cols = c;
            ++rows;
            ws();
            if (eat("]")) break;
            if (!expect(",")) return false;
        }
        if (rows != cols || (rows != 2 && rows != 4)) return error("matrix is not 2x2 or 4x4");
        *dim = rows;
        return true;
    }
};

int lowest_bit(uint64_t m) { return m ? __builtin_ctzll(m) : -1; }

// One `SingleOp::name`: ["C" ctrl "_"] atomic name.
bool parse_one(Text& t, qvnt_gate* g) {
    t.ws();
    const size_t start = t.at;
    uint64_t ctrl = 0;
    if (t.peek("C") && t.at + 1 < t.n && t.s[t.at + 1] >= '0' && t.s[t.at + 1] <= '9') {
        ++t.at;
        if (!t.uint(&ctrl) || !(t.eat("_") || t.error("expected '_' after the control mask"))) return false;
    }
    struct Named {
        const char* lit;
        uint32_t kind;
        bool angle;
    };
    // Longest literal first where one is a prefix of another (RXX / RX, SWAP / S, ...).
    static const Named named[] = {
        {"sqrt(iSWAP", QVNT_GATE_SQRT_ISWAP, false}, {"sqrt(SWAP", QVNT_GATE_SQRT_SWAP, false},
        {"iSWAP", QVNT_GATE_ISWAP, false},          {"SWAP", QVNT_GATE_SWAP, false},
        {"RXX", QVNT_GATE_RXX, true},               {"RYY", QVNT_GATE_RYY, true},
        {"RZZ", QVNT_GATE_RZZ, true},               {"RX", QVNT_GATE_RX, true},
        {"RY", QVNT_GATE_RY, true},                 {"RZ", QVNT_GATE_RZ, true},
        {"Id", QVNT_GATE_ID, false},                {"X", QVNT_GATE_X, false},
        {"Y", QVNT_GATE_Y, false},                  {"Z", QVNT_GATE_Z, false},
        {"S", QVNT_GATE_S, false},                  {"T", QVNT_GATE_T, false},
        {"H", QVNT_GATE_H1, false},                 {"U", QVNT_GATE_U1, false},
    };
    const Named* hit = nullptr;
    for (const Named& nm : named)
        if (t.eat(nm.lit)) {
            hit = &nm;
            break;
        }
    if (!hit) return t.error("unknown operator name");
    uint32_t kind = hit->kind;
    uint64_t mask = 0, a = 0, b = 0;
    double angle = 0.0, m[32] = {0};
    if (kind != QVNT_GATE_ID && !t.uint(&mask)) return false;
    a = mask;
    if (kind == QVNT_GATE_SQRT_SWAP || kind == QVNT_GATE_SQRT_ISWAP) {
        if (!(t.eat(")") || t.error("expected ')'"))) return false;
    } else if (hit->angle) {
        if (!(t.eat("(") || t.error("expected '('")) || !t.real(&angle) || !t.expect(")")) return false;
    } else if (kind == QVNT_GATE_H1) {
        // "H3" is h2::Op (h2.rs:40-42); a and b as op::h pairs them (multi/h.rs:14-45): a the
        // higher bit, b the lower.  H2 is symmetric in a and b.
        if (__builtin_popcountll(mask) == 2) {
            kind = QVNT_GATE_H2;
            b = 1ull << lowest_bit(mask);
            a = mask & ~b;
        }
    } else if (kind == QVNT_GATE_U1) {
        int dim = 0;
        if (!t.matrix(m, &dim)) return false;
        if (dim == 4) {
            // The name holds a | b only; a is taken as the lower bit, b the higher (the order the
            // reference's own u2 tests use, u2.rs:90-130).  The matrix is in that (a, b) layout.
            kind = QVNT_GATE_U2;
            if (__builtin_popcountll(mask) != 2) return t.error("a 4x4 unitary needs a two-bit mask");
            a = 1ull << lowest_bit(mask);
            b = mask & ~a;
        } else {
            // Rows of 4 were filled; compact the 2x2 into matrix[0..8).
            double c[8] = {m[0], m[1], m[2], m[3], m[8], m[9], m[10], m[11]};
            memset(m, 0, sizeof m);
            memcpy(m, c, sizeof c);
        }
    }
    qvnt_gate out;
    const bool dense = kind == QVNT_GATE_U1 || kind == QVNT_GATE_U2;
    const int st = qvnt_gate_make(kind, a, b, angle, dense ? m : nullptr, &out);
    if (st != QVNT_OK) {
        t.at = start;
        return t.error(kind == QVNT_GATE_U1 || kind == QVNT_GATE_U2 ? "invalid mask or matrix not unitary"
                                                                    : "invalid mask for this operator");
    }
    if (ctrl) {
        if (qvnt_gate_c(&out, ctrl) != QVNT_OK) {
            t.at = start;
            return t.error("control mask overlaps the operator's mask");
        }
    }
    *g = out;
    return true;
}

// `[name, name, ...]` (the MultiOp `{:?}` list) into out.
bool parse_list(Text& t, std::vector<qvnt_gate>& out) {
    if (!t.expect("[")) return false;
    t.ws();
    if (t.eat("]")) return true;
    for (;;) {
        qvnt_gate g;
        if (!parse_one(t, &g)) return false;
        out.push_back(g);
        t.ws();
        if (t.eat("]")) return true;
        if (!t.expect(",")) return false;
    }
}

// Rust `{:b}` of a usize: binary digits, no prefix.
bool binary(Text& t, uint64_t* v) {
    t.ws();
    const size_t start = t.at;
    uint64_t x = 0;
    while (t.at < t.n && (t.s[t.at] == '0' || t.s[t.at] == '1')) {
        if (t.at - start >= 64) return t.error("binary number longer than 64 bits");
        x = (x << 1) | (uint64_t)(t.s[t.at] - '0');
        ++t.at;
    }
    if (t.at == start) return t.error("expected a binary number");
    *v = x;
    return true;
}

std::string binary_string(uint64_t v) {
    if (!v) return "0";
    std::string s;
    for (; v; v >>= 1) s.insert(s.begin(), (char)('0' + (v & 1)));
    return s;
}

int list_name(const qvnt_gate* g, size_t n, std::string* out) {
    size_t need = 0;
    int st = qvnt_ops_name(g, n, nullptr, 0, &need);
    if (st) return st;
    std::vector<char> buf(need + 1);
    st = qvnt_ops_name(g, n, buf.data(), buf.size(), &need);
    if (st) return st;
    out->assign(buf.data(), need);
    return QVNT_OK;
}

}  // namespace

extern "C" {

int qvnt_ops_parse(const char* text, size_t len, qvnt_gate* out, size_t cap, size_t* count) {
    if (!count) return set_error(QVNT_ERR_BAD_ARG, "null count pointer");
    if (!text && len) return set_error(QVNT_ERR_BAD_ARG, "null text");
    Text t{text, len};
    size_t n = 0;
    bool ok = true;
    t.ws();
    if (t.peek("[")) {
        std::vector<qvnt_gate> list;
        ok = parse_list(t, list);
        for (size_t i = 0; ok && i < list.size(); ++i)
            if (out && i < cap) out[i] = list[i];
        n = list.size();
    } else {
        qvnt_gate g;
        if ((ok = parse_one(t, &g))) {
            if (out && cap) out[0] = g;
            n = 1;
        }
    }
    if (ok) {
        t.ws();
        if (t.at != t.n) ok = t.error("trailing characters");
    }
    if (!ok) return set_error(QVNT_ERR_BAD_ARG, "operator name: %s at byte %zu", t.why, t.why_at);
    *count = n;
    return QVNT_OK;
}

int qvnt_ops_name(const qvnt_gate* gates, size_t count, char* buf, size_t cap, size_t* needed) {
    if (count && !gates) return set_error(QVNT_ERR_BAD_ARG, "null gate list");
    std::string s = "[";  // `f.debug_list().entries(..)` (multi/mod.rs:90-94)
    std::vector<char> one(256);
    for (size_t i = 0; i < count; ++i) {
        size_t need = 0;
        int st = qvnt_gate_name(&gates[i], one.data(), one.size(), &need);
        if (st == QVNT_OK && need + 1 > one.size()) {
            one.resize(need + 1);
            st = qvnt_gate_name(&gates[i], one.data(), one.size(), &need);
        }
        if (st != QVNT_OK) return st;
        if (i) s += ", ";
        s.append(one.data(), need);
    }
    s += "]";
    if (needed) *needed = s.size();
    if (buf && cap) {
        const size_t k = s.size() < cap - 1 ? s.size() : cap - 1;
        memcpy(buf, s.data(), k);
        buf[k] = 0;
    }
    return QVNT_OK;
}

int qvnt_wire_encode_gates(const qvnt_gate* gates, size_t count, uint8_t* buf, size_t cap, size_t* len) {
    if (!len) return set_error(QVNT_ERR_BAD_ARG, "null length pointer");
    if (count && !gates) return set_error(QVNT_ERR_BAD_ARG, "null gate list");
    Out o;
    header(o, kTypeGates);
    o.var(count);
    const int st = put_gates(o, gates, count);
    if (st) return st;
    return finish(o, buf, cap, len);
}

int qvnt_wire_decode_gates(const uint8_t* buf, size_t len, qvnt_gate* out, size_t cap, size_t* count) {
    if (!count) return set_error(QVNT_ERR_BAD_ARG, "null count pointer");
    In in{buf, len};
    int st = open_frame(in, kTypeGates);
    if (st) return st;
    const uint64_t n = in.var();
    // Every record takes at least 3 bytes: a count beyond that is corrupt (and must not drive
    // the loop below for 2^64 iterations).
    if (!in.fail && n > (in.n - in.at) / 3) return set_error(QVNT_ERR_BAD_ARG, "wire stream: gate count %llu exceeds the stream", (unsigned long long)n);
    st = get_gates(in, n, out, cap);
    if (st) return st;
    if (in.at != in.n) return set_error(QVNT_ERR_BAD_ARG, "wire stream: %zu trailing bytes", in.n - in.at);
    *count = (size_t)n;
    return QVNT_OK;
}

int qvnt_wire_encode_request(uint32_t q_num, uint64_t state, int flags, const qvnt_gate* gates, size_t ngates,
                             const qvnt_call* calls, uint32_t ncalls, uint8_t* buf, size_t cap, size_t* len) {
    if (!len) return set_error(QVNT_ERR_BAD_ARG, "null length pointer");
    if (ngates && !gates) return set_error(QVNT_ERR_BAD_ARG, "null gate list");
    if (ncalls && !calls) return set_error(QVNT_ERR_BAD_ARG, "null call list");
    if (flags < 0) return set_error(QVNT_ERR_BAD_ARG, "negative flags");
    uint64_t applied = 0;
    for (uint32_t c = 0; c < ncalls; ++c) {
        if (calls[c].op != QVNT_CALL_APPLY && calls[c].op != QVNT_CALL_MEASURE)
            return set_error(QVNT_ERR_BAD_ARG, "call %u: unknown op %u", c, calls[c].op);
        if (calls[c].reserved) return set_error(QVNT_ERR_BAD_ARG, "call %u: reserved field is not zero", c);
        if (calls[c].op == QVNT_CALL_APPLY) applied += calls[c].gate_count;
    }
    if (applied != ngates)
        return set_error(QVNT_ERR_BAD_ARG, "the calls apply %llu gates, the list holds %zu", (unsigned long long)applied, ngates);
    Out o;
    header(o, kTypeRequest);
    o.var(ngates);
    o.var(q_num);
    o.var(state);
    o.var((uint64_t)flags);
    o.var(ncalls);
    int st = put_gates(o, gates, ngates);
    if (st) return st;
    for (uint32_t c = 0; c < ncalls; ++c) {
        o.u8((uint8_t)calls[c].op);
        o.var(calls[c].gate_count);
        o.var(calls[c].mask);
        o.f64(calls[c].u01);
    }
    return finish(o, buf, cap, len);
}

int qvnt_wire_decode_request(const uint8_t* buf, size_t len, uint32_t* q_num, uint64_t* state, int* flags,
                             qvnt_gate* gates, size_t gcap, size_t* ngates, qvnt_call* calls, uint32_t ccap,
                             uint32_t* ncalls) {
    if (!q_num || !state || !flags || !ngates || !ncalls) return set_error(QVNT_ERR_BAD_ARG, "null output pointer");
    In in{buf, len};
    int st = open_frame(in, kTypeRequest);
    if (st) return st;
    const uint64_t ng = in.var();
    const uint64_t q = in.var(), s0 = in.var(), fl = in.var(), nc = in.var();
    if (in.fail) return set_error(QVNT_ERR_BAD_ARG, "wire stream: %s at byte %zu", in.why, in.at);
    if (q > 64) return set_error(QVNT_ERR_BAD_ARG, "wire stream: q_num %llu", (unsigned long long)q);
    if (fl > 0x7FFFFFFF) return set_error(QVNT_ERR_BAD_ARG, "wire stream: flags %llu", (unsigned long long)fl);
    if (nc > 0xFFFFFFFFull) return set_error(QVNT_ERR_BAD_ARG, "wire stream: %llu calls", (unsigned long long)nc);
    // Gate records take at least 3 bytes, call records at least 11.
    const size_t rest = in.n - in.at;
    if (ng > rest / 3 || nc > rest / 11 || ng * 3 + nc * 11 > rest)
        return set_error(QVNT_ERR_BAD_ARG, "wire stream: %llu gates and %llu calls exceed the stream",
                         (unsigned long long)ng, (unsigned long long)nc);
    st = get_gates(in, ng, gates, gcap);
    if (st) return st;
    uint64_t applied = 0;
    for (uint64_t c = 0; c < nc; ++c) {
        qvnt_call k;
        memset(&k, 0, sizeof k);
        k.op = in.u8();
        k.gate_count = in.var();
        k.mask = in.var();
        k.u01 = in.f64();
        if (in.fail) return set_error(QVNT_ERR_BAD_ARG, "wire stream: %s at byte %zu", in.why, in.at);
        if (k.op != QVNT_CALL_APPLY && k.op != QVNT_CALL_MEASURE)
            return set_error(QVNT_ERR_BAD_ARG, "wire stream: call %llu: unknown op %u", (unsigned long long)c, k.op);
        if (k.op == QVNT_CALL_APPLY) {
            if (k.gate_count > ng - applied)
                return set_error(QVNT_ERR_BAD_ARG, "wire stream: call %llu applies more gates than the list holds", (unsigned long long)c);
            applied += k.gate_count;
        }
        if (calls && c < ccap) calls[c] = k;
    }
    if (applied != ng)
        return set_error(QVNT_ERR_BAD_ARG, "wire stream: the calls apply %llu of %llu gates", (unsigned long long)applied,
                         (unsigned long long)ng);
    if (in.at != in.n) return set_error(QVNT_ERR_BAD_ARG, "wire stream: %zu trailing bytes", in.n - in.at);
    *q_num = (uint32_t)q;
    *state = s0;
    *flags = (int)fl;
    *ngates = (size_t)ng;
    *ncalls = (uint32_t)nc;
    return QVNT_OK;
}

// qvnt's `Debug` of the interpreted program, `int::Op` (src/qasm/int/ext_op.rs:77-112), which
// `Int::get_ops_tree` returns (src/qasm/int/mod.rs:398-400): "[H1] -> Measure(1 => 1) -> if c[1] ==
// 1 { [X2] } -> [Z2]".
int qvnt_program_format(const qvnt_gate* gates, const qvnt_block* blocks, uint32_t nblocks, uint64_t trailing_gates,
                        char* buf, size_t cap, size_t* needed) {
    if (nblocks && !blocks) return set_error(QVNT_ERR_BAD_ARG, "null block list");
    uint64_t ng = trailing_gates;
    for (uint32_t b = 0; b < nblocks; ++b) {
        if (blocks[b].sep > QVNT_SEP_RESET) return set_error(QVNT_ERR_BAD_ARG, "block %u: unknown separator %u", b, blocks[b].sep);
        ng += blocks[b].gate_count;
    }
    if (ng && !gates) return set_error(QVNT_ERR_BAD_ARG, "null gate list");
    std::string s, ops;
    uint64_t g0 = 0;
    int st;
    for (uint32_t b = 0; b < nblocks; ++b) {
        const qvnt_block& k = blocks[b];
        if ((st = list_name(gates + g0, (size_t)k.gate_count, &ops))) return st;
        g0 += k.gate_count;
        // the first block prints its list even when empty (`{:?}`); later ones via `fmt_op`
        const std::string shown = (b == 0 || k.gate_count) ? (b == 0 ? ops : " -> " + ops) : "";
        switch (k.sep) {
        case QVNT_SEP_NOP: s += shown; break;
        case QVNT_SEP_MEASURE: s += shown + " -> Measure(" + binary_string(k.a) + " => " + binary_string(k.b) + ")"; break;
        case QVNT_SEP_IF: s += " -> if c[" + binary_string(k.a) + "] == " + binary_string(k.b) + " { " + ops + " }"; break;
        default: s += shown + " -> Reset(" + binary_string(k.a) + ")"; break;
        }
    }
    if ((st = list_name(gates + g0, (size_t)trailing_gates, &ops))) return st;
    if (!nblocks) s = ops;
    else if (trailing_gates) s += " -> " + ops;
    if (needed) *needed = s.size();
    if (buf && cap) {
        const size_t k = s.size() < cap - 1 ? s.size() : cap - 1;
        memcpy(buf, s.data(), k);
        buf[k] = 0;
    }
    return QVNT_OK;
}

int qvnt_program_parse(const char* text, size_t len, qvnt_gate* gates, size_t gcap, size_t* ngates, qvnt_block* blocks,
                       uint32_t bcap, uint32_t* nblocks, uint64_t* trailing_gates) {
    if (!ngates || !nblocks || !trailing_gates) return set_error(QVNT_ERR_BAD_ARG, "null count pointer");
    if (!text && len) return set_error(QVNT_ERR_BAD_ARG, "null text");
    Text t{text, len};
    std::vector<qvnt_gate> all, pending;
    std::vector<qvnt_block> out;
    bool have_pending = false, ok = true;
    auto close = [&](uint32_t sep, uint64_t a, uint64_t b) {
        qvnt_block k;
        memset(&k, 0, sizeof k);
        k.sep = sep;
        k.gate_count = pending.size();
        k.a = a;
        k.b = b;
        all.insert(all.end(), pending.begin(), pending.end());
        out.push_back(k);
        pending.clear();
        have_pending = false;
    };
    bool first = true;
    for (;;) {
        t.ws();
        if (t.at == t.n) break;
        if (!first && !(ok = t.eat("->") || t.error("expected '->'"))) break;
        if (first) t.eat("->");  // an IF block first prints " -> if ..."
        first = false;
        t.ws();
        if (t.peek("[")) {
            if (have_pending) close(QVNT_SEP_NOP, 0, 0);  // two lists in a row: the first was a Nop block
            if (!(ok = parse_list(t, pending))) break;
            have_pending = true;
        } else if (t.eat("Measure(")) {
            uint64_t q = 0, c = 0;
            if (!(ok = binary(t, &q) && t.expect("=>") && binary(t, &c) && t.expect(")"))) break;
            close(QVNT_SEP_MEASURE, q, c);
        } else if (t.eat("Reset(")) {
            uint64_t q = 0;
            if (!(ok = binary(t, &q) && t.expect(")"))) break;
            close(QVNT_SEP_RESET, q, 0);
        } else if (t.eat("if")) {
            uint64_t c = 0, v = 0;
            if (!(ok = t.expect("c") && t.expect("[") && binary(t, &c) && t.expect("]") && t.expect("==") &&
                       binary(t, &v) && t.expect("{")))
                break;
            if (have_pending) close(QVNT_SEP_NOP, 0, 0);
            if (!(ok = parse_list(t, pending) && t.expect("}"))) break;
            close(QVNT_SEP_IF, c, v);
        } else {
            ok = t.error("expected a gate list, Measure, Reset or if");
            break;
        }
    }
    if (!ok) return set_error(QVNT_ERR_BAD_ARG, "program text: %s at byte %zu", t.why, t.why_at);
    if (out.size() > 0xFFFFFFFFull) return set_error(QVNT_ERR_BAD_ARG, "too many blocks");
    const uint64_t tail = pending.size();
    all.insert(all.end(), pending.begin(), pending.end());
    for (size_t i = 0; gates && i < all.size() && i < gcap; ++i) gates[i] = all[i];
    for (size_t i = 0; blocks && i < out.size() && i < bcap; ++i) blocks[i] = out[i];
    *ngates = all.size();
    *nblocks = (uint32_t)out.size();
    *trailing_gates = tail;
    return QVNT_OK;
}

}  // extern "C"
