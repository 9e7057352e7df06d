// OpenQASM 2.0 front end for hosts without qvnt's Rust interpreter: program text to the blocks of
// qvnt_program_run, as `Int::new(Ast::from_source(source))` (src/qasm/int/mod.rs:56-60) lowers it.
//
// Parsing follows the OpenQASM 2.0 grammar (qvnt takes its parser from the qvnt-qasm crate);
// `include` lines are skipped because qvnt's gate table builds the qelib gates itself.  Lowering
// follows src/qasm/int: qubits and bits are allocated in declaration order; a gate name is looked up
// among the program's `gate` definitions, then in qvnt's table (int/gates.rs:86-126): a leading c/C
// controls the rest by the first register, the registers are OR-ed into one mask, sdg/tdg build S/T;
// arguments are evaluated in the context qvnt gives meval (int/parse.rs:5-25: pi, sqrt, exp, ln,
// abs, floor, ceil, round, atan2, max, min); gates are pushed with `int::Op::push` (ext_op.rs:40-50),
// measure and reset close the pending gates into their block (`branch_with_id`), and `if` is
// branch(Nop), the gate, branch(If) (int/mod.rs:286-305, 374-384).
#include <cctype>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../../include/qvnt_gb300.h"

namespace qvnt {
int set_error(int status, const char* fmt, ...);
}  // namespace qvnt

namespace {

struct QasmError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

[[noreturn]] void fail(const std::string& what) { throw QasmError(what); }

// ------------------------------------------------------------------------------------- lexer

bool is_ident_start(char c) { return std::isalpha((unsigned char)c) || c == '_'; }
bool is_ident(char c) { return std::isalnum((unsigned char)c) || c == '_'; }
bool is_digit(char c) { return c >= '0' && c <= '9'; }

// A number: digits [. digits*] [e[+-]digits] or . digits [e[+-]digits]; returns its length.
size_t number_len(const std::string& s, size_t i) {
    size_t j = i;
    if (is_digit(s[j])) {
        while (j < s.size() && is_digit(s[j])) ++j;
        if (j < s.size() && s[j] == '.') {
            ++j;
            while (j < s.size() && is_digit(s[j])) ++j;
        }
    } else if (s[j] == '.' && j + 1 < s.size() && is_digit(s[j + 1])) {
        ++j;
        while (j < s.size() && is_digit(s[j])) ++j;
    } else {
        return 0;
    }
    if (j < s.size() && (s[j] == 'e' || s[j] == 'E')) {
        size_t k = j + 1;
        if (k < s.size() && (s[k] == '+' || s[k] == '-')) ++k;
        if (k < s.size() && is_digit(s[k])) {
            while (k < s.size() && is_digit(s[k])) ++k;
            j = k;
        }
    }
    return j - i;
}

std::vector<std::string> lex(const std::string& s) {
    std::vector<std::string> out;
    size_t i = 0;
    while (i < s.size()) {
        const char c = s[i];
        if (std::isspace((unsigned char)c)) {
            ++i;
        } else if (c == '/' && i + 1 < s.size() && s[i + 1] == '/') {
            while (i < s.size() && s[i] != '\n') ++i;
        } else if (c == '"') {
            size_t j = s.find('"', i + 1);
            if (j == std::string::npos) {  // an unterminated quote is a one-character token
                out.emplace_back(1, c);
                ++i;
            } else {
                out.push_back(s.substr(i, j + 1 - i));
                i = j + 1;
            }
        } else if ((c == '-' && i + 1 < s.size() && s[i + 1] == '>') || (c == '=' && i + 1 < s.size() && s[i + 1] == '=')) {
            out.push_back(s.substr(i, 2));
            i += 2;
        } else if (is_ident_start(c)) {
            size_t j = i;
            while (j < s.size() && is_ident(s[j])) ++j;
            out.push_back(s.substr(i, j - i));
            i = j;
        } else if (size_t k = number_len(s, i)) {
            out.push_back(s.substr(i, k));
            i += k;
        } else {
            out.emplace_back(1, c);
            ++i;
        }
    }
    return out;
}

bool is_ident_token(const std::string& t) { return !t.empty() && is_ident_start(t[0]); }

// ------------------------------------------------------------------------------------- expressions

using Vars = std::vector<std::pair<std::string, double>>;

double fmax_rust(double m, double x) { return std::isnan(x) ? m : ((std::isnan(m) || x > m) ? x : m); }
double fmin_rust(double m, double x) { return std::isnan(x) ? m : ((std::isnan(m) || x < m) ? x : m); }
double round_rust(double v) {
    if (!std::isfinite(v)) return v;
    const double a = std::fabs(v), r = std::floor(a);
    return std::copysign(a - r >= 0.5 ? r + 1.0 : r, v);
}

struct Expr {
    const std::vector<std::string>& t;
    size_t i;
    const Vars& vars;

    const std::string* peek() const { return i < t.size() ? &t[i] : nullptr; }
    bool at(const char* s) const { return i < t.size() && t[i] == s; }
    const std::string& take() {
        if (i >= t.size()) fail("expression ends early");
        return t[i++];
    }
    void expect(const char* s) {
        if (!at(s)) fail(std::string("expression: expected '") + s + "'");
        ++i;
    }
    double atom() {
        const std::string tok = take();
        if (tok == "(") {
            const double v = add();
            expect(")");
            return v;
        }
        if (is_digit(tok[0]) || (tok[0] == '.' && tok.size() > 1)) return std::strtod(tok.c_str(), nullptr);
        if (is_ident_token(tok)) {
            if (at("(")) {
                ++i;
                std::vector<double> a{add()};
                while (at(",")) {
                    ++i;
                    a.push_back(add());
                }
                expect(")");
                auto one = [&](double (*f)(double)) {
                    if (a.size() != 1) fail("expression: " + tok + " takes 1 argument");
                    return f(a[0]);
                };
                if (tok == "sqrt") return one(std::sqrt);
                if (tok == "exp") return one(std::exp);
                if (tok == "ln") return one(std::log);
                if (tok == "abs") return one(std::fabs);
                if (tok == "floor") return one(std::floor);
                if (tok == "ceil") return one(std::ceil);
                if (tok == "round") return one(round_rust);
                if (tok == "atan2") {
                    if (a.size() != 2) fail("expression: atan2 takes 2 arguments");
                    return std::atan2(a[0], a[1]);
                }
                if (tok == "max" || tok == "min") {  // meval's max_array / min_array
                    double m = tok == "max" ? -INFINITY : INFINITY;
                    for (double x : a) m = tok == "max" ? fmax_rust(m, x) : fmin_rust(m, x);
                    return m;
                }
                fail("expression: unknown function " + tok);
            }
            for (const auto& v : vars)
                if (v.first == tok) return v.second;
            if (tok == "pi") return M_PI;
            fail("expression: unknown variable " + tok);
        }
        fail("expression: unexpected '" + tok + "'");
    }
    double power() {
        const double base = atom();
        if (at("^")) {
            ++i;
            return std::pow(base, unary());
        }
        return base;
    }
    double unary() {
        if (at("-") || at("+")) {
            const double sign = take() == "-" ? -1.0 : 1.0;
            return sign * unary();
        }
        return power();
    }
    double mul() {
        double v = unary();
        while (at("*") || at("/") || at("%")) {
            const std::string o = take();
            const double r = unary();
            v = o == "*" ? v * r : (o == "/" ? v / r : std::fmod(v, r));
        }
        return v;
    }
    double add() {
        double v = mul();
        while (at("+") || at("-")) {
            const std::string o = take();
            const double r = mul();
            v = o == "+" ? v + r : v - r;
        }
        return v;
    }
};

double eval(const std::vector<std::string>& toks, const Vars& vars) {
    if (toks.empty()) fail("empty expression");
    Expr e{toks, 0, vars};
    const double v = e.add();
    if (e.i != toks.size()) fail("expression: trailing '" + toks[e.i] + "'");
    return v;
}

// ------------------------------------------------------------------------------------- parser

struct Arg {
    std::string name;
    long long idx;  // -1: the whole register
};

struct Apply {
    std::string name;
    std::vector<std::vector<std::string>> params;  // expression tokens
    std::vector<Arg> regs;
};

struct Node {
    enum Kind { QREG, CREG, BARRIER, RESET, MEASURE, APPLY, GATE, IF, OPAQUE } kind;
    std::string name;
    long long size = 0;
    Arg a, b;
    Apply apply;
    std::vector<std::string> gate_regs, gate_params;
    std::vector<Apply> body;
    long long value = 0;
};

struct Parser {
    std::vector<std::string> t;
    size_t i = 0;

    const std::string* peek(size_t k = 0) const { return i + k < t.size() ? &t[i + k] : nullptr; }
    bool at(const char* s) const { return i < t.size() && t[i] == s; }
    std::string take() {
        if (i >= t.size()) fail("unexpected end of source");
        return t[i++];
    }
    void expect(const char* s) {
        if (!at(s)) fail(std::string("expected '") + s + "' at token " + std::to_string(i));
        ++i;
    }
    void semi() {
        if (!at(";")) fail("missing semicolon at token " + std::to_string(i));
        ++i;
    }
    std::string ident() {
        if (i >= t.size() || !is_ident_token(t[i])) fail("missing identifier at token " + std::to_string(i));
        return t[i++];
    }
    long long integer() {
        if (i >= t.size() || t[i].empty()) fail("missing integer at token " + std::to_string(i));
        for (char c : t[i])
            if (!is_digit(c)) fail("missing integer at token " + std::to_string(i));
        if (t[i].size() > 18) fail("integer too large at token " + std::to_string(i));
        return std::atoll(t[i++].c_str());
    }
    Arg arg() {
        Arg a{ident(), -1};
        if (at("[")) {
            ++i;
            a.idx = integer();
            expect("]");
        }
        return a;
    }
    std::vector<Arg> args() {
        std::vector<Arg> out{arg()};
        while (at(",")) {
            ++i;
            out.push_back(arg());
        }
        return out;
    }
    std::vector<std::vector<std::string>> exprs() {
        expect("(");
        std::vector<std::vector<std::string>> out;
        std::vector<std::string> cur;
        int depth = 0;
        for (;;) {
            std::string tok = take();
            if (tok == "(") {
                ++depth;
            } else if (tok == ")") {
                if (depth == 0) break;
                --depth;
            } else if (tok == "," && depth == 0) {
                out.push_back(cur);
                cur.clear();
                continue;
            }
            cur.push_back(tok);
        }
        if (!cur.empty() || !out.empty()) out.push_back(cur);
        return out;
    }
    Apply apply() {
        Apply a;
        a.name = ident();
        if (at("(")) a.params = exprs();
        a.regs = args();
        semi();
        return a;
    }
    bool statement(Node* n) {
        const std::string k = *peek();
        if (k == "include") {
            ++i;
            take();
            semi();
            return false;
        }
        if (k == "qreg" || k == "creg") {
            ++i;
            n->kind = k == "qreg" ? Node::QREG : Node::CREG;
            n->name = ident();
            expect("[");
            n->size = integer();
            expect("]");
            semi();
            return true;
        }
        if (k == "barrier") {
            ++i;
            args();
            semi();
            n->kind = Node::BARRIER;
            return true;
        }
        if (k == "reset") {
            ++i;
            n->kind = Node::RESET;
            n->a = arg();
            semi();
            return true;
        }
        if (k == "measure") {
            ++i;
            n->kind = Node::MEASURE;
            n->a = arg();
            expect("->");
            n->b = arg();
            semi();
            return true;
        }
        if (k == "opaque") {
            ++i;
            ident();
            if (at("(")) exprs();
            args();
            semi();
            n->kind = Node::OPAQUE;
            return true;
        }
        if (k == "gate") {
            ++i;
            n->kind = Node::GATE;
            n->name = ident();
            if (at("(")) {
                for (auto& e : exprs()) {
                    std::string p;
                    for (auto& s : e) p += (p.empty() ? "" : " ") + s;
                    n->gate_params.push_back(p);
                }
            }
            for (auto& a : args()) n->gate_regs.push_back(a.name);
            expect("{");
            while (!at("}")) {
                if (!peek()) fail("unterminated gate " + n->name);
                const std::string& w = *peek();
                if (w == "barrier") {
                    ++i;
                    args();
                    semi();
                    continue;
                }
                if (w == "measure" || w == "reset" || w == "if" || w == "qreg" || w == "creg" || w == "gate")
                    fail("operation " + w + " is not allowed in gate " + n->name);
                n->body.push_back(apply());
            }
            ++i;
            return true;
        }
        if (k == "if") {
            ++i;
            n->kind = Node::IF;
            expect("(");
            n->name = ident();
            expect("==");
            n->value = integer();
            expect(")");
            if (at("measure") || at("reset") || at("barrier")) fail(*peek() + " is not allowed in an if");
            n->apply = apply();
            return true;
        }
        n->kind = Node::APPLY;
        n->apply = apply();
        return true;
    }
    std::vector<Node> program() {
        if (at("OPENQASM")) {
            ++i;
            const std::string v = take();
            if (v != "2.0" && v != "2") fail("unsupported version " + v);
            semi();
        }
        std::vector<Node> out;
        while (peek()) {
            Node n;
            if (statement(&n)) out.push_back(std::move(n));
        }
        return out;
    }
};

// ------------------------------------------------------------------------------------- lowering

using Gates = std::vector<qvnt_gate>;

unsigned bits(uint64_t m) { return (unsigned)__builtin_popcountll(m); }

Gates one(uint32_t kind, uint64_t mask, double angle = 0.0) {
    qvnt_gate g;
    if (qvnt_gate_make(kind, mask, 0, angle, nullptr, &g) != QVNT_OK) fail("invalid mask for gate");
    return Gates{g};
}

Gates list(int (*builder)(uint64_t, qvnt_gate*, size_t, size_t*), uint64_t mask) {
    size_t n = 0;
    builder(mask, nullptr, 0, &n);
    Gates g(n);
    builder(mask, g.data(), n, &n);
    return g;
}

uint64_t act_on(const Gates& g) {
    uint64_t m = 0;
    for (auto& x : g) m |= qvnt_gate_act_on(&x);
    return m;
}

bool named(const std::string& name, const char* lower) {
    std::string upper(lower);
    for (auto& c : upper) c = (char)std::toupper((unsigned char)c);
    return name == lower || name == upper;
}

// `gates::process` (int/gates.rs:86-126).
Gates builtin(const std::string& name, const std::vector<uint64_t>& regs, const std::vector<double>& args) {
    if (!name.empty() && (name[0] == 'c' || name[0] == 'C')) {
        if (regs.empty()) fail(name + ": no control register");
        Gates sub = builtin(name.substr(1), std::vector<uint64_t>(regs.begin() + 1, regs.end()), args);
        if (act_on(sub) & regs[0])
            fail(name + ": control mask " + std::to_string(regs[0]) + " overlaps " + std::to_string(act_on(sub)));
        if (qvnt_ops_c(sub.data(), sub.size(), regs[0]) != QVNT_OK) fail(name + ": invalid control");
        return sub;
    }
    uint64_t m = 0;
    for (uint64_t r : regs) m |= r;
    struct Any {
        const char* n;
        uint32_t kind;
    };
    static const Any any[] = {{"x", QVNT_GATE_X}, {"y", QVNT_GATE_Y}, {"z", QVNT_GATE_Z}, {"s", QVNT_GATE_S},
                              {"sdg", QVNT_GATE_S}, {"t", QVNT_GATE_T}, {"tdg", QVNT_GATE_T}};
    for (const Any& a : any)
        if (named(name, a.n)) {
            if (!m) fail(name + ": no qubits");
            if (!args.empty()) fail(name + ": takes no arguments");
            return one(a.kind, m);
        }
    if (named(name, "h") || named(name, "qft")) {
        if (!m) fail(name + ": no qubits");
        if (!args.empty()) fail(name + ": takes no arguments");
        return list(named(name, "h") ? qvnt_op_h : qvnt_op_qft, m);
    }
    struct Rot {
        const char* n;
        uint32_t kind;
        unsigned nb;
    };
    static const Rot rot[] = {{"rx", QVNT_GATE_RX, 1}, {"ry", QVNT_GATE_RY, 1}, {"rz", QVNT_GATE_RZ, 1},
                              {"rxx", QVNT_GATE_RXX, 2}, {"ryy", QVNT_GATE_RYY, 2}, {"rzz", QVNT_GATE_RZZ, 2}};
    for (const Rot& r : rot)
        if (named(name, r.n)) {
            if (bits(m) != r.nb) fail(name + ": wrong number of qubits");
            if (args.size() != 1) fail(name + ": takes 1 argument");
            return one(r.kind, m, args[0]);
        }
    static const Any two[] = {{"swap", QVNT_GATE_SWAP}, {"sqrt_swap", QVNT_GATE_SQRT_SWAP},
                              {"i_swap", QVNT_GATE_ISWAP}, {"sqrt_i_swap", QVNT_GATE_SQRT_ISWAP}};
    for (const Any& a : two)
        if (named(name, a.n)) {
            if (bits(m) != 2) fail(name + ": needs 2 qubits");
            if (!args.empty()) fail(name + ": takes no arguments");
            return one(a.kind, m);
        }
    if (named(name, "u1") || named(name, "u2") || named(name, "u3")) {
        const size_t na = (size_t)(name[1] - '0');
        if (bits(m) != 1) fail(name + ": needs 1 qubit");
        if (args.size() != na) fail(name + ": wrong number of arguments");
        if (na == 1) return one(QVNT_GATE_RZ, m, args[0]);  // op::u1 = rz (operator/mod.rs:472-474)
        Gates g(3);
        size_t n = 0;
        if (na == 2) qvnt_op_u2(args[0], args[1], m, g.data(), 3, &n);
        else qvnt_op_u3(args[0], args[1], args[2], m, g.data(), 3, &n);
        g.resize(n);
        return g;
    }
    fail("unknown gate " + name);
}

struct Macro {
    std::vector<std::string> regs, params;
    std::vector<Apply> body;
};

struct Program {
    std::vector<std::pair<Gates, qvnt_block>> blocks;
    Gates last;

    static qvnt_block sep(uint32_t kind, uint64_t a = 0, uint64_t b = 0) {
        qvnt_block k;
        memset(&k, 0, sizeof k);
        k.sep = kind;
        k.a = a;
        k.b = b;
        return k;
    }
    void push(const Gates& g) {  // ext_op.rs:40-50
        if (last.empty()) {
            if (!blocks.empty() && blocks.back().second.sep == QVNT_SEP_NOP) {
                blocks.back().first.insert(blocks.back().first.end(), g.begin(), g.end());
            } else {
                last = g;
            }
        } else {
            last.insert(last.end(), g.begin(), g.end());
        }
    }
    void branch(const qvnt_block& k) {  // int/mod.rs:374-379
        if (last.empty()) return;
        blocks.emplace_back(std::move(last), k);
        last.clear();
    }
    void branch_with_id(const qvnt_block& k) {  // int/mod.rs:381-384
        blocks.emplace_back(std::move(last), k);
        last.clear();
    }
};

struct Interp {
    std::vector<std::string> q_reg, c_reg;
    std::map<std::string, Macro> macros;
    Program prog;

    static uint64_t idx(const std::vector<std::string>& regs, const Arg& a, const char* what) {
        uint64_t m = 0;
        for (size_t k = 0; k < regs.size(); ++k)
            if (regs[k] == a.name) m |= 1ull << k;
        if (!m) fail(std::string("no ") + what + " " + a.name);
        if (a.idx < 0) return m;
        long long n = a.idx;
        for (uint64_t r = m; r; r &= r - 1)
            if (n-- == 0) return r & (~r + 1);
        fail("index " + a.name + "[" + std::to_string(a.idx) + "] out of range");
    }
    uint64_t q(const Arg& a) const { return idx(q_reg, a, "qreg"); }
    uint64_t c(const Arg& a) const { return idx(c_reg, a, "creg"); }

    void declare(std::vector<std::string>& regs, const std::string& name, long long size) {
        if (name.size() >= 32) fail("identifier " + name + " is too long");
        if (size >= 64) fail("register " + name + " is too large");
        for (auto& r : q_reg)
            if (r == name) fail("register " + name + " is declared twice");
        for (auto& r : c_reg)
            if (r == name) fail("register " + name + " is declared twice");
        if (regs.size() + (size_t)size > 64) fail("more than 64 qubits or bits in all (a mask holds 64)");
        regs.insert(regs.end(), (size_t)size, name);
    }

    Gates expand(const std::string& name, const Macro& mac, const std::vector<uint64_t>& regs,
                 const std::vector<double>& args, int depth) {  // macros.rs:103-148
        if (regs.size() != mac.regs.size()) fail(name + ": wrong number of registers");
        if (args.size() != mac.params.size()) fail(name + ": wrong number of arguments");
        if (depth > 64) fail(name + ": gate definitions nest too deeply");
        Vars env;
        for (size_t k = 0; k < args.size(); ++k) env.emplace_back(mac.params[k], args[k]);
        Gates out;
        for (const Apply& b : mac.body) {
            std::vector<uint64_t> r;
            for (const Arg& a : b.regs)
                for (size_t k = 0; k < mac.regs.size(); ++k)
                    if (mac.regs[k] == a.name) {
                        r.push_back(regs[k]);
                        break;
                    }
            std::vector<double> v;
            for (auto& e : b.params) v.push_back(eval(e, env));
            Gates g;
            auto it = macros.find(b.name);
            if (it != macros.end()) {
                if (b.name == name) fail("recursive gate " + name);
                g = expand(b.name, it->second, r, v, depth + 1);
            } else {
                g = builtin(b.name, r, v);
            }
            out.insert(out.end(), g.begin(), g.end());
        }
        return out;
    }

    void apply(const Apply& a) {
        std::vector<uint64_t> r;
        for (const Arg& x : a.regs) r.push_back(q(x));
        std::vector<double> v;
        for (auto& e : a.params) v.push_back(eval(e, Vars{}));
        auto it = macros.find(a.name);
        prog.push(it != macros.end() ? expand(a.name, it->second, r, v, 0) : builtin(a.name, r, v));
    }

    void node(const Node& n) {
        switch (n.kind) {
        case Node::QREG: declare(q_reg, n.name, n.size); break;
        case Node::CREG: declare(c_reg, n.name, n.size); break;
        case Node::BARRIER:
        case Node::OPAQUE: break;
        case Node::RESET: prog.branch_with_id(Program::sep(QVNT_SEP_RESET, q(n.a))); break;
        case Node::MEASURE: {
            const uint64_t qm = q(n.a), cm = c(n.b);
            if (bits(qm) != bits(cm)) fail("measure: unmatched register sizes");
            prog.branch_with_id(Program::sep(QVNT_SEP_MEASURE, qm, cm));
            break;
        }
        case Node::APPLY: apply(n.apply); break;
        case Node::GATE: {
            if (macros.count(n.name)) fail("gate " + n.name + " is defined twice");
            if (n.name.size() >= 32) fail("identifier " + n.name + " is too long");
            Macro m{n.gate_regs, n.gate_params, n.body};
            Vars probe;
            for (auto& p : m.params) probe.emplace_back(p, 1.0);
            for (const Apply& b : m.body) {  // macros.rs:64-100
                for (const Arg& a : b.regs) {
                    if (a.idx >= 0) fail("indexing qubits isn't allowed in gate " + n.name);
                    bool known = false;
                    for (auto& r : m.regs) known |= r == a.name;
                    if (!known) fail("no register " + a.name + " in gate " + n.name);
                }
                for (auto& e : b.params) eval(e, probe);
            }
            macros[n.name] = std::move(m);
            break;
        }
        case Node::IF: {
            prog.branch(Program::sep(QVNT_SEP_NOP));
            const uint64_t val = c(Arg{n.name, -1});
            apply(n.apply);
            prog.branch(Program::sep(QVNT_SEP_IF, val, (uint64_t)n.value));
            break;
        }
        }
    }
};

}  // namespace

extern "C" int qvnt_qasm_compile(const char* source, size_t len, uint32_t* q_num, uint32_t* c_num, qvnt_gate* gates,
                                 size_t gcap, size_t* ngates, qvnt_block* blocks, uint32_t bcap, uint32_t* nblocks,
                                 uint64_t* trailing_gates) {
    if (!q_num || !c_num || !ngates || !nblocks || !trailing_gates)
        return qvnt::set_error(QVNT_ERR_BAD_ARG, "null output pointer");
    if (!source && len) return qvnt::set_error(QVNT_ERR_BAD_ARG, "null source");
    try {
        Parser p;
        p.t = lex(std::string(source ? source : "", len));
        if (p.t.empty()) fail("empty source");
        Interp in;
        for (const Node& n : p.program()) in.node(n);
        if (in.prog.blocks.size() > 0xFFFFFFFFull) fail("too many blocks");
        size_t g = 0;
        uint32_t b = 0;
        auto put = [&](const Gates& list) {
            for (const qvnt_gate& x : list) {
                if (gates && g < gcap) gates[g] = x;
                ++g;
            }
        };
        for (auto& blk : in.prog.blocks) {
            qvnt_block k = blk.second;
            k.gate_count = blk.first.size();
            if (blocks && b < bcap) blocks[b] = k;
            ++b;
            put(blk.first);
        }
        put(in.prog.last);
        *q_num = (uint32_t)in.q_reg.size();
        *c_num = (uint32_t)in.c_reg.size();
        *ngates = g;
        *nblocks = b;
        *trailing_gates = in.prog.last.size();
        return QVNT_OK;
    } catch (const QasmError& e) {
        return qvnt::set_error(QVNT_ERR_BAD_ARG, "qasm: %s", e.what());
    } catch (const std::exception& e) {
        return qvnt::set_error(QVNT_ERR_BAD_ARG, "qasm: %s", e.what());
    }
}
