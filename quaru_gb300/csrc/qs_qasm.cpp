// qs_qasm.cpp — OpenQASM 2.0 front end: parser and runner over the register C ABI.
//
// Mirrors openqasm::run_openqasm (src/openqasm.rs:52-142). The reference
// delegates parsing to the external crate openqasm-parser 1.0.0 (not vendored);
// this is a project-written parser for the OpenQASM 2.0 language: OPENQASM
// header, include, qreg/creg, gate definitions with parameters, U, CX,
// measure, reset, barrier, if(creg == int), expressions with pi, + - * / ^,
// unary minus and sin cos tan exp ln sqrt, and register broadcasting. Gate
// calls are flattened into the basic operations the reference executes:
//   U(t, p, l) q  -> Register::apply(u(t as f32 as f64, ...)) (the parser crate
//                    hands angles over as f32, src/openqasm.rs:92-100)
//   CX a, b       -> Register::apply(cnot(a, b)); an error if a and b are in
//                    different registers (src/openqasm.rs:101-111)
//   measure q->c  -> c = Register::measure(q)             (src/openqasm.rs:112-123)
//   reset q       -> the whole register q back to |0..0>  (src/openqasm.rs:124-130)
//   reset c       -> every bit of c cleared               (src/openqasm.rs:131-137)
//   if(c == n) op -> op only when creg c, read little-endian, equals n (:75-86, :175-190)
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "qs_internal.h"
#include "qs_kernels.h"

namespace qs {
namespace qasm {

struct Error {
    int code;
    std::string msg;
};

// ---------------------------------------------------------------- lexer
enum TokKind { T_ID, T_NUM, T_STR, T_SYM, T_END };
struct Tok {
    TokKind k;
    std::string s;
    double v = 0;
    bool integer = false;
    int line = 0;
};

static std::vector<Tok> lex(const std::string& src) {
    std::vector<Tok> out;
    size_t i = 0;
    int line = 1;
    while (i < src.size()) {
        const char c = src[i];
        if (c == '\n') {
            line++;
            i++;
        } else if (isspace((unsigned char)c)) {
            i++;
        } else if (c == '/' && i + 1 < src.size() && src[i + 1] == '/') {
            while (i < src.size() && src[i] != '\n') i++;
        } else if (isalpha((unsigned char)c) || c == '_') {
            size_t j = i;
            while (j < src.size() && (isalnum((unsigned char)src[j]) || src[j] == '_')) j++;
            out.push_back({T_ID, src.substr(i, j - i), 0, false, line});
            i = j;
        } else if (isdigit((unsigned char)c) || (c == '.' && i + 1 < src.size() && isdigit((unsigned char)src[i + 1]))) {
            size_t j = i;
            bool integer = true;
            while (j < src.size() && isdigit((unsigned char)src[j])) j++;
            if (j < src.size() && src[j] == '.') {
                integer = false;
                j++;
                while (j < src.size() && isdigit((unsigned char)src[j])) j++;
            }
            if (j < src.size() && (src[j] == 'e' || src[j] == 'E')) {
                size_t k = j + 1;
                if (k < src.size() && (src[k] == '+' || src[k] == '-')) k++;
                if (k < src.size() && isdigit((unsigned char)src[k])) {
                    integer = false;
                    j = k;
                    while (j < src.size() && isdigit((unsigned char)src[j])) j++;
                }
            }
            Tok t{T_NUM, src.substr(i, j - i), 0, integer, line};
            t.v = std::strtod(t.s.c_str(), nullptr);
            out.push_back(t);
            i = j;
        } else if (c == '"') {
            size_t j = i + 1;
            while (j < src.size() && src[j] != '"') j++;
            out.push_back({T_STR, src.substr(i + 1, j - i - 1), 0, false, line});
            i = j + 1;
        } else if (c == '-' && i + 1 < src.size() && src[i + 1] == '>') {
            out.push_back({T_SYM, "->", 0, false, line});
            i += 2;
        } else if (c == '=' && i + 1 < src.size() && src[i + 1] == '=') {
            out.push_back({T_SYM, "==", 0, false, line});
            i += 2;
        } else if (strchr(";,()[]{}+-*/^", c)) {
            out.push_back({T_SYM, std::string(1, c), 0, false, line});
            i++;
        } else {
            throw Error{QS_QASM_PARSE_ERROR, "line " + std::to_string(line) + ": unexpected character '" +
                                                 std::string(1, c) + "'"};
        }
    }
    out.push_back({T_END, "", 0, false, line});
    return out;
}

// ---------------------------------------------------------------- AST
struct Expr {
    enum Kind { NUM, VAR, NEG, BIN, FUN } kind = NUM;
    double v = 0;
    std::string name;
    char op = 0;
    std::shared_ptr<Expr> a, b;
};

struct Arg {
    std::string reg;
    int index = -1;  // -1: the whole register
};

struct Call {  // U, CX, measure, reset, barrier or a gate call
    std::string name;
    std::vector<std::shared_ptr<Expr>> params;
    std::vector<Arg> args;
    int line = 0;
};

struct Stmt {
    Call call;
    bool cond = false;
    std::string creg;
    uint64_t value = 0;
};

struct GateDef {
    std::vector<std::string> params, qargs;
    std::vector<Call> body;
};

struct Program {
    std::vector<std::pair<std::string, size_t>> qregs, cregs;  // declaration order
    std::map<std::string, GateDef> gates;
    std::vector<Stmt> stmts;
};

// The standard gate library, defined from the gates' mathematical definitions in U and CX.
static const char* kStdGates = R"(
gate u3(theta, phi, lambda) q { U(theta, phi, lambda) q; }
gate u2(phi, lambda) q { U(pi / 2, phi, lambda) q; }
gate u1(lambda) q { U(0, 0, lambda) q; }
gate cx c, t { CX c, t; }
gate id a { U(0, 0, 0) a; }
gate u0(gamma) q { U(0, 0, 0) q; }
gate x a { u3(pi, 0, pi) a; }
gate y a { u3(pi, pi / 2, pi / 2) a; }
gate z a { u1(pi) a; }
gate h a { u2(0, pi) a; }
gate s a { u1(pi / 2) a; }
gate sdg a { u1(-pi / 2) a; }
gate t a { u1(pi / 4) a; }
gate tdg a { u1(-pi / 4) a; }
gate rx(theta) a { u3(theta, -pi / 2, pi / 2) a; }
gate ry(theta) a { u3(theta, 0, 0) a; }
gate rz(phi) a { u1(phi) a; }
gate cz a, b { h b; cx a, b; h b; }
gate cy a, b { sdg b; cx a, b; s b; }
gate swap a, b { cx a, b; cx b, a; cx a, b; }
gate cu1(lambda) a, b { u1(lambda / 2) a; cx a, b; u1(-lambda / 2) b; cx a, b; u1(lambda / 2) b; }
gate crz(lambda) a, b { u1(lambda / 2) b; cx a, b; u1(-lambda / 2) b; cx a, b; }
gate ccx a, b, c { h c; cx b, c; tdg c; cx a, c; t c; cx b, c; tdg c; cx a, c; t b; t c; h c; cx a, b; t a; tdg b; cx a, b; }
)";

// ---------------------------------------------------------------- parser
class Parser {
   public:
    Parser(const std::vector<Tok>& t, Program* p, std::string base) : t_(t), p_(p), base_(std::move(base)) {}

    void program(bool header) {
        if (header) {
            expect_id("OPENQASM");
            const Tok v = next();
            if (v.k != T_NUM) fail(v, "expected a version number");
            if (v.v < 2.0 || v.v >= 3.0) fail(v, "only OpenQASM 2.x is supported");
            expect(";");
        }
        while (peek().k != T_END) statement();
    }

   private:
    const std::vector<Tok>& t_;
    Program* p_;
    std::string base_;
    size_t i_ = 0;

    [[noreturn]] void fail(const Tok& t, const std::string& m) {
        throw Error{QS_QASM_PARSE_ERROR, "line " + std::to_string(t.line) + ": " + m};
    }
    const Tok& peek(size_t o = 0) { return t_[std::min(i_ + o, t_.size() - 1)]; }
    Tok next() {
        Tok t = peek();
        if (i_ < t_.size() - 1) i_++;
        return t;
    }
    bool is(const char* s) { return (peek().k == T_SYM || peek().k == T_ID) && peek().s == s; }
    void expect(const char* s) {
        const Tok t = next();
        if (t.s != s || (t.k != T_SYM && t.k != T_ID)) fail(t, std::string("expected '") + s + "'");
    }
    void expect_id(const char* s) {
        const Tok t = next();
        if (t.k != T_ID || t.s != s) fail(t, std::string("expected '") + s + "'");
    }
    std::string ident() {
        const Tok t = next();
        if (t.k != T_ID) fail(t, "expected an identifier");
        return t.s;
    }
    uint64_t integer() {
        const Tok t = next();
        if (t.k != T_NUM || !t.integer) fail(t, "expected a non-negative integer");
        return uint64_t(std::strtoull(t.s.c_str(), nullptr, 10));
    }

    // exp := term (('+'|'-') term)* ; term := unary (('*'|'/') unary)* ; unary := '-' unary | power
    // power := atom ('^' unary)?
    std::shared_ptr<Expr> exp() {
        auto a = term();
        while (is("+") || is("-")) {
            const char op = next().s[0];
            auto e = std::make_shared<Expr>();
            e->kind = Expr::BIN;
            e->op = op;
            e->a = a;
            e->b = term();
            a = e;
        }
        return a;
    }
    std::shared_ptr<Expr> term() {
        auto a = unary();
        while (is("*") || is("/")) {
            const char op = next().s[0];
            auto e = std::make_shared<Expr>();
            e->kind = Expr::BIN;
            e->op = op;
            e->a = a;
            e->b = unary();
            a = e;
        }
        return a;
    }
    std::shared_ptr<Expr> unary() {
        if (is("-")) {
            next();
            auto e = std::make_shared<Expr>();
            e->kind = Expr::NEG;
            e->a = unary();
            return e;
        }
        if (is("+")) {
            next();
            return unary();
        }
        auto a = atom();
        if (is("^")) {
            next();
            auto e = std::make_shared<Expr>();
            e->kind = Expr::BIN;
            e->op = '^';
            e->a = a;
            e->b = unary();
            return e;
        }
        return a;
    }
    std::shared_ptr<Expr> atom() {
        const Tok t = next();
        auto e = std::make_shared<Expr>();
        if (t.k == T_NUM) {
            e->kind = Expr::NUM;
            e->v = t.v;
        } else if (t.k == T_ID) {
            static const char* funs[] = {"sin", "cos", "tan", "exp", "ln", "sqrt"};
            bool fun = false;
            for (const char* f : funs) fun |= (t.s == f);
            if (fun) {
                expect("(");
                e->kind = Expr::FUN;
                e->name = t.s;
                e->a = exp();
                expect(")");
            } else if (t.s == "pi") {
                e->kind = Expr::NUM;
                e->v = 3.14159265358979323846;
            } else {
                e->kind = Expr::VAR;
                e->name = t.s;
            }
        } else if (t.k == T_SYM && t.s == "(") {
            e = exp();
            expect(")");
        } else {
            fail(t, "expected an expression");
        }
        return e;
    }

    Arg arg() {
        Arg a;
        a.reg = ident();
        if (is("[")) {
            next();
            a.index = int(integer());
            expect("]");
        }
        return a;
    }

    Call call(bool in_gate) {
        Call c;
        c.line = peek().line;
        c.name = ident();
        if (c.name == "measure") {
            c.args.push_back(arg());
            expect("->");
            c.args.push_back(arg());
        } else if (c.name == "reset") {
            c.args.push_back(arg());
        } else {
            if (is("(")) {
                next();
                if (!is(")")) {
                    c.params.push_back(exp());
                    while (is(",")) {
                        next();
                        c.params.push_back(exp());
                    }
                }
                expect(")");
            }
            if (c.name != "barrier" || !is(";")) {
                c.args.push_back(arg());
                while (is(",")) {
                    next();
                    c.args.push_back(arg());
                }
            }
            if (in_gate)
                for (const Arg& a : c.args)
                    if (a.index >= 0) fail(peek(), "indexed arguments are not allowed in a gate body");
        }
        expect(";");
        return c;
    }

    void statement() {
        const Tok& t = peek();
        if (t.k != T_ID) fail(t, "expected a statement");
        if (t.s == "include") {
            next();
            const Tok f = next();
            if (f.k != T_STR) fail(f, "expected a file name");
            expect(";");
            include(f);
        } else if (t.s == "qreg" || t.s == "creg") {
            const bool q = next().s == "qreg";
            const std::string name = ident();
            expect("[");
            const uint64_t size = integer();
            expect("]");
            expect(";");
            auto& regs = q ? p_->qregs : p_->cregs;
            for (auto& r : p_->qregs)
                if (r.first == name) fail(t, "register '" + name + "' declared twice");
            for (auto& r : p_->cregs)
                if (r.first == name) fail(t, "register '" + name + "' declared twice");
            if (size == 0 || size > 64) fail(t, "register size must be in 1..64");
            regs.push_back({name, size_t(size)});
        } else if (t.s == "gate") {
            next();
            const std::string name = ident();
            GateDef g;
            if (is("(")) {
                next();
                if (!is(")")) {
                    g.params.push_back(ident());
                    while (is(",")) {
                        next();
                        g.params.push_back(ident());
                    }
                }
                expect(")");
            }
            g.qargs.push_back(ident());
            while (is(",")) {
                next();
                g.qargs.push_back(ident());
            }
            expect("{");
            while (!is("}")) g.body.push_back(call(true));
            expect("}");
            p_->gates[name] = g;
        } else if (t.s == "opaque") {
            fail(t, "opaque gates cannot be simulated");
        } else if (t.s == "if") {
            next();
            expect("(");
            Stmt s;
            s.cond = true;
            s.creg = ident();
            expect("==");
            s.value = integer();
            expect(")");
            s.call = call(false);
            p_->stmts.push_back(s);
        } else {
            Stmt s;
            s.call = call(false);
            p_->stmts.push_back(s);
        }
    }

    void include(const Tok& f) {
        std::string text;
        if (f.s == "qelib1.inc") {
            text = kStdGates;
        } else {
            std::ifstream in(base_.empty() ? f.s : base_ + "/" + f.s);
            if (!in) fail(f, "cannot open include file '" + f.s + "'");
            std::stringstream ss;
            ss << in.rdbuf();
            text = ss.str();
        }
        std::vector<Tok> toks = lex(text);
        Parser sub(toks, p_, base_);
        sub.program(false);
    }
};

static double eval(const Expr& e, const std::map<std::string, double>& env, int line) {
    switch (e.kind) {
        case Expr::NUM: return e.v;
        case Expr::VAR: {
            auto it = env.find(e.name);
            if (it == env.end())
                throw Error{QS_QASM_PARSE_ERROR, "line " + std::to_string(line) + ": unknown parameter '" + e.name + "'"};
            return it->second;
        }
        case Expr::NEG: return -eval(*e.a, env, line);
        case Expr::FUN: {
            const double x = eval(*e.a, env, line);
            if (e.name == "sin") return std::sin(x);
            if (e.name == "cos") return std::cos(x);
            if (e.name == "tan") return std::tan(x);
            if (e.name == "exp") return std::exp(x);
            if (e.name == "ln") return std::log(x);
            return std::sqrt(x);
        }
        case Expr::BIN: {
            const double a = eval(*e.a, env, line), b = eval(*e.b, env, line);
            switch (e.op) {
                case '+': return a + b;
                case '-': return a - b;
                case '*': return a * b;
                case '/': return a / b;
                default: return std::pow(a, b);
            }
        }
    }
    return 0;
}

// ---------------------------------------------------------------- runner
struct Basic {  // a flattened operation
    enum Kind { U, CX, MEASURE, RESETQ, RESETC } kind;
    double p[3] = {0, 0, 0};
    std::string r0, r1;
    size_t i0 = 0, i1 = 0;
    bool cond = false;
    std::string creg;
    uint64_t value = 0;
    int line = 0;
};

class Flattener {
   public:
    Flattener(const Program& p) : p_(p) {}
    std::vector<Basic> run() {
        for (const Stmt& s : p_.stmts) {
            cond_ = s.cond;
            creg_ = s.creg;
            value_ = s.value;
            if (s.cond && !find_reg(p_.cregs, s.creg))
                fail(s.call.line, "unknown classical register '" + s.creg + "'");
            top(s.call);
        }
        return std::move(out_);
    }

   private:
    const Program& p_;
    std::vector<Basic> out_;
    bool cond_ = false;
    std::string creg_;
    uint64_t value_ = 0;

    [[noreturn]] void fail(int line, const std::string& m) {
        throw Error{QS_QASM_PARSE_ERROR, "line " + std::to_string(line) + ": " + m};
    }
    const std::pair<std::string, size_t>* find_reg(const std::vector<std::pair<std::string, size_t>>& regs,
                                                   const std::string& n) {
        for (auto& r : regs)
            if (r.first == n) return &r;
        return nullptr;
    }
    Basic base(Basic::Kind k, int line) {
        Basic b;
        b.kind = k;
        b.cond = cond_;
        b.creg = creg_;
        b.value = value_;
        b.line = line;
        return b;
    }

    // A top-level call with register arguments: broadcast over whole registers.
    void top(const Call& c) {
        if (c.name == "barrier") return;
        if (c.name == "measure") {
            auto q = find_reg(p_.qregs, c.args[0].reg);
            auto r = find_reg(p_.cregs, c.args[1].reg);
            if (!q) fail(c.line, "unknown quantum register '" + c.args[0].reg + "'");
            if (!r) fail(c.line, "unknown classical register '" + c.args[1].reg + "'");
            const bool wq = c.args[0].index < 0, wr = c.args[1].index < 0;
            if (wq != wr || (wq && q->second != r->second)) fail(c.line, "measure arguments do not match in size");
            const size_t cnt = wq ? q->second : 1;
            for (size_t i = 0; i < cnt; i++) {
                Basic b = base(Basic::MEASURE, c.line);
                b.r0 = q->first;
                b.i0 = wq ? i : size_t(c.args[0].index);
                b.r1 = r->first;
                b.i1 = wr ? i : size_t(c.args[1].index);
                if (b.i0 >= q->second || b.i1 >= r->second) fail(c.line, "register index out of range");
                out_.push_back(b);
            }
            return;
        }
        if (c.name == "reset") {
            auto q = find_reg(p_.qregs, c.args[0].reg);
            auto r = find_reg(p_.cregs, c.args[0].reg);
            if (!q && !r) fail(c.line, "unknown register '" + c.args[0].reg + "'");
            Basic b = base(q ? Basic::RESETQ : Basic::RESETC, c.line);
            b.r0 = c.args[0].reg;
            out_.push_back(b);
            return;
        }
        // broadcast: every whole-register argument must have the same size
        size_t width = 1;
        for (const Arg& a : c.args) {
            auto q = find_reg(p_.qregs, a.reg);
            if (!q) fail(c.line, "unknown quantum register '" + a.reg + "'");
            if (a.index >= 0 && size_t(a.index) >= q->second) fail(c.line, "register index out of range");
            if (a.index < 0) {
                if (width != 1 && width != q->second) fail(c.line, "register arguments differ in size");
                width = q->second;
            }
        }
        std::map<std::string, double> env;
        std::vector<double> params;
        for (auto& e : c.params) params.push_back(eval(*e, env, c.line));
        for (size_t i = 0; i < width; i++) {
            std::vector<std::pair<std::string, size_t>> qs;
            for (const Arg& a : c.args) qs.push_back({a.reg, a.index < 0 ? i : size_t(a.index)});
            apply(c.name, params, qs, c.line, 0);
        }
    }

    void apply(const std::string& name, const std::vector<double>& params,
               const std::vector<std::pair<std::string, size_t>>& qs, int line, int depth) {
        if (depth > 64) fail(line, "gate definitions nest too deeply");
        if (name == "U") {
            if (params.size() != 3 || qs.size() != 1) fail(line, "U takes 3 parameters and 1 qubit");
            Basic b = base(Basic::U, line);
            for (int k = 0; k < 3; k++) b.p[k] = params[k];
            b.r0 = qs[0].first;
            b.i0 = qs[0].second;
            out_.push_back(b);
            return;
        }
        if (name == "CX") {
            if (!params.empty() || qs.size() != 2) fail(line, "CX takes 2 qubits");
            if (qs[0] == qs[1]) fail(line, "CX needs two different qubits");
            Basic b = base(Basic::CX, line);
            b.r0 = qs[0].first;
            b.i0 = qs[0].second;
            b.r1 = qs[1].first;
            b.i1 = qs[1].second;
            out_.push_back(b);
            return;
        }
        if (name == "barrier") return;
        auto it = p_.gates.find(name);
        if (it == p_.gates.end()) fail(line, "unknown gate '" + name + "'");
        const GateDef& g = it->second;
        if (g.params.size() != params.size() || g.qargs.size() != qs.size())
            fail(line, "gate '" + name + "' called with the wrong number of arguments");
        for (size_t a = 0; a < qs.size(); a++)
            for (size_t b = a + 1; b < qs.size(); b++)
                if (qs[a] == qs[b]) fail(line, "gate '" + name + "' called with a repeated qubit");
        std::map<std::string, double> env;
        for (size_t k = 0; k < params.size(); k++) env[g.params[k]] = params[k];
        for (const Call& c : g.body) {
            std::vector<double> ps;
            for (auto& e : c.params) ps.push_back(eval(*e, env, c.line));
            std::vector<std::pair<std::string, size_t>> sub;
            for (const Arg& a : c.args) {
                size_t k = 0;
                while (k < g.qargs.size() && g.qargs[k] != a.reg) k++;
                if (k == g.qargs.size()) fail(c.line, "unknown qubit '" + a.reg + "' in gate '" + name + "'");
                sub.push_back(qs[k]);
            }
            apply(c.name, ps, sub, c.line, depth + 1);
        }
    }
};

// openqasm::u (src/openqasm.rs:145-163) for f64 angles.
static void u_matrix(double th, double ph, double la, double* m) {
    const double c = std::cos(th / 2.0), s = std::sin(th / 2.0);
    auto cexp = [](double x, double* out) {
        out[0] = std::cos(x);
        out[1] = std::sin(x);
    };
    double e[2];
    cexp(-(ph + la) / 2.0, e);
    m[0] = e[0] * c, m[1] = e[1] * c;
    cexp(-(ph - la) / 2.0, e);
    m[2] = -e[0] * s, m[3] = -e[1] * s;
    cexp((ph - la) / 2.0, e);
    m[4] = e[0] * s, m[5] = e[1] * s;
    cexp((ph + la) / 2.0, e);
    m[6] = e[0] * c, m[7] = e[1] * c;
}

}  // namespace qasm
}  // namespace qs

struct qs_qasm_result {
    std::vector<std::string> qnames, cnames;
    std::vector<qs_register*> qregs;
    std::vector<std::vector<uint8_t>> cregs;
    ~qs_qasm_result() {
        for (auto* r : qregs) qs_register_free(r);
    }
};

namespace {

struct SplitMix {
    uint64_t s;
    uint64_t next() {
        s += 0x9E3779B97F4A7C15ull;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return double(next() >> 11) * (1.0 / 9007199254740992.0); }
};

int run_program(const std::string& source, const std::string& base, uint64_t seed, int precision,
                qs_qasm_result** out) {
    using namespace qs::qasm;
    if (!out) {
        qs::set_last_error_message("output pointer is null");
        return QS_INVALID_ARGUMENT;
    }
    *out = nullptr;
    std::unique_ptr<qs_qasm_result> res(new qs_qasm_result());
    try {
        Program prog;
        std::vector<Tok> toks = lex(source);
        Parser(toks, &prog, base).program(true);
        std::vector<Basic> ops = Flattener(prog).run();
        for (auto& r : prog.qregs) {
            qs_register* h = nullptr;
            std::vector<uint8_t> zeros(r.second, 0);
            int rc = qs_register_new(zeros.data(), r.second, precision, &h);
            if (rc) return rc;
            res->qnames.push_back(r.first);
            res->qregs.push_back(h);
        }
        for (auto& r : prog.cregs) {
            res->cnames.push_back(r.first);
            res->cregs.push_back(std::vector<uint8_t>(r.second, 0));
        }
        auto qidx = [&](const std::string& n) {
            for (size_t i = 0; i < res->qnames.size(); i++)
                if (res->qnames[i] == n) return i;
            return size_t(-1);
        };
        auto cidx = [&](const std::string& n) {
            for (size_t i = 0; i < res->cnames.size(); i++)
                if (res->cnames[i] == n) return i;
            return size_t(-1);
        };
        SplitMix rng{seed};
        static const double cnot_m[32] = {1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0,
                                          0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 1, 0, 0, 0};
        for (const Basic& b : ops) {
            if (b.cond) {  // creg_to_u32: creg[0] is the least significant bit
                const auto& bits = res->cregs[cidx(b.creg)];
                if (bits.size() > 32) throw Error{QS_QASM_RUN_ERROR, "Registers larger than 32 bits are not allowed"};
                uint64_t v = 0;
                for (size_t i = bits.size(); i-- > 0;) v = (v << 1) | bits[i];
                if (v != b.value) continue;
            }
            int rc = QS_OK;
            size_t err[3] = {0, 0, 0};
            switch (b.kind) {
                case Basic::U: {
                    double m[8];
                    u_matrix(double(float(b.p[0])), double(float(b.p[1])), double(float(b.p[2])), m);
                    const size_t t = b.i0;
                    rc = qs_try_apply_fast(res->qregs[qidx(b.r0)], m, 2, 2, &t, 1, err);
                    break;
                }
                case Basic::CX: {
                    if (b.r0 != b.r1)
                        throw Error{QS_QASM_RUN_ERROR,
                                    "The simulator currently does not support applying CX on qubits in two different "
                                    "registers"};
                    const size_t t[2] = {b.i1, b.i0};  // cnot(control, target) has targets [target, control]
                    rc = qs_try_apply_fast(res->qregs[qidx(b.r0)], cnot_m, 4, 4, t, 2, err);
                    break;
                }
                case Basic::MEASURE: {
                    int outcome = 0;
                    rc = qs_try_measure(res->qregs[qidx(b.r0)], b.i0, rng.uniform(), &outcome, nullptr, nullptr, err);
                    res->cregs[cidx(b.r1)][b.i1] = uint8_t(outcome);
                    break;
                }
                case Basic::RESETQ: {
                    const size_t k = qidx(b.r0);
                    const size_t n = qs_register_size(res->qregs[k]);
                    qs_register* h = nullptr;
                    std::vector<uint8_t> zeros(n, 0);
                    rc = qs_register_new(zeros.data(), n, precision, &h);
                    if (!rc) {
                        qs_register_free(res->qregs[k]);
                        res->qregs[k] = h;
                    }
                    break;
                }
                case Basic::RESETC: {
                    auto& bits = res->cregs[cidx(b.r0)];
                    std::fill(bits.begin(), bits.end(), 0);
                    break;
                }
            }
            if (rc) return rc;
        }
    } catch (const Error& e) {
        qs::set_last_error_message(e.msg);
        return e.code;
    }
    *out = res.release();
    return QS_OK;
}

}  // namespace

extern "C" {

int qs_qasm_run(const char* source, const char* base_dir, uint64_t seed, int precision, qs_qasm_result** out) {
    if (!source) {
        qs::set_last_error_message("source is null");
        return QS_INVALID_ARGUMENT;
    }
    return run_program(source, base_dir ? base_dir : "", seed, precision, out);
}

int qs_qasm_run_file(const char* path, uint64_t seed, int precision, qs_qasm_result** out) {
    if (!path) {
        qs::set_last_error_message("path is null");
        return QS_INVALID_ARGUMENT;
    }
    std::ifstream in(path);
    if (!in) {
        qs::set_last_error_message(std::string("cannot open ") + path);
        return QS_QASM_PARSE_ERROR;
    }
    std::stringstream ss;
    ss << in.rdbuf();
    std::string p(path);
    const size_t slash = p.find_last_of('/');
    return run_program(ss.str(), slash == std::string::npos ? "" : p.substr(0, slash), seed, precision, out);
}

size_t qs_qasm_qreg_count(const qs_qasm_result* r) { return r ? r->qregs.size() : 0; }
const char* qs_qasm_qreg_name(const qs_qasm_result* r, size_t i) {
    return (r && i < r->qnames.size()) ? r->qnames[i].c_str() : nullptr;
}
qs_register* qs_qasm_qreg(qs_qasm_result* r, size_t i) { return (r && i < r->qregs.size()) ? r->qregs[i] : nullptr; }
size_t qs_qasm_creg_count(const qs_qasm_result* r) { return r ? r->cregs.size() : 0; }
const char* qs_qasm_creg_name(const qs_qasm_result* r, size_t i) {
    return (r && i < r->cnames.size()) ? r->cnames[i].c_str() : nullptr;
}
size_t qs_qasm_creg_size(const qs_qasm_result* r, size_t i) { return (r && i < r->cregs.size()) ? r->cregs[i].size() : 0; }
int qs_qasm_creg_bits(const qs_qasm_result* r, size_t i, uint8_t* bits) {
    if (!r || i >= r->cregs.size() || !bits) return QS_INVALID_ARGUMENT;
    std::memcpy(bits, r->cregs[i].data(), r->cregs[i].size());
    return QS_OK;
}
void qs_qasm_free(qs_qasm_result* r) { delete r; }

}  // extern "C"
