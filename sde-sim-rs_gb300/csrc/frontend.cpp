// frontend.cpp -- equation grammar (src/proc/util.rs) and fasteval-style
// expression grammar (src/func.rs), plus symbolic derivatives for the
// pathwise adjoint.
#include "frontend.h"

#include <cctype>
#include <cmath>
#include <cstring>
#include <functional>

namespace sde {

// ---------------------------------------------------------------------------
// Expression parser.  Precedence climbing over the fasteval operator table:
//   || (1)  && (2)  == != < <= > >= (3)  + - (4)  * / % (5)  ^ (6, right)
// Unary - + ! apply to the following value, so they bind tighter than ^.
// ---------------------------------------------------------------------------

namespace {

struct FnInfo { const char* name; Fn fn; int lo, hi; };
const FnInfo kFns[] = {
    {"min", Fn::Min, 1, 64}, {"max", Fn::Max, 1, 64}, {"abs", Fn::Abs, 1, 1},
    {"sign", Fn::Sign, 1, 1}, {"int", Fn::Int, 1, 1}, {"ceil", Fn::Ceil, 1, 1},
    {"floor", Fn::Floor, 1, 1}, {"round", Fn::Round, 1, 2}, {"log", Fn::Log, 1, 2},
    {"e", Fn::E, 0, 0}, {"pi", Fn::Pi, 0, 0}, {"sin", Fn::Sin, 1, 1},
    {"cos", Fn::Cos, 1, 1}, {"tan", Fn::Tan, 1, 1}, {"asin", Fn::Asin, 1, 1},
    {"acos", Fn::Acos, 1, 1}, {"atan", Fn::Atan, 1, 1}, {"sinh", Fn::Sinh, 1, 1},
    {"cosh", Fn::Cosh, 1, 1}, {"tanh", Fn::Tanh, 1, 1}, {"asinh", Fn::Asinh, 1, 1},
    {"acosh", Fn::Acosh, 1, 1}, {"atanh", Fn::Atanh, 1, 1}, {"sqrt", Fn::Sqrt, 1, 1},
    {"exp", Fn::Exp, 1, 1},
};

class Parser {
public:
    explicit Parser(const std::string& s) : s_(s) {}

    ExprP parse() {
        ExprP e = expr(1);
        ws();
        if (i_ != s_.size()) fail("unexpected trailing input");
        return e;
    }

private:
    const std::string& s_;
    size_t i_ = 0;

    [[noreturn]] void fail(const char* what) {
        throw ParseError(std::string("Parse Error: ") + what + " at offset " + std::to_string(i_) +
                         " in '" + s_ + "'");
    }
    void ws() {
        while (i_ < s_.size() && (s_[i_] == ' ' || s_[i_] == '\t' || s_[i_] == '\n' || s_[i_] == '\r'))
            ++i_;
    }
    bool eat(const char* tok) {
        ws();
        size_t n = std::strlen(tok);
        if (s_.compare(i_, n, tok) == 0) { i_ += n; return true; }
        return false;
    }
    // Binary operator at the cursor (not consumed): op, precedence, length.
    bool peek_bin(Op& op, int& prec, size_t& len) {
        ws();
        if (i_ >= s_.size()) return false;
        auto two = s_.substr(i_, 2);
        if (two == "||") { op = Op::Or; prec = 1; len = 2; return true; }
        if (two == "&&") { op = Op::And; prec = 2; len = 2; return true; }
        if (two == "==") { op = Op::Eq; prec = 3; len = 2; return true; }
        if (two == "!=") { op = Op::Ne; prec = 3; len = 2; return true; }
        if (two == "<=") { op = Op::Le; prec = 3; len = 2; return true; }
        if (two == ">=") { op = Op::Ge; prec = 3; len = 2; return true; }
        len = 1;
        switch (s_[i_]) {
        case '<': op = Op::Lt; prec = 3; return true;
        case '>': op = Op::Gt; prec = 3; return true;
        case '+': op = Op::Add; prec = 4; return true;
        case '-': op = Op::Sub; prec = 4; return true;
        case '*': op = Op::Mul; prec = 5; return true;
        case '/': op = Op::Div; prec = 5; return true;
        case '%': op = Op::Mod; prec = 5; return true;
        case '^': op = Op::Pow; prec = 6; return true;
        default: return false;
        }
    }
    ExprP expr(int min_prec) {
        ExprP lhs = value();
        for (;;) {
            Op op; int prec; size_t len;
            if (!peek_bin(op, prec, len) || prec < min_prec) break;
            i_ += len;
            ExprP rhs = expr(op == Op::Pow ? prec : prec + 1);
            auto e = std::make_shared<Expr>();
            e->op = op;
            e->args = {lhs, rhs};
            lhs = e;
        }
        return lhs;
    }
    ExprP value() {
        ws();
        if (i_ >= s_.size()) fail("unexpected end of expression");
        char c = s_[i_];
        if (c == '-' || c == '+' || c == '!') {
            ++i_;
            ExprP v = value();
            if (c == '+') return v;
            auto e = std::make_shared<Expr>();
            e->op = c == '-' ? Op::Neg : Op::Not;
            e->args = {v};
            return e;
        }
        if (c == '(') {
            ++i_;
            ExprP v = expr(1);
            if (!eat(")")) fail("expected ')'");
            return v;
        }
        if ((c >= '0' && c <= '9') || c == '.') {
            size_t j = i_;
            while (j < s_.size() && ((s_[j] >= '0' && s_[j] <= '9') || s_[j] == '.')) ++j;
            if (j < s_.size() && (s_[j] == 'e' || s_[j] == 'E')) {
                size_t k = j + 1;
                if (k < s_.size() && (s_[k] == '+' || s_[k] == '-')) ++k;
                if (k < s_.size() && s_[k] >= '0' && s_[k] <= '9') {
                    while (k < s_.size() && s_[k] >= '0' && s_[k] <= '9') ++k;
                    j = k;
                }
            }
            std::string lit = s_.substr(i_, j - i_);
            char* end = nullptr;
            double v = std::strtod(lit.c_str(), &end);
            if (lit.empty() || end != lit.c_str() + lit.size()) fail("bad number");
            i_ = j;
            auto e = std::make_shared<Expr>();
            e->op = Op::Const;
            e->value = v;
            return e;
        }
        auto ident_start = [](char ch) { return std::isalpha((unsigned char)ch) || ch == '_'; };
        auto ident_char = [](char ch) { return std::isalnum((unsigned char)ch) || ch == '_'; };
        if (ident_start(c)) {
            size_t j = i_;
            while (j < s_.size() && ident_char(s_[j])) ++j;
            std::string name = s_.substr(i_, j - i_);
            i_ = j;
            ws();
            if (i_ < s_.size() && s_[i_] == '(') {
                const FnInfo* fi = nullptr;
                for (const auto& f : kFns)
                    if (name == f.name) fi = &f;
                if (!fi) fail("unknown function");
                ++i_;
                auto e = std::make_shared<Expr>();
                e->op = Op::Call;
                e->fn = fi->fn;
                e->name = name;
                ws();
                if (!(i_ < s_.size() && s_[i_] == ')')) {
                    for (;;) {
                        e->args.push_back(expr(1));
                        if (eat(",")) continue;
                        break;
                    }
                }
                if (!eat(")")) fail("expected ')' after arguments");
                if ((int)e->args.size() < fi->lo || (int)e->args.size() > fi->hi)
                    fail("wrong number of arguments");
                return e;
            }
            auto e = std::make_shared<Expr>();
            e->op = Op::Var;
            e->name = name;
            return e;
        }
        fail("unexpected character");
    }
};

}  // namespace

ExprP parse_expression(const std::string& text) { return Parser(text).parse(); }

// ---------------------------------------------------------------------------
// Builders and derivatives
// ---------------------------------------------------------------------------

ExprP mk_const(double v) {
    auto e = std::make_shared<Expr>();
    e->op = Op::Const;
    e->value = v;
    return e;
}

ExprP mk_var(VarKind k, int idx, const std::string& name) {
    auto e = std::make_shared<Expr>();
    e->op = Op::Var;
    e->vk = k;
    e->idx = idx;
    e->name = name;
    return e;
}

bool is_const(const ExprP& e, double v) { return e->op == Op::Const && e->value == v; }

ExprP mk_un(Op op, ExprP a) {
    if (op == Op::Neg && a->op == Op::Const) return mk_const(-a->value);
    if (op == Op::Neg && a->op == Op::Neg) return a->args[0];
    auto e = std::make_shared<Expr>();
    e->op = op;
    e->args = {a};
    return e;
}

ExprP mk_bin(Op op, ExprP a, ExprP b) {
    switch (op) {
    case Op::Add:
        if (is_const(a, 0.0)) return b;
        if (is_const(b, 0.0)) return a;
        break;
    case Op::Sub:
        if (is_const(b, 0.0)) return a;
        if (is_const(a, 0.0)) return mk_un(Op::Neg, b);
        break;
    case Op::Mul:
        if (is_const(a, 0.0) || is_const(b, 0.0)) return mk_const(0.0);
        if (is_const(a, 1.0)) return b;
        if (is_const(b, 1.0)) return a;
        break;
    case Op::Div:
        if (is_const(a, 0.0)) return mk_const(0.0);
        if (is_const(b, 1.0)) return a;
        break;
    default:
        break;
    }
    auto e = std::make_shared<Expr>();
    e->op = op;
    e->args = {a, b};
    return e;
}

ExprP mk_call(Fn fn, std::vector<ExprP> args) {
    auto e = std::make_shared<Expr>();
    e->op = Op::Call;
    e->fn = fn;
    e->args = std::move(args);
    return e;
}

bool depends_on(const ExprP& e, VarKind kind, int idx) {
    if (e->op == Op::Var) return e->vk == kind && e->idx == idx;
    for (const auto& a : e->args)
        if (depends_on(a, kind, idx)) return true;
    return false;
}

// Chain-rule factor f'(g) * g': zero wherever g' is zero, even when f'(g)
// is infinite there (sqrt or a negative power at 0).
static ExprP chain(const ExprP& outer, const ExprP& inner) {
    if (is_const(inner, 0.0)) return mk_const(0.0);
    if (is_const(inner, 1.0)) return outer;
    if (is_const(outer, 1.0)) return inner;
    return mk_call(Fn::Mul0, {outer, inner});
}

static ExprP select(const ExprP& cond, const ExprP& a, const ExprP& b) {
    if (a->op == Op::Const && b->op == Op::Const && a->value == b->value) return a;
    return mk_call(Fn::Sel, {cond, a, b});
}

ExprP derivative(const ExprP& e, VarKind kind, int idx) {
    if (!depends_on(e, kind, idx)) return mk_const(0.0);
    auto d = [&](int i) { return derivative(e->args[i], kind, idx); };
    auto one = [] { return mk_const(1.0); };
    const auto& A = e->args;
    switch (e->op) {
    case Op::Const: return mk_const(0.0);
    case Op::Var: return mk_const(1.0);
    case Op::Neg: return mk_un(Op::Neg, d(0));
    case Op::Add: return mk_bin(Op::Add, d(0), d(1));
    case Op::Sub: return mk_bin(Op::Sub, d(0), d(1));
    case Op::Mul: return mk_bin(Op::Add, chain(A[1], d(0)), chain(A[0], d(1)));
    case Op::Div:
        // (a/b)' = a'/b - a b' / b^2
        return mk_bin(Op::Sub, chain(mk_bin(Op::Div, one(), A[1]), d(0)),
                      chain(mk_bin(Op::Div, A[0], mk_bin(Op::Mul, A[1], A[1])), d(1)));
    case Op::Mod: return d(0);  // a - trunc(a/b) b, piecewise
    case Op::Pow: {
        if (A[1]->op == Op::Const) {  // c a^(c-1) a'
            double c = A[1]->value;
            if (c == 0.0) return mk_const(0.0);
            ExprP pw = c == 1.0 ? one() : (c == 2.0 ? A[0] : mk_bin(Op::Pow, A[0], mk_const(c - 1.0)));
            return chain(mk_bin(Op::Mul, mk_const(c), pw), d(0));
        }
        // a^b (b' ln a + b a'/a)
        ExprP lna = mk_call(Fn::Log, {mk_call(Fn::E, {}), A[0]});
        return mk_bin(Op::Add, chain(mk_bin(Op::Mul, e, lna), d(1)),
                      chain(mk_bin(Op::Div, mk_bin(Op::Mul, e, A[1]), A[0]), d(0)));
    }
    case Op::Eq: case Op::Ne: case Op::Lt: case Op::Le: case Op::Gt: case Op::Ge:
    case Op::Not:
        return mk_const(0.0);
    case Op::And:  // a if a == 0 else b
        return select(mk_call(Fn::Abs, {A[0]}), d(1), d(0));
    case Op::Or:   // a if a != 0 else b
        return select(mk_call(Fn::Abs, {A[0]}), d(0), d(1));
    case Op::Call:
        break;
    }
    switch (e->fn) {
    case Fn::Min: case Fn::Max: {
        // fold left: m = op(m, a_i); the derivative follows the operand taken
        ExprP m = A[0], dm = d(0);
        for (size_t i = 1; i < A.size(); ++i) {
            ExprP di = derivative(A[i], kind, idx);
            ExprP diff = e->fn == Fn::Max ? mk_bin(Op::Sub, A[i], m) : mk_bin(Op::Sub, m, A[i]);
            dm = select(diff, di, dm);
            m = mk_call(e->fn, {m, A[i]});
        }
        return dm;
    }
    case Fn::Abs: return chain(mk_call(Fn::Sign, {A[0]}), d(0));
    case Fn::Sign: case Fn::Int: case Fn::Ceil: case Fn::Floor: case Fn::Round:
    case Fn::E: case Fn::Pi: case Fn::Step:
        return mk_const(0.0);
    case Fn::Log: {
        if (A.size() == 1)
            return chain(mk_bin(Op::Div, one(), mk_bin(Op::Mul, A[0], mk_const(std::log(10.0)))), d(0));
        // log_b(x) = ln x / ln b
        ExprP lnx = mk_call(Fn::Log, {mk_call(Fn::E, {}), A[1]});
        ExprP lnb = mk_call(Fn::Log, {mk_call(Fn::E, {}), A[0]});
        ExprP dx = chain(mk_bin(Op::Div, one(), mk_bin(Op::Mul, A[1], lnb)), derivative(A[1], kind, idx));
        ExprP db = chain(mk_bin(Op::Div, lnx, mk_bin(Op::Mul, A[0], mk_bin(Op::Mul, lnb, lnb))),
                         derivative(A[0], kind, idx));
        return mk_bin(Op::Sub, dx, db);
    }
    case Fn::Sin: return chain(mk_call(Fn::Cos, {A[0]}), d(0));
    case Fn::Cos: return chain(mk_un(Op::Neg, mk_call(Fn::Sin, {A[0]})), d(0));
    case Fn::Tan: {
        ExprP c = mk_call(Fn::Cos, {A[0]});
        return chain(mk_bin(Op::Div, one(), mk_bin(Op::Mul, c, c)), d(0));
    }
    case Fn::Asin:
        return chain(mk_bin(Op::Div, one(), mk_call(Fn::Sqrt, {mk_bin(Op::Sub, one(), mk_bin(Op::Mul, A[0], A[0]))})), d(0));
    case Fn::Acos:
        return chain(mk_bin(Op::Div, mk_const(-1.0), mk_call(Fn::Sqrt, {mk_bin(Op::Sub, one(), mk_bin(Op::Mul, A[0], A[0]))})), d(0));
    case Fn::Atan:
        return chain(mk_bin(Op::Div, one(), mk_bin(Op::Add, one(), mk_bin(Op::Mul, A[0], A[0]))), d(0));
    case Fn::Sinh: return chain(mk_call(Fn::Cosh, {A[0]}), d(0));
    case Fn::Cosh: return chain(mk_call(Fn::Sinh, {A[0]}), d(0));
    case Fn::Tanh: {
        ExprP th = mk_call(Fn::Tanh, {A[0]});
        return chain(mk_bin(Op::Sub, one(), mk_bin(Op::Mul, th, th)), d(0));
    }
    case Fn::Asinh:
        return chain(mk_bin(Op::Div, one(), mk_call(Fn::Sqrt, {mk_bin(Op::Add, mk_bin(Op::Mul, A[0], A[0]), one())})), d(0));
    case Fn::Acosh:
        return chain(mk_bin(Op::Div, one(), mk_call(Fn::Sqrt, {mk_bin(Op::Sub, mk_bin(Op::Mul, A[0], A[0]), one())})), d(0));
    case Fn::Atanh:
        return chain(mk_bin(Op::Div, one(), mk_bin(Op::Sub, one(), mk_bin(Op::Mul, A[0], A[0]))), d(0));
    case Fn::Sqrt:
        return chain(mk_bin(Op::Div, one(), mk_bin(Op::Mul, mk_const(2.0), mk_call(Fn::Sqrt, {A[0]}))), d(0));
    case Fn::Exp:
        return chain(e, d(0));
    case Fn::Mul0: case Fn::Sel:
        return mk_const(0.0);  // never differentiated: only produced by derivatives
    }
    return mk_const(0.0);
}

// ---------------------------------------------------------------------------
// Equation grammar: restatement of parse_single_equation / build_incrementor
// (src/proc/util.rs:68-166).
// ---------------------------------------------------------------------------

namespace {

bool is_ws(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\v' || c == '\f'; }

std::string trim(const std::string& s) {
    size_t a = 0, b = s.size();
    while (a < b && is_ws(s[a])) ++a;
    while (b > a && is_ws(s[b - 1])) --b;
    return s.substr(a, b - a);
}

std::string trim_start(const std::string& s) {
    size_t a = 0;
    while (a < s.size() && is_ws(s[a])) ++a;
    return s.substr(a);
}

// balanced_parens (util.rs:16-38): length consumed before an unmatched ')'
// or the end, or -1 when a nested pair does not close.
long balanced(const std::string& s, size_t from) {
    size_t i = from;
    while (i < s.size()) {
        if (s[i] == '(') {
            long c = balanced(s, i + 1);
            if (c < 0) return -1;
            i += 1 + (size_t)c;
            if (i >= s.size() || s[i] != ')') return -1;
            ++i;
        } else if (s[i] == ')') {
            break;
        } else {
            while (i < s.size() && s[i] != '(' && s[i] != ')') ++i;
        }
    }
    return (long)(i - from);
}

// delimited('(', balanced_parens, ')') at s[at] == '(' : content, total length
bool delimited(const std::string& s, size_t at, std::string& content, size_t& total) {
    if (at >= s.size() || s[at] != '(') return false;
    long c = balanced(s, at + 1);
    if (c < 0) return false;
    size_t close = at + 1 + (size_t)c;
    if (close >= s.size() || s[close] != ')') return false;
    content = s.substr(at + 1, (size_t)c);
    total = (size_t)c + 2;
    return true;
}

}  // namespace

int Universe::process_index(const std::string& name) const {
    int idx = -1;
    for (int p = 0; p < (int)procs.size(); ++p)
        if (procs[p].name == name) idx = p;
    return idx;
}

ExprP Universe::resolve(const ExprP& e) const {
    if (e->op == Op::Var) {
        int p = process_index(e->name);
        if (p >= 0) return mk_var(VarKind::Process, p, e->name);
        if (e->name == "t") return mk_var(VarKind::Time, 0, e->name);
        for (int k = 0; k < (int)params.size(); ++k)
            if (params[k] == e->name) return mk_var(VarKind::Param, k, e->name);
        throw ParseError("Unknown variable '" + e->name + "'");
    }
    if (e->args.empty()) return e;
    auto c = std::make_shared<Expr>(*e);
    for (auto& a : c->args) a = resolve(a);
    return c;
}

static Term build_term(Universe& u, const std::string& coeff, const std::string& inc) {
    Term t;
    try {
        t.coef = parse_expression(trim(coeff));
    } catch (const ParseError& e) {
        throw ParseError(std::string("Math error in coefficient: ") + e.what());
    }
    if (inc == "dt") {
        t.kind = IncKind::Dt;
        return t;
    }
    bool w = inc.rfind("dW", 0) == 0, n = inc.rfind("dN", 0) == 0;
    if (!w && !n) throw ParseError("Unknown incrementor type: " + inc);
    int idx = -1;
    for (int i = 0; i < (int)u.tokens.size(); ++i)
        if (u.tokens[i] == inc) idx = i;
    if (idx < 0) {
        idx = (int)u.tokens.size();
        u.tokens.push_back(inc);
        u.token_kind.push_back(w ? IncKind::Dw : IncKind::Dn);
    }
    t.sidx = idx;
    if (w) {
        t.kind = IncKind::Dw;
        return t;
    }
    // extract_lambda (util.rs:41-50)
    size_t lp = inc.find('(');
    if (lp == std::string::npos) throw ParseError("Missing '(' in dN incrementor");
    std::string content;
    size_t total;
    if (!delimited(inc, lp, content, total))
        throw ParseError("Unbalanced parentheses in jump term: " + inc);
    std::string lam = trim(content);
    try {
        t.lambda = parse_expression(lam);
    } catch (const ParseError& e) {
        throw ParseError("Math error in jump lambda '" + lam + "': " + e.what());
    }
    t.kind = IncKind::Dn;
    return t;
}

static Process parse_single(Universe& u, const std::string& eq) {
    size_t first = eq.find('=');
    if (first == std::string::npos || eq.find('=', first + 1) != std::string::npos)
        throw ParseError("Missing '='");
    std::string lhs = trim(eq.substr(0, first));
    std::string rhs = trim(eq.substr(first + 1));
    Process p;
    p.levy = !lhs.empty() && lhs[0] == 'd';
    p.name = p.levy ? lhs.substr(1) : lhs;
    if (!p.levy) {
        p.alg = parse_expression(rhs);
        return p;
    }
    std::string cur = rhs;
    for (;;) {
        size_t start = cur.find('(');
        if (start == std::string::npos) break;
        std::string coeff;
        size_t total;
        if (!delimited(cur, start, coeff, total)) throw ParseError("Unbalanced parentheses in coefficient");
        std::string after = trim_start(cur.substr(start + total));
        if (after.empty() || after[0] != '*') break;
        std::string as = trim_start(after.substr(1));
        std::string inc, rest;
        if (as.rfind("dN", 0) == 0) {
            size_t dp = as.find('(');
            if (dp == std::string::npos) throw ParseError("dN missing opening bracket");
            std::string inside;
            size_t dtot;
            if (!delimited(as, dp, inside, dtot)) throw ParseError("Unbalanced parentheses in dN intensity");
            inc = as.substr(0, dp + dtot);
            rest = as.substr(dp + dtot);
        } else {
            size_t sp = as.find(' ');
            size_t end = sp == std::string::npos ? as.size() : sp;
            inc = as.substr(0, end);
            rest = as.substr(end);
        }
        p.terms.push_back(build_term(u, coeff, inc));
        cur = rest;
    }
    return p;
}

Universe parse_universe(const std::vector<std::string>& equations,
                        const std::vector<std::string>& params) {
    Universe u;
    u.params = params;
    for (const auto& eq : equations) u.procs.push_back(parse_single(u, eq));
    for (int p = 0; p < (int)u.procs.size(); ++p) {
        if (u.procs[p].levy) u.levy.push_back(p);
        else u.alg.push_back(p);
    }
    for (int k = 0; k < (int)params.size(); ++k)
        if (u.process_index(params[k]) >= 0)
            throw ParseError("Parameter '" + params[k] + "' has the name of a process");
    for (auto& p : u.procs) {
        for (auto& t : p.terms) {
            t.coef = u.resolve(t.coef);
            if (t.lambda) t.lambda = u.resolve(t.lambda);
        }
        if (p.alg) p.alg = u.resolve(p.alg);
    }
    return u;
}

}  // namespace sde
