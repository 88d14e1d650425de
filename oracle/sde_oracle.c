/*
 * sde_oracle.c -- CPU restatement of the sde-sim-rs path-simulation
 * algorithm.  TEST INFRASTRUCTURE ONLY: what the GPU engine's parity tests
 * compare with, and the timed CPU baseline; never part of the product path.
 *
 * Compile with -ffp-contract=off: the reference (Rust) never contracts
 * a*b+c into a fused multiply-add, and aarch64 gcc would otherwise do so.
 *
 * Every function cites the reference file:line it restates.  Paths are
 * relative to the sde-sim-rs crate root.
 */
#include "sde_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define ORC_MAXARGS 16

static void set_err(char* err, size_t n, const char* fmt, ...) {
    if (!err || n == 0) return;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(err, n, fmt, ap);
    va_end(ap);
}

/* ======================================================================
 * Expression grammar -- restatement of fasteval 0.2.4 as used by
 * src/func.rs:18-42.  Unary + - ! bind to the following value (tighter than
 * ^); ^ is right associative; precedence low->high: || && comparisons + -
 * * / % ^.  Comparisons yield 1.0 / 0.0; == != <= >= use fasteval's 8*eps
 * absolute tolerance.  Builtins: min max abs sign int ceil floor round log e
 * pi sin cos tan asin acos atan sinh cosh tanh asinh acosh atanh, plus the
 * documented extensions sqrt and exp.
 * ==================================================================== */

typedef enum {
    N_CONST, N_VAR, N_NEG, N_NOT, N_BIN, N_CALL
} nkind;

typedef enum {
    B_OR, B_AND, B_EQ, B_NE, B_LT, B_LE, B_GT, B_GE,
    B_ADD, B_SUB, B_MUL, B_DIV, B_MOD, B_POW
} bop;

typedef enum {
    F_MIN, F_MAX, F_ABS, F_SIGN, F_INT, F_CEIL, F_FLOOR, F_ROUND, F_LOG,
    F_E, F_PI, F_SIN, F_COS, F_TAN, F_ASIN, F_ACOS, F_ATAN, F_SINH, F_COSH,
    F_TANH, F_ASINH, F_ACOSH, F_ATANH, F_SQRT, F_EXP
} fnid;

typedef struct enode {
    nkind kind;
    int op;            /* bop or fnid */
    double c;          /* constant */
    char* name;        /* variable name (before resolution) */
    int slot;          /* resolved slot */
    int nargs;
    struct enode* a[ORC_MAXARGS];
} enode;

static void enode_free(enode* e) {
    if (!e) return;
    for (int i = 0; i < e->nargs; ++i) enode_free(e->a[i]);
    free(e->name);
    free(e);
}

static enode* enode_new(nkind k) {
    enode* e = (enode*)calloc(1, sizeof(enode));
    e->kind = k;
    e->slot = -1;
    return e;
}

typedef struct {
    const char* s;
    size_t i, n;
    char* err;
    size_t errlen;
    int failed;
} lexer;

static void skip_ws(lexer* L) {
    while (L->i < L->n && (L->s[L->i] == ' ' || L->s[L->i] == '\t' ||
                           L->s[L->i] == '\n' || L->s[L->i] == '\r'))
        L->i++;
}

static int peek(lexer* L) { skip_ws(L); return L->i < L->n ? (unsigned char)L->s[L->i] : 0; }

static int accept2(lexer* L, const char* tok) {
    skip_ws(L);
    size_t k = strlen(tok);
    if (L->i + k <= L->n && strncmp(L->s + L->i, tok, k) == 0) { L->i += k; return 1; }
    return 0;
}

static enode* parse_or(lexer* L);

static void fail(lexer* L, const char* msg) {
    if (!L->failed) {
        set_err(L->err, L->errlen, "Parse Error: %s at offset %zu in '%.*s'", msg, L->i,
                (int)L->n, L->s);
    }
    L->failed = 1;
}

static const struct { const char* name; fnid id; int minargs, maxargs; } FUNCS[] = {
    {"min", F_MIN, 1, ORC_MAXARGS}, {"max", F_MAX, 1, ORC_MAXARGS},
    {"abs", F_ABS, 1, 1}, {"sign", F_SIGN, 1, 1}, {"int", F_INT, 1, 1},
    {"ceil", F_CEIL, 1, 1}, {"floor", F_FLOOR, 1, 1}, {"round", F_ROUND, 1, 2},
    {"log", F_LOG, 1, 2}, {"e", F_E, 0, 0}, {"pi", F_PI, 0, 0},
    {"sin", F_SIN, 1, 1}, {"cos", F_COS, 1, 1}, {"tan", F_TAN, 1, 1},
    {"asin", F_ASIN, 1, 1}, {"acos", F_ACOS, 1, 1}, {"atan", F_ATAN, 1, 1},
    {"sinh", F_SINH, 1, 1}, {"cosh", F_COSH, 1, 1}, {"tanh", F_TANH, 1, 1},
    {"asinh", F_ASINH, 1, 1}, {"acosh", F_ACOSH, 1, 1}, {"atanh", F_ATANH, 1, 1},
    {"sqrt", F_SQRT, 1, 1}, {"exp", F_EXP, 1, 1},
};

static int is_ident_start(int c) { return (c >= 'a' && c <= 'z') || (c >= 'A' && c <= 'Z') || c == '_'; }
static int is_ident_char(int c) { return is_ident_start(c) || (c >= '0' && c <= '9'); }

static enode* parse_value(lexer* L) {
    int c = peek(L);
    if (L->failed) return NULL;
    if (c == '-' || c == '+' || c == '!') {
        L->i++;
        enode* v = parse_value(L);
        if (!v) return NULL;
        if (c == '+') return v;
        enode* e = enode_new(c == '-' ? N_NEG : N_NOT);
        e->a[0] = v;
        e->nargs = 1;
        return e;
    }
    if (c == '(') {
        L->i++;
        enode* v = parse_or(L);
        if (!v) return NULL;
        if (!accept2(L, ")")) { enode_free(v); fail(L, "expected ')'"); return NULL; }
        return v;
    }
    if ((c >= '0' && c <= '9') || c == '.') {
        const char* start = L->s + L->i;
        size_t j = L->i;
        while (j < L->n && ((L->s[j] >= '0' && L->s[j] <= '9') || L->s[j] == '.')) j++;
        if (j < L->n && (L->s[j] == 'e' || L->s[j] == 'E')) {
            size_t k = j + 1;
            if (k < L->n && (L->s[k] == '+' || L->s[k] == '-')) k++;
            if (k < L->n && L->s[k] >= '0' && L->s[k] <= '9') {
                while (k < L->n && L->s[k] >= '0' && L->s[k] <= '9') k++;
                j = k;
            }
        }
        char buf[128];
        size_t len = j - L->i;
        if (len == 0 || len >= sizeof buf) { fail(L, "bad number"); return NULL; }
        memcpy(buf, start, len);
        buf[len] = 0;
        char* endp = NULL;
        double v = strtod(buf, &endp);
        if (endp != buf + len) { fail(L, "bad number"); return NULL; }
        L->i = j;
        enode* e = enode_new(N_CONST);
        e->c = v;
        return e;
    }
    if (is_ident_start(c)) {
        size_t j = L->i;
        while (j < L->n && is_ident_char((unsigned char)L->s[j])) j++;
        size_t len = j - L->i;
        char* name = (char*)malloc(len + 1);
        memcpy(name, L->s + L->i, len);
        name[len] = 0;
        L->i = j;
        if (peek(L) == '(') {
            int fi = -1;
            for (size_t k = 0; k < sizeof FUNCS / sizeof FUNCS[0]; ++k)
                if (strcmp(FUNCS[k].name, name) == 0) { fi = (int)k; break; }
            if (fi < 0) { free(name); fail(L, "unknown function"); return NULL; }
            free(name);
            L->i++; /* '(' */
            enode* e = enode_new(N_CALL);
            e->op = FUNCS[fi].id;
            if (peek(L) != ')') {
                for (;;) {
                    if (e->nargs >= ORC_MAXARGS) { enode_free(e); fail(L, "too many arguments"); return NULL; }
                    enode* a = parse_or(L);
                    if (!a) { enode_free(e); return NULL; }
                    e->a[e->nargs++] = a;
                    if (accept2(L, ",")) continue;
                    break;
                }
            }
            if (!accept2(L, ")")) { enode_free(e); fail(L, "expected ')' after arguments"); return NULL; }
            if (e->nargs < FUNCS[fi].minargs || e->nargs > FUNCS[fi].maxargs) {
                enode_free(e); fail(L, "wrong number of arguments"); return NULL;
            }
            return e;
        }
        enode* e = enode_new(N_VAR);
        e->name = name;
        return e;
    }
    fail(L, c ? "unexpected character" : "unexpected end of expression");
    return NULL;
}

static enode* mkbin(int op, enode* l, enode* r) {
    enode* e = enode_new(N_BIN);
    e->op = op;
    e->a[0] = l;
    e->a[1] = r;
    e->nargs = 2;
    return e;
}

static enode* parse_pow(lexer* L) {
    enode* l = parse_value(L);
    if (!l) return NULL;
    if (peek(L) == '^') {
        L->i++;
        enode* r = parse_pow(L);
        if (!r) { enode_free(l); return NULL; }
        return mkbin(B_POW, l, r);
    }
    return l;
}

static enode* parse_mul(lexer* L) {
    enode* l = parse_pow(L);
    while (l) {
        int c = peek(L);
        int op = c == '*' ? B_MUL : c == '/' ? B_DIV : c == '%' ? B_MOD : -1;
        if (op < 0) break;
        L->i++;
        enode* r = parse_pow(L);
        if (!r) { enode_free(l); return NULL; }
        l = mkbin(op, l, r);
    }
    return l;
}

static enode* parse_add(lexer* L) {
    enode* l = parse_mul(L);
    while (l) {
        int c = peek(L);
        int op = c == '+' ? B_ADD : c == '-' ? B_SUB : -1;
        if (op < 0) break;
        L->i++;
        enode* r = parse_mul(L);
        if (!r) { enode_free(l); return NULL; }
        l = mkbin(op, l, r);
    }
    return l;
}

static enode* parse_cmp(lexer* L) {
    enode* l = parse_add(L);
    while (l) {
        int op = -1;
        if (accept2(L, "==")) op = B_EQ;
        else if (accept2(L, "!=")) op = B_NE;
        else if (accept2(L, "<=")) op = B_LE;
        else if (accept2(L, ">=")) op = B_GE;
        else if (accept2(L, "<")) op = B_LT;
        else if (accept2(L, ">")) op = B_GT;
        if (op < 0) break;
        enode* r = parse_add(L);
        if (!r) { enode_free(l); return NULL; }
        l = mkbin(op, l, r);
    }
    return l;
}

static enode* parse_and(lexer* L) {
    enode* l = parse_cmp(L);
    while (l && accept2(L, "&&")) {
        enode* r = parse_cmp(L);
        if (!r) { enode_free(l); return NULL; }
        l = mkbin(B_AND, l, r);
    }
    return l;
}

static enode* parse_or(lexer* L) {
    enode* l = parse_and(L);
    while (l && accept2(L, "||")) {
        enode* r = parse_and(L);
        if (!r) { enode_free(l); return NULL; }
        l = mkbin(B_OR, l, r);
    }
    return l;
}

static enode* parse_expr(const char* s, size_t n, char* err, size_t errlen) {
    lexer L = {s, 0, n, err, errlen, 0};
    enode* e = parse_or(&L);
    if (e && peek(&L) != 0) {
        fail(&L, "unexpected trailing input");
        enode_free(e);
        return NULL;
    }
    if (!e && !L.failed) fail(&L, "empty expression");
    return e;
}

#define F64_EPS8 (8.0 * 2.220446049250313e-16)

static double ev(const enode* e, const double* slots) {
    switch (e->kind) {
    case N_CONST: return e->c;
    case N_VAR: return slots[e->slot];
    case N_NEG: return -ev(e->a[0], slots);
    case N_NOT: return fabs(ev(e->a[0], slots)) <= F64_EPS8 ? 1.0 : 0.0;
    case N_BIN: {
        if (e->op == B_AND) {
            double l = ev(e->a[0], slots);
            return fabs(l) <= F64_EPS8 ? l : ev(e->a[1], slots);
        }
        if (e->op == B_OR) {
            double l = ev(e->a[0], slots);
            return fabs(l) > F64_EPS8 ? l : ev(e->a[1], slots);
        }
        double l = ev(e->a[0], slots), r = ev(e->a[1], slots);
        switch (e->op) {
        case B_ADD: return l + r;
        case B_SUB: return l - r;
        case B_MUL: return l * r;
        case B_DIV: return l / r;
        case B_MOD: return fmod(l, r);
        case B_POW: return pow(l, r);
        case B_EQ: return fabs(l - r) <= F64_EPS8 ? 1.0 : 0.0;
        case B_NE: return fabs(l - r) > F64_EPS8 ? 1.0 : 0.0;
        case B_LT: return l < r ? 1.0 : 0.0;
        case B_GT: return l > r ? 1.0 : 0.0;
        case B_LE: return l <= r + F64_EPS8 ? 1.0 : 0.0;
        case B_GE: return l + F64_EPS8 >= r ? 1.0 : 0.0;
        }
        return NAN;
    }
    case N_CALL: {
        double x = e->nargs > 0 ? ev(e->a[0], slots) : 0.0;
        switch (e->op) {
        case F_MIN: case F_MAX: {
            double m = x;
            for (int i = 1; i < e->nargs; ++i) {
                double y = ev(e->a[i], slots);
                m = e->op == F_MIN ? fmin(m, y) : fmax(m, y);
            }
            return m;
        }
        case F_ABS: return fabs(x);
        case F_SIGN: return isnan(x) ? x : (signbit(x) ? -1.0 : 1.0);
        case F_INT: return trunc(x);
        case F_CEIL: return ceil(x);
        case F_FLOOR: return floor(x);
        case F_ROUND: {
            if (e->nargs == 1) return round(x);
            double v = ev(e->a[1], slots);
            return round(v / x) * x;
        }
        case F_LOG: {
            if (e->nargs == 1) return log(x) / log(10.0);
            double v = ev(e->a[1], slots);
            return log(v) / log(x);
        }
        case F_E: return 2.718281828459045;
        case F_PI: return 3.141592653589793;
        case F_SIN: return sin(x);
        case F_COS: return cos(x);
        case F_TAN: return tan(x);
        case F_ASIN: return asin(x);
        case F_ACOS: return acos(x);
        case F_ATAN: return atan(x);
        case F_SINH: return sinh(x);
        case F_COSH: return cosh(x);
        case F_TANH: return tanh(x);
        case F_ASINH: return asinh(x);
        case F_ACOSH: return acosh(x);
        case F_ATANH: return atanh(x);
        case F_SQRT: return sqrt(x);
        case F_EXP: return exp(x);
        }
        return NAN;
    }
    }
    return NAN;
}

/* ======================================================================
 * Universe -- src/proc/mod.rs:61-89, src/proc/util.rs:52-166
 * ==================================================================== */

enum { INC_DT = 0, INC_DW = 1, INC_DN = 2 };

typedef struct {
    int kind;
    int idx;          /* stochastic index (dW/dN) */
    enode* lambda;    /* dN intensity */
} inc_t;

typedef struct {
    char* name;
    int levy;
    int nterms;
    enode** coef;
    inc_t* inc;
    enode* alg;       /* algebraic expression */
} proc_t;

struct orc_universe {
    int P;
    proc_t* procs;
    int n_inc;
    char** tokens;    /* stochastic registry, index -> token */
    int* tok_kind;
    int n_params;
    char** param_names;
    double* param_vals;
    int nlevy, nalg;
    int* levy_idx;
    int* alg_idx;
};

static char* strndup_(const char* s, size_t n) {
    char* r = (char*)malloc(n + 1);
    memcpy(r, s, n);
    r[n] = 0;
    return r;
}

static int is_ws(int c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\v' || c == '\f'; }

static void trim(const char** s, size_t* n) {
    while (*n && is_ws((unsigned char)**s)) { (*s)++; (*n)--; }
    while (*n && is_ws((unsigned char)(*s)[*n - 1])) (*n)--;
}

static void trim_start(const char** s, size_t* n) {
    while (*n && is_ws((unsigned char)**s)) { (*s)++; (*n)--; }
}

/* balanced_parens (src/proc/util.rs:16-38): consume text up to an unmatched
 * ')' or the end; nested pairs must balance.  Returns -1 on failure. */
static long balanced(const char* s, size_t n) {
    size_t i = 0;
    while (i < n) {
        if (s[i] == '(') {
            long c = balanced(s + i + 1, n - i - 1);
            if (c < 0) return -1;
            i += 1 + (size_t)c;
            if (i >= n || s[i] != ')') return -1;
            i++;
        } else if (s[i] == ')') {
            break;
        } else {
            while (i < n && s[i] != '(' && s[i] != ')') i++;
        }
    }
    return (long)i;
}

/* delimited('(', balanced_parens, ')') at s[0]=='(' -> content length, or -1 */
static long delimited(const char* s, size_t n, size_t* total) {
    if (n == 0 || s[0] != '(') return -1;
    long c = balanced(s + 1, n - 1);
    if (c < 0) return -1;
    if ((size_t)c + 1 >= n || s[c + 1] != ')') return -1;
    *total = (size_t)c + 2;
    return c;
}

static const char* memchr_c(const char* s, size_t n, char c) { return (const char*)memchr(s, c, n); }

/* build_incrementor (src/proc/util.rs:136-166) */
static int build_incrementor(orc_universe* u, const char* tok, size_t tn, inc_t* out,
                             char* err, size_t errlen) {
    memset(out, 0, sizeof *out);
    if (tn == 2 && strncmp(tok, "dt", 2) == 0) { out->kind = INC_DT; return 0; }
    int idx = -1;
    for (int i = 0; i < u->n_inc; ++i)
        if (strlen(u->tokens[i]) == tn && strncmp(u->tokens[i], tok, tn) == 0) { idx = i; break; }
    int is_w = tn >= 2 && strncmp(tok, "dW", 2) == 0;
    int is_n = tn >= 2 && strncmp(tok, "dN", 2) == 0;
    if (!is_w && !is_n) {
        set_err(err, errlen, "Unknown incrementor type: %.*s", (int)tn, tok);
        return 1;
    }
    if (idx < 0) {
        u->tokens = (char**)realloc(u->tokens, sizeof(char*) * (u->n_inc + 1));
        u->tok_kind = (int*)realloc(u->tok_kind, sizeof(int) * (u->n_inc + 1));
        u->tokens[u->n_inc] = strndup_(tok, tn);
        u->tok_kind[u->n_inc] = is_w ? INC_DW : INC_DN;
        idx = u->n_inc++;
    }
    out->idx = idx;
    if (is_w) { out->kind = INC_DW; return 0; }
    /* extract_lambda (src/proc/util.rs:41-50) */
    const char* lp = memchr_c(tok, tn, '(');
    if (!lp) { set_err(err, errlen, "Missing '(' in dN incrementor"); return 1; }
    size_t total;
    long c = delimited(lp, tn - (size_t)(lp - tok), &total);
    if (c < 0) { set_err(err, errlen, "Unbalanced parentheses in jump term: %.*s", (int)tn, tok); return 1; }
    const char* ls = lp + 1;
    size_t ln = (size_t)c;
    trim(&ls, &ln);
    char sub[512];
    out->lambda = parse_expr(ls, ln, sub, sizeof sub);
    if (!out->lambda) {
        set_err(err, errlen, "Math error in jump lambda '%.*s': %s", (int)ln, ls, sub);
        return 1;
    }
    out->kind = INC_DN;
    return 0;
}

/* parse_single_equation (src/proc/util.rs:68-134) */
static int parse_single(orc_universe* u, const char* eq, proc_t* p, char* err, size_t errlen) {
    memset(p, 0, sizeof *p);
    size_t n = strlen(eq);
    const char* eqp = memchr_c(eq, n, '=');
    if (!eqp || memchr_c(eqp + 1, n - (size_t)(eqp - eq) - 1, '=')) {
        set_err(err, errlen, "Missing '='");
        return 1;
    }
    const char* lhs = eq;
    size_t lhn = (size_t)(eqp - eq);
    const char* rhs = eqp + 1;
    size_t rhn = n - lhn - 1;
    trim(&lhs, &lhn);
    trim(&rhs, &rhn);
    int levy = lhn > 0 && lhs[0] == 'd';
    p->name = levy ? strndup_(lhs + 1, lhn - 1) : strndup_(lhs, lhn);
    p->levy = levy;
    if (!levy) {
        p->alg = parse_expr(rhs, rhn, err, errlen);
        return p->alg ? 0 : 1;
    }
    const char* cur = rhs;
    size_t cn = rhn;
    for (;;) {
        const char* op = memchr_c(cur, cn, '(');
        if (!op) break;
        size_t off = (size_t)(op - cur), total;
        long clen = delimited(op, cn - off, &total);
        if (clen < 0) { set_err(err, errlen, "Unbalanced parentheses in coefficient"); return 1; }
        const char* coeff = op + 1;
        size_t coeffn = (size_t)clen;
        const char* after = op + total;
        size_t an = cn - off - total;
        trim_start(&after, &an);
        if (an == 0 || after[0] != '*') break;
        const char* as = after + 1;
        size_t asn = an - 1;
        trim_start(&as, &asn);
        const char* tok = as;
        size_t tn;
        const char* rest;
        size_t restn;
        if (asn >= 2 && strncmp(as, "dN", 2) == 0) {
            const char* dp = memchr_c(as, asn, '(');
            if (!dp) { set_err(err, errlen, "dN missing opening bracket"); return 1; }
            size_t dtot;
            if (delimited(dp, asn - (size_t)(dp - as), &dtot) < 0) {
                set_err(err, errlen, "Unbalanced parentheses in dN intensity");
                return 1;
            }
            tn = (size_t)(dp - as) + dtot;
            rest = as + tn;
            restn = asn - tn;
        } else {
            const char* sp = memchr_c(as, asn, ' ');
            tn = sp ? (size_t)(sp - as) : asn;
            rest = as + tn;
            restn = asn - tn;
        }
        trim(&coeff, &coeffn);
        char sub[512];
        enode* ce = parse_expr(coeff, coeffn, sub, sizeof sub);
        if (!ce) { set_err(err, errlen, "Math error in coefficient: %s", sub); return 1; }
        inc_t inc;
        if (build_incrementor(u, tok, tn, &inc, err, errlen)) { enode_free(ce); return 1; }
        p->coef = (enode**)realloc(p->coef, sizeof(enode*) * (p->nterms + 1));
        p->inc = (inc_t*)realloc(p->inc, sizeof(inc_t) * (p->nterms + 1));
        p->coef[p->nterms] = ce;
        p->inc[p->nterms] = inc;
        p->nterms++;
        cur = rest;
        cn = restn;
    }
    return 0;
}

/* Name -> slot: 0 is "t", 1+p is process p (the registry keeps the last
 * process of a name, src/proc/mod.rs:75-77), then parameters. */
static int resolve(const orc_universe* u, enode* e, char* err, size_t errlen) {
    if (!e) return 0;
    if (e->kind == N_VAR) {
        int slot = -1;
        for (int p = 0; p < u->P; ++p)
            if (strcmp(u->procs[p].name, e->name) == 0) slot = 1 + p;
        if (slot < 0 && strcmp(e->name, "t") == 0) slot = 0;
        if (slot < 0)
            for (int k = 0; k < u->n_params; ++k)
                if (strcmp(u->param_names[k], e->name) == 0) slot = 1 + u->P + k;
        if (slot < 0) { set_err(err, errlen, "Unknown variable '%s'", e->name); return 1; }
        e->slot = slot;
        return 0;
    }
    for (int i = 0; i < e->nargs; ++i)
        if (resolve(u, e->a[i], err, errlen)) return 1;
    return 0;
}

void orc_free(orc_universe* u) {
    if (!u) return;
    for (int p = 0; p < u->P; ++p) {
        proc_t* q = &u->procs[p];
        free(q->name);
        for (int j = 0; j < q->nterms; ++j) { enode_free(q->coef[j]); enode_free(q->inc[j].lambda); }
        free(q->coef);
        free(q->inc);
        enode_free(q->alg);
    }
    free(u->procs);
    for (int i = 0; i < u->n_inc; ++i) free(u->tokens[i]);
    free(u->tokens);
    free(u->tok_kind);
    for (int k = 0; k < u->n_params; ++k) free(u->param_names[k]);
    free(u->param_names);
    free(u->param_vals);
    free(u->levy_idx);
    free(u->alg_idx);
    free(u);
}

/* parse_equations (src/proc/util.rs:52-66) + ProcessUniverse::new
 * (src/proc/mod.rs:70-89) */
int orc_parse(const char* const* eqs, int n_eq, const char* const* param_names,
              const double* param_vals, int n_params, orc_universe** out,
              char* err, size_t errlen) {
    orc_universe* u = (orc_universe*)calloc(1, sizeof *u);
    u->procs = (proc_t*)calloc(n_eq > 0 ? n_eq : 1, sizeof(proc_t));
    u->n_params = n_params;
    u->param_names = (char**)calloc(n_params > 0 ? n_params : 1, sizeof(char*));
    u->param_vals = (double*)calloc(n_params > 0 ? n_params : 1, sizeof(double));
    for (int k = 0; k < n_params; ++k) {
        u->param_names[k] = strndup_(param_names[k], strlen(param_names[k]));
        u->param_vals[k] = param_vals[k];
    }
    for (int i = 0; i < n_eq; ++i) {
        if (parse_single(u, eqs[i], &u->procs[i], err, errlen)) {
            u->P = i + 1;
            orc_free(u);
            return 1;
        }
        u->P = i + 1;
    }
    u->P = n_eq;
    u->levy_idx = (int*)calloc(n_eq > 0 ? n_eq : 1, sizeof(int));
    u->alg_idx = (int*)calloc(n_eq > 0 ? n_eq : 1, sizeof(int));
    for (int p = 0; p < n_eq; ++p) {
        if (u->procs[p].levy) u->levy_idx[u->nlevy++] = p;
        else u->alg_idx[u->nalg++] = p;
    }
    for (int p = 0; p < n_eq; ++p) {
        proc_t* q = &u->procs[p];
        for (int j = 0; j < q->nterms; ++j)
            if (resolve(u, q->coef[j], err, errlen) || resolve(u, q->inc[j].lambda, err, errlen)) {
                orc_free(u);
                return 1;
            }
        if (resolve(u, q->alg, err, errlen)) { orc_free(u); return 1; }
    }
    *out = u;
    return 0;
}

int orc_n_processes(const orc_universe* u) { return u->P; }
int orc_n_stochastic(const orc_universe* u) { return u->n_inc; }
int orc_process_is_levy(const orc_universe* u, int i) { return u->procs[i].levy; }
int orc_process_name(const orc_universe* u, int i, char* buf, size_t n) {
    if (i < 0 || i >= u->P) return 1;
    snprintf(buf, n, "%s", u->procs[i].name);
    return 0;
}
int orc_stochastic_token(const orc_universe* u, int i, char* buf, size_t n) {
    if (i < 0 || i >= u->n_inc) return 1;
    snprintf(buf, n, "%s", u->tokens[i]);
    return 0;
}
int orc_process_index(const orc_universe* u, const char* name) {
    int idx = -1;
    for (int p = 0; p < u->P; ++p)
        if (strcmp(u->procs[p].name, name) == 0) idx = p;
    return idx;
}

/* ======================================================================
 * RNG primitives
 * ==================================================================== */

#define ROTL32(x, n) (((x) << (n)) | ((x) >> (32 - (n))))
#define QR(a, b, c, d)                                   \
    a += b; d ^= a; d = ROTL32(d, 16);                   \
    c += d; b ^= c; b = ROTL32(b, 12);                   \
    a += b; d ^= a; d = ROTL32(d, 8);                    \
    c += d; b ^= c; b = ROTL32(b, 7);

/* ChaCha block with a 64-bit block counter (words 12-13) and a 64-bit
 * stream id (words 14-15), as rand_chacha 0.9 uses it. */
void orc_chacha_block(const uint32_t key[8], uint64_t counter, uint64_t stream,
                      int rounds, uint32_t out[16]) {
    uint32_t s[16] = {0x61707865u, 0x3320646eu, 0x79622d32u, 0x6b206574u,
                      key[0], key[1], key[2], key[3], key[4], key[5], key[6], key[7],
                      (uint32_t)counter, (uint32_t)(counter >> 32),
                      (uint32_t)stream, (uint32_t)(stream >> 32)};
    uint32_t x[16];
    memcpy(x, s, sizeof x);
    for (int r = 0; r < rounds; r += 2) {
        QR(x[0], x[4], x[8], x[12]) QR(x[1], x[5], x[9], x[13])
        QR(x[2], x[6], x[10], x[14]) QR(x[3], x[7], x[11], x[15])
        QR(x[0], x[5], x[10], x[15]) QR(x[1], x[6], x[11], x[12])
        QR(x[2], x[7], x[8], x[13]) QR(x[3], x[4], x[9], x[14])
    }
    for (int i = 0; i < 16; ++i) out[i] = x[i] + s[i];
}

/* rand_core 0.9 SeedableRng::seed_from_u64: PCG32 (XSH-RR output) fills the
 * 32-byte seed four bytes at a time, advancing the state before each word. */
void orc_seed_from_u64(uint64_t state, uint32_t key[8]) {
    const uint64_t MUL = 6364136223846793005ull;
    const uint64_t INC = 11634580027462260723ull;
    for (int i = 0; i < 8; ++i) {
        state = state * MUL + INC;
        uint32_t xorshifted = (uint32_t)(((state >> 18) ^ state) >> 27);
        uint32_t rot = (uint32_t)(state >> 59);
        key[i] = (xorshifted >> rot) | (xorshifted << ((32 - rot) & 31));
    }
}

typedef struct {
    uint32_t key[8];
    uint64_t block;     /* next block to generate */
    uint32_t buf[16];
    int pos;            /* next word in buf; 16 = empty */
} chacha_stream;

static void cs_init(chacha_stream* c, uint64_t seed) {
    orc_seed_from_u64(seed, c->key);
    c->block = 0;
    c->pos = 16;
}

/* BlockRng::next_u64: two consecutive words, low word first.  Reads start
 * at word 0 and always take pairs, so a pair never straddles a block. */
static uint64_t cs_next_u64(chacha_stream* c) {
    if (c->pos >= 16) {
        orc_chacha_block(c->key, c->block++, 0, 8, c->buf);
        c->pos = 0;
    }
    uint64_t lo = c->buf[c->pos], hi = c->buf[c->pos + 1];
    c->pos += 2;
    return lo | (hi << 32);
}

/* rand's StandardUniform for f64: 53 high bits times 2^-53. */
double orc_u64_to_f64(uint64_t x) { return (double)(x >> 11) * (1.0 / 9007199254740992.0); }

void orc_chacha8_u64(uint64_t seed, uint64_t first, uint64_t n, uint64_t* out) {
    chacha_stream c;
    cs_init(&c, seed);
    c.block = first / 8;
    c.pos = 16;
    uint64_t skip = first % 8;
    for (uint64_t i = 0; i < skip; ++i) cs_next_u64(&c);
    for (uint64_t i = 0; i < n; ++i) out[i] = cs_next_u64(&c);
}

/* XOR scramble masks (an extension; the reference only has the random
 * shift): replicate r, dimension d -> high word of u64 number d of
 * ChaCha8Rng::seed_from_u64(seed + r). */
uint32_t orc_xor_mask(uint64_t seed, int replicate, int dim) {
    uint64_t v;
    orc_chacha8_u64(seed + (uint64_t)replicate, (uint64_t)dim, 1, &v);
    return (uint32_t)(v >> 32);
}

/* ======================================================================
 * Sobol -- Joe-Kuo D6 direction numbers, Gray-code order
 * (the sobol 1.0.2 crate, called from src/rng/sobol.rs:15-21)
 * ==================================================================== */

int orc_sobol_directions(const int64_t* poly, const int64_t* vinit, int dims, uint32_t* V) {
    for (int d = 0; d < dims; ++d) {
        uint32_t* v = V + (size_t)d * 32;
        if (d == 0) {
            for (int k = 0; k < 32; ++k) v[k] = 1u << (31 - k);
            continue;
        }
        int64_t p = poly[d];
        int s = 0;
        while ((p >> (s + 1)) != 0) s++;
        if (s < 1 || s > 18) return 1;
        uint64_t m[33];
        for (int k = 1; k <= s && k <= 32; ++k) m[k] = (uint64_t)vinit[(size_t)d * 18 + (k - 1)];
        for (int k = s + 1; k <= 32; ++k) {
            uint64_t x = m[k - s] ^ (m[k - s] << s);
            for (int i = 1; i < s; ++i)
                if ((p >> (s - i)) & 1) x ^= m[k - i] << i;
            m[k] = x;
        }
        for (int k = 1; k <= 32; ++k) v[k - 1] = (uint32_t)(m[k] << (32 - k));
    }
    return 0;
}

static uint32_t sobol_point(const uint32_t* V, int d, uint64_t n) {
    uint64_t g = n ^ (n >> 1);
    uint32_t x = 0;
    const uint32_t* v = V + (size_t)d * 32;
    for (int b = 0; g; ++b, g >>= 1)
        if (g & 1) x ^= v[b];
    return x;
}

void orc_sobol_points(const uint32_t* V, int dims, uint64_t first, uint64_t n, uint32_t* out) {
    for (uint64_t i = 0; i < n; ++i)
        for (int d = 0; d < dims; ++d) out[i * dims + d] = sobol_point(V, d, first + i);
}

/* ======================================================================
 * Inverse CDFs -- src/proc/increment.rs:161-200
 * ==================================================================== */

double orc_icdf_as26(double p) {
    double t = p < 0.5 ? sqrt(-2.0 * log(p)) : sqrt(-2.0 * log(1.0 - p));
    const double c0 = 2.515517, c1 = 0.802853, c2 = 0.010328;
    const double d1 = 1.432788, d2 = 0.189269, d3 = 0.001308;
    double x = t - ((c2 * t + c1) * t + c0) / (((d3 * t + d2) * t + d1) * t + 1.0);
    return p < 0.5 ? -x : x;
}

/* The "accurate" option (not in the reference): AS 26.2.23 refined by two
 * Halley steps on Phi(z) - p, the residual formed from the tail probability
 * through erfc.  Same algorithm as the engine's FP64 kernels. */
double orc_icdf_accurate(double p) {
    double z = orc_icdf_as26(p);
    int lower = p < 0.5;
    double tail = lower ? p : 1.0 - p;
    for (int it = 0; it < 2; ++it) {
        double ft = 0.5 * erfc((lower ? -z : z) * 0.70710678118654752);
        double r = lower ? ft - tail : tail - ft;
        double u = r * 2.5066282746310002 * exp(0.5 * z * z);
        z = z - u / (1.0 + 0.5 * z * u);
    }
    return z;
}

uint64_t orc_poisson(double u, double lambda) {
    if (lambda <= 0.0) return 0;
    double p = exp(-lambda);
    double f = p;
    uint64_t k = 0;
    while (u > f && k < 200) {
        k += 1;
        p *= lambda / (double)k;
        f += p;
    }
    return k;
}

/* ======================================================================
 * One scenario: filtration (src/filtration.rs:12-79), RNG
 * (src/rng/pseudo.rs, src/rng/sobol.rs), schemes (src/sim/euler.rs,
 * src/sim/runge_kutta.rs)
 * ==================================================================== */

typedef struct {
    const orc_universe* u;
    const orc_cfg* cfg;
    const double* times;
    int T, P, nslots;
    int times_strict;
    double* dts;
    double* sqrt_dts;
    double* raw;         /* [T][P] */
    double cache_time;
    double* slots;       /* name->value cache */
    /* pseudo */
    chacha_stream cs;
    int64_t cached_tidx;
    double* step_vals;
    /* sobol */
    double* sobol_vals;  /* [(T-1)*n_inc] */
    orc_jump* trace;     /* optional record of every Poisson draw */
    int trace_max, trace_n;
    int err;
    char* errbuf;
    size_t errlen;
} scen_t;

/* get_time_idx (src/filtration.rs:66-68): HashMap built from enumerate, so
 * the last index of a repeated time wins; a missing time maps to 0. */
static int time_index(const scen_t* s, double t) {
    if (s->times_strict) {
        int lo = 0, hi = s->T - 1;
        while (lo <= hi) {
            int mid = (lo + hi) / 2;
            if (s->times[mid] == t) return mid;
            if (s->times[mid] < t) lo = mid + 1; else hi = mid - 1;
        }
        return 0;
    }
    for (int i = s->T - 1; i >= 0; --i)
        if (s->times[i] == t) return i;
    return 0;
}

/* refresh_cache (src/filtration.rs:70-79) */
static void refresh_cache(scen_t* s, double t) {
    s->cache_time = t;
    s->slots[0] = t;
    int ti = time_index(s, t);
    for (int p = 0; p < s->P; ++p) s->slots[1 + p] = s->raw[(size_t)ti * s->P + p];
}

/* Function::eval (src/func.rs:32-42) */
static double feval(scen_t* s, const enode* e, double t) {
    if (t != s->cache_time) refresh_cache(s, t);
    return ev(e, s->slots);
}

/* BaseRng::sample (src/rng/pseudo.rs:35-59, src/rng/sobol.rs:57-59) */
static double rng_sample(scen_t* s, int tidx, int idx) {
    int n_inc = s->u->n_inc;
    if (s->cfg->rng == ORC_PSEUDO) {
        if (s->cached_tidx != tidx) {
            for (int i = 0; i < n_inc; ++i) s->step_vals[i] = orc_u64_to_f64(cs_next_u64(&s->cs));
            s->cached_tidx = tidx;
        }
        if (idx >= n_inc) {
            if (!s->err) set_err(s->errbuf, s->errlen, "RNG Index %d out of bounds (max %d)", idx, n_inc);
            s->err = 1;
            return 0.0;
        }
        return s->step_vals[idx];
    }
    size_t k = (size_t)tidx * n_inc + idx;
    if (idx >= n_inc || tidx >= s->T - 1) {
        if (!s->err) set_err(s->errbuf, s->errlen, "Sobol index %zu out of bounds", k);
        s->err = 1;
        return 0.0;
    }
    return s->sobol_vals[k];
}

/* Incrementor::sample (src/proc/increment.rs:46-148) */
/* Records one Poisson draw when the caller asked for a trace. */
static uint64_t traced_poisson(scen_t* s, int tidx, int idx, double uu, double lam) {
    uint64_t k = orc_poisson(uu, lam);
    if (s->trace && s->trace_n < s->trace_max) {
        orc_jump* r = &s->trace[s->trace_n++];
        r->t = tidx;
        r->idx = idx;
        r->u = uu;
        r->lam = lam;
        r->k = k;
    }
    return k;
}

static double inc_sample(scen_t* s, const inc_t* inc, int tidx) {
    switch (inc->kind) {
    case INC_DT: return s->dts[tidx];
    case INC_DW: {
        double q = rng_sample(s, tidx, inc->idx);
        return s->sqrt_dts[tidx] * (s->cfg->icdf ? orc_icdf_accurate(q) : orc_icdf_as26(q));
    }
    default: {
        double uu = rng_sample(s, tidx, inc->idx);
        double lam = feval(s, inc->lambda, s->times[tidx]) * s->dts[tidx];
        return (double)traced_poisson(s, tidx, inc->idx, uu, lam);
    }
    }
}

/* euler_iteration (src/sim/euler.rs:5-37) */
static void euler_step(scen_t* s, int t) {
    const orc_universe* u = s->u;
    double tc = s->times[t], tn = s->times[t + 1];
    for (int li = 0; li < u->nlevy; ++li) {
        int p = u->levy_idx[li];
        const proc_t* q = &u->procs[p];
        double val = s->raw[(size_t)t * s->P + p];
        for (int j = 0; j < q->nterms; ++j) {
            double c = feval(s, q->coef[j], tc);
            double x = inc_sample(s, &q->inc[j], t);
            val += c * x;
        }
        s->raw[(size_t)(t + 1) * s->P + p] = val;
    }
    for (int ai = 0; ai < u->nalg; ++ai) {
        int p = u->alg_idx[ai];
        double val = feval(s, u->procs[p].alg, tn);
        s->raw[(size_t)(t + 1) * s->P + p] = val;
    }
}

/* runge_kutta_iteration (src/sim/runge_kutta.rs:5-107), including the sign
 * variable taken from stochastic index 0 and the stale name->value cache. */
static void rk_step(scen_t* s, int t, double* incs, double* xt, double* k1, double* k2) {
    const orc_universe* u = s->u;
    int P = s->P;
    double tc = s->times[t], tn = s->times[t + 1];
    double dt = tn - tc;
    double sqrt_dt = sqrt(dt);
    double sk = rng_sample(s, t, 0) > 0.5 ? 1.0 : -1.0;
    /* pre-sample, process by process, term by term */
    size_t off = 0;
    for (int p = 0; p < P; ++p) {
        const proc_t* q = &u->procs[p];
        if (!q->levy) continue;
        for (int j = 0; j < q->nterms; ++j) incs[off + j] = inc_sample(s, &q->inc[j], t);
        off += q->nterms;
    }
    for (int p = 0; p < P; ++p) xt[p] = s->raw[(size_t)t * P + p];
    off = 0;
    for (int p = 0; p < P; ++p) {
        k1[p] = 0.0;
        const proc_t* q = &u->procs[p];
        if (!q->levy) continue;
        for (int j = 0; j < q->nterms; ++j) k1[p] += feval(s, q->coef[j], tc) * incs[off + j];
        off += q->nterms;
    }
    for (int p = 0; p < P; ++p) {
        const proc_t* q = &u->procs[p];
        if (!q->levy) continue;
        double pert = 0.0;
        for (int j = 0; j < q->nterms; ++j)
            if (q->inc[j].kind == INC_DW) pert += feval(s, q->coef[j], tc) * sk * sqrt_dt;
        s->raw[(size_t)(t + 1) * P + p] = xt[p] + k1[p] + pert;
    }
    off = 0;
    for (int p = 0; p < P; ++p) {
        k2[p] = 0.0;
        const proc_t* q = &u->procs[p];
        if (!q->levy) continue;
        for (int j = 0; j < q->nterms; ++j) k2[p] += feval(s, q->coef[j], tn) * incs[off + j];
        off += q->nterms;
    }
    for (int li = 0; li < u->nlevy; ++li) {
        int p = u->levy_idx[li];
        s->raw[(size_t)(t + 1) * P + p] = xt[p] + 0.5 * (k1[p] + k2[p]);
    }
    for (int ai = 0; ai < u->nalg; ++ai) {
        int p = u->alg_idx[ai];
        double val = feval(s, u->procs[p].alg, tn);
        s->raw[(size_t)(t + 1) * P + p] = val;
    }
}

/* "textbook" semantics (an extension): every evaluation sees the state it
 * names.  Coefficients of step t see row t; algebraic processes at t+1 see
 * the new Levy values and the algebraic values already updated at t+1. */
static void fill_slots(scen_t* s, double t, const double* row) {
    s->slots[0] = t;
    for (int p = 0; p < s->P; ++p) s->slots[1 + p] = row[p];
}

static void settle_algebraic_textbook(scen_t* s, int t) {
    const orc_universe* u = s->u;
    double* row = s->raw + (size_t)(t + 1) * s->P;
    const double* prev = s->raw + (size_t)t * s->P;
    for (int ai = 0; ai < u->nalg; ++ai) row[u->alg_idx[ai]] = prev[u->alg_idx[ai]];
    for (int ai = 0; ai < u->nalg; ++ai) {
        int p = u->alg_idx[ai];
        fill_slots(s, s->times[t + 1], row);
        row[p] = ev(u->procs[p].alg, s->slots);
    }
}

static double inc_sample_tb(scen_t* s, const inc_t* inc, int t, const double* row) {
    if (inc->kind != INC_DN) return inc_sample(s, inc, t);
    double uu = rng_sample(s, t, inc->idx);
    fill_slots(s, s->times[t], row);
    double lam = ev(inc->lambda, s->slots) * s->dts[t];
    return (double)traced_poisson(s, t, inc->idx, uu, lam);
}

static void euler_step_tb(scen_t* s, int t) {
    const orc_universe* u = s->u;
    const double* row = s->raw + (size_t)t * s->P;
    for (int li = 0; li < u->nlevy; ++li) {
        int p = u->levy_idx[li];
        const proc_t* q = &u->procs[p];
        double val = row[p];
        for (int j = 0; j < q->nterms; ++j) {
            fill_slots(s, s->times[t], row);
            double c = ev(q->coef[j], s->slots);
            double x = inc_sample_tb(s, &q->inc[j], t, row);
            val += c * x;
        }
        s->raw[(size_t)(t + 1) * s->P + p] = val;
    }
    settle_algebraic_textbook(s, t);
}

static void rk_step_tb(scen_t* s, int t, double* incs, double* probe, double* k1, double* k2) {
    const orc_universe* u = s->u;
    int P = s->P;
    const double* row = s->raw + (size_t)t * P;
    double tc = s->times[t], tn = s->times[t + 1];
    double sqrt_dt = sqrt(tn - tc);
    double sk = rng_sample(s, t, 0) > 0.5 ? 1.0 : -1.0;
    size_t off = 0;
    for (int p = 0; p < P; ++p) {
        const proc_t* q = &u->procs[p];
        if (!q->levy) continue;
        for (int j = 0; j < q->nterms; ++j) incs[off + j] = inc_sample_tb(s, &q->inc[j], t, row);
        off += q->nterms;
    }
    fill_slots(s, tc, row);
    off = 0;
    for (int p = 0; p < P; ++p) {
        const proc_t* q = &u->procs[p];
        k1[p] = 0.0;
        probe[p] = row[p];
        if (!q->levy) continue;
        double pert = 0.0;
        for (int j = 0; j < q->nterms; ++j) {
            double c = ev(q->coef[j], s->slots);
            k1[p] += c * incs[off + j];
            if (q->inc[j].kind == INC_DW) pert += c * sk * sqrt_dt;
        }
        probe[p] = row[p] + k1[p] + pert;
        off += q->nterms;
    }
    fill_slots(s, tn, probe);
    off = 0;
    for (int p = 0; p < P; ++p) {
        const proc_t* q = &u->procs[p];
        k2[p] = 0.0;
        if (!q->levy) continue;
        for (int j = 0; j < q->nterms; ++j) k2[p] += ev(q->coef[j], s->slots) * incs[off + j];
        off += q->nterms;
    }
    for (int li = 0; li < u->nlevy; ++li) {
        int p = u->levy_idx[li];
        s->raw[(size_t)(t + 1) * P + p] = row[p] + 0.5 * (k1[p] + k2[p]);
    }
    settle_algebraic_textbook(s, t);
}

typedef struct {
    const orc_universe* u;
    const double* times;
    int T;
    const double* x0;
    const orc_cfg* cfg;
    uint64_t begin, end;
    double* out_full;
    double* out_terminal;
    uint64_t out_base;
    const enode* payoff;
    double sum, sumc, sq, sqc;
    orc_jump* trace;
    int trace_max, trace_n;
    int err;
    char errbuf[256];
} job_t;

static void neumaier(double* sum, double* comp, double x) {
    double t = *sum + x;
    if (fabs(*sum) >= fabs(x)) *comp += (*sum - t) + x;
    else *comp += (x - t) + *sum;
    *sum = t;
}

static void* run_job(void* arg) {
    job_t* J = (job_t*)arg;
    const orc_universe* u = J->u;
    const orc_cfg* cfg = J->cfg;
    int T = J->T, P = u->P;
    scen_t s;
    memset(&s, 0, sizeof s);
    s.u = u;
    s.cfg = cfg;
    s.times = J->times;
    s.T = T;
    s.P = P;
    s.nslots = 1 + P + u->n_params;
    s.errbuf = J->errbuf;
    s.errlen = sizeof J->errbuf;
    s.trace = J->trace;
    s.trace_max = J->trace_max;
    s.trace_n = 0;
    s.times_strict = 1;
    for (int i = 1; i < T; ++i)
        if (!(J->times[i] > J->times[i - 1])) s.times_strict = 0;
    s.dts = (double*)calloc(T > 1 ? T - 1 : 1, sizeof(double));
    s.sqrt_dts = (double*)calloc(T > 1 ? T - 1 : 1, sizeof(double));
    for (int i = 0; i + 1 < T; ++i) {
        s.dts[i] = J->times[i + 1] - J->times[i];
        s.sqrt_dts[i] = sqrt(J->times[i + 1] - J->times[i]);
    }
    s.raw = (double*)malloc(sizeof(double) * (size_t)T * (P > 0 ? P : 1));
    s.slots = (double*)calloc(s.nslots, sizeof(double));
    for (int k = 0; k < u->n_params; ++k) s.slots[1 + P + k] = u->param_vals[k];
    s.step_vals = (double*)calloc(u->n_inc > 0 ? u->n_inc : 1, sizeof(double));
    size_t ndims = (size_t)(T - 1) * u->n_inc;
    s.sobol_vals = (double*)calloc(ndims > 0 ? ndims : 1, sizeof(double));
    int nterms_total = 0;
    for (int p = 0; p < P; ++p) nterms_total += u->procs[p].nterms;
    double* incs = (double*)calloc(nterms_total > 0 ? nterms_total : 1, sizeof(double));
    double* va = (double*)calloc(P > 0 ? P : 1, sizeof(double));
    double* vb = (double*)calloc(P > 0 ? P : 1, sizeof(double));
    double* vc = (double*)calloc(P > 0 ? P : 1, sizeof(double));
    double* prow = (double*)calloc(s.nslots, sizeof(double));
    uint32_t* masks = (uint32_t*)calloc(ndims > 0 ? ndims : 1, sizeof(uint32_t));
    uint64_t mask_rep = UINT64_MAX;

    for (uint64_t sc = J->begin; sc < J->end && !s.err; ++sc) {
        /* ScenarioFiltration::new (src/filtration.rs:22-53) */
        memset(s.raw, 0, sizeof(double) * (size_t)T * P);
        for (int p = 0; p < P; ++p) s.raw[p] = J->x0[p];
        refresh_cache(&s, J->times[0]);
        /* RNG per scenario (src/sim/mod.rs:54-66) */
        cs_init(&s.cs, cfg->seed + sc);
        s.cached_tidx = -1;
        if (cfg->rng == ORC_SOBOL) {
            if ((int)ndims > cfg->sobol_dims) {
                set_err(J->errbuf, sizeof J->errbuf, "Sobol needs %zu dimensions, table has %d", ndims, cfg->sobol_dims);
                s.err = 1;
                break;
            }
            if (cfg->scramble == ORC_SCRAMBLE_SHIFT) {
                /* point s+5 (serial order of the shared .skip(5) iterator),
                 * shifted by ChaCha8(seed+s) doubles modulo 1
                 * (src/rng/sobol.rs:35-53, 62-79) */
                for (size_t d = 0; d < ndims; ++d) {
                    double x = (double)sobol_point(cfg->sobol_v, (int)d, sc + 5) * (1.0 / 4294967296.0);
                    double sh = orc_u64_to_f64(cs_next_u64(&s.cs));
                    double v = x + sh;
                    s.sobol_vals[d] = v - trunc(v);
                }
            } else {
                /* XOR masks of replicate r (high words of ChaCha8(seed + r)),
                 * made once per replicate and thread */
                uint64_t N = cfg->n_paths_per_replicate ? cfg->n_paths_per_replicate : 1;
                uint64_t r = sc / N, n = sc % N;
                if (r != mask_rep) {
                    chacha_stream ms;
                    cs_init(&ms, cfg->seed + r);
                    for (size_t d = 0; d < ndims; ++d) masks[d] = (uint32_t)(cs_next_u64(&ms) >> 32);
                    mask_rep = r;
                }
                for (size_t d = 0; d < ndims; ++d) {
                    uint32_t y = sobol_point(cfg->sobol_v, (int)d, n) ^ masks[d];
                    s.sobol_vals[d] = ((double)y + 0.5) * (1.0 / 4294967296.0);
                }
            }
        }
        for (int t = 0; t + 1 < T && !s.err; ++t) {
            if (cfg->semantics == ORC_SEM_REFERENCE) {
                if (cfg->scheme == ORC_EULER) euler_step(&s, t);
                else rk_step(&s, t, incs, va, vb, vc);
            } else {
                if (cfg->scheme == ORC_EULER) euler_step_tb(&s, t);
                else rk_step_tb(&s, t, incs, va, vb, vc);
            }
        }
        if (s.err) break;
        uint64_t o = sc - J->out_base;
        if (J->out_full) memcpy(J->out_full + o * (size_t)T * P, s.raw, sizeof(double) * (size_t)T * P);
        if (J->out_terminal) memcpy(J->out_terminal + o * P, s.raw + (size_t)(T - 1) * P, sizeof(double) * P);
        if (J->payoff) {
            prow[0] = J->times[T - 1];
            for (int p = 0; p < P; ++p) prow[1 + p] = s.raw[(size_t)(T - 1) * P + p];
            for (int k = 0; k < u->n_params; ++k) prow[1 + P + k] = u->param_vals[k];
            double f = ev(J->payoff, prow);
            neumaier(&J->sum, &J->sumc, f);
            neumaier(&J->sq, &J->sqc, f * f);
        }
    }
    J->err = s.err;
    J->trace_n = s.trace_n;
    free(s.dts); free(s.sqrt_dts); free(s.raw); free(s.slots); free(s.step_vals);
    free(s.sobol_vals); free(incs); free(va); free(vb); free(vc); free(prow); free(masks);
    return NULL;
}

static int run_jobs(const orc_universe* u, const double* times, int n_times, const double* x0,
                    uint64_t begin, uint64_t end, const orc_cfg* cfg, double* out_full,
                    double* out_terminal, const enode* payoff, int n_threads,
                    double* sum, double* sumsq, char* err, size_t errlen) {
    if (n_times < 1) { set_err(err, errlen, "need at least one time point"); return 2; }
    if (cfg->scheme != ORC_EULER && cfg->scheme != ORC_RK) { set_err(err, errlen, "unknown scheme"); return 2; }
    if (cfg->scheme == ORC_RK && u->n_inc == 0 && n_times > 1) {
        set_err(err, errlen, "RNG Index 0 out of bounds (max 0)");
        return 6;
    }
    if (n_threads < 1) n_threads = 1;
    uint64_t n = end > begin ? end - begin : 0;
    if ((uint64_t)n_threads > n) n_threads = n > 0 ? (int)n : 1;
    job_t* jobs = (job_t*)calloc(n_threads, sizeof(job_t));
    pthread_t* th = (pthread_t*)calloc(n_threads, sizeof(pthread_t));
    for (int i = 0; i < n_threads; ++i) {
        job_t* J = &jobs[i];
        J->u = u; J->times = times; J->T = n_times; J->x0 = x0; J->cfg = cfg;
        J->begin = begin + n * i / n_threads;
        J->end = begin + n * (i + 1) / n_threads;
        J->out_full = out_full; J->out_terminal = out_terminal; J->out_base = begin;
        J->payoff = payoff;
    }
    if (n_threads == 1) run_job(&jobs[0]);
    else {
        for (int i = 0; i < n_threads; ++i) pthread_create(&th[i], NULL, run_job, &jobs[i]);
        for (int i = 0; i < n_threads; ++i) pthread_join(th[i], NULL);
    }
    int rc = 0;
    double s = 0, sc = 0, q = 0, qc = 0;
    for (int i = 0; i < n_threads; ++i) {
        if (jobs[i].err && !rc) { rc = 6; set_err(err, errlen, "%s", jobs[i].errbuf); }
        neumaier(&s, &sc, jobs[i].sum); neumaier(&s, &sc, jobs[i].sumc);
        neumaier(&q, &qc, jobs[i].sq); neumaier(&q, &qc, jobs[i].sqc);
    }
    if (sum) *sum = s + sc;
    if (sumsq) *sumsq = q + qc;
    free(jobs);
    free(th);
    return rc;
}

int orc_simulate(const orc_universe* u, const double* times, int n_times, const double* x0,
                 uint64_t path_begin, uint64_t path_end, const orc_cfg* cfg, double* out_full,
                 double* out_terminal, int n_threads, char* err, size_t errlen) {
    return run_jobs(u, times, n_times, x0, path_begin, path_end, cfg, out_full, out_terminal,
                    NULL, n_threads, NULL, NULL, err, errlen);
}

int orc_estimate(const orc_universe* u, const double* times, int n_times, const double* x0,
                 uint64_t path_begin, uint64_t path_end, const orc_cfg* cfg, const char* payoff,
                 int n_threads, double* sum, double* sumsq, char* err, size_t errlen) {
    enode* e = parse_expr(payoff, strlen(payoff), err, errlen);
    if (!e) return 1;
    if (resolve(u, e, err, errlen)) { enode_free(e); return 1; }
    int rc = run_jobs(u, times, n_times, x0, path_begin, path_end, cfg, NULL, NULL, e,
                      n_threads, sum, sumsq, err, errlen);
    enode_free(e);
    return rc;
}

int orc_eval_payoff(const orc_universe* u, const char* expr, double t, const double* rows,
                    int64_t n, double* out, char* err, size_t errlen) {
    enode* e = parse_expr(expr, strlen(expr), err, errlen);
    if (!e) return 1;
    if (resolve(u, e, err, errlen)) { enode_free(e); return 1; }
    int P = u->P;
    double* slots = (double*)calloc(1 + P + u->n_params, sizeof(double));
    for (int k = 0; k < u->n_params; ++k) slots[1 + P + k] = u->param_vals[k];
    slots[0] = t;
    for (int64_t i = 0; i < n; ++i) {
        for (int p = 0; p < P; ++p) slots[1 + p] = rows[i * P + p];
        out[i] = ev(e, slots);
    }
    free(slots);
    enode_free(e);
    return 0;
}

/* Every Poisson draw of one scenario (its step, stochastic index, uniform,
 * lambda * dt and count), in draw order: the record that tells whether a
 * jump count differing from another implementation's sits on a CDF
 * boundary.  Test infrastructure only. */
int orc_jump_trace(const orc_universe* u, const double* times, int n_times, const double* x0,
                   uint64_t scenario, const orc_cfg* cfg, orc_jump* out, int max_out, int* n_out,
                   char* err, size_t errlen) {
    if (n_times < 1) { set_err(err, errlen, "need at least one time point"); return 2; }
    if (cfg->scheme == ORC_RK && u->n_inc == 0 && n_times > 1) {
        set_err(err, errlen, "RNG Index 0 out of bounds (max 0)");
        return 6;
    }
    job_t J;
    memset(&J, 0, sizeof J);
    J.u = u; J.times = times; J.T = n_times; J.x0 = x0; J.cfg = cfg;
    J.begin = scenario; J.end = scenario + 1; J.out_base = scenario;
    J.trace = out; J.trace_max = max_out;
    run_job(&J);
    if (J.err) { set_err(err, errlen, "%s", J.errbuf); return 6; }
    *n_out = J.trace_n;
    return 0;
}
