// codegen.cpp -- lowers a process universe to one CUDA kernel per plan.
//
// One thread owns one path for the whole time loop (src/sim/mod.rs:41-87 is
// the reference's loop over scenarios and steps).  Every coefficient is an
// inline expression, so the step loop interprets nothing.  The step body
// follows euler_iteration (src/sim/euler.rs:5-37) or runge_kutta_iteration
// (src/sim/runge_kutta.rs:5-107) including the reference's name->value cache
// (src/func.rs:32-42, src/filtration.rs:70-79), which the lowered code keeps
// in registers C<p> and refreshes exactly where the reference refreshes it.
#include "codegen.h"

#include <cmath>
#include <cstdio>
#include <functional>
#include <numeric>
#include <sstream>

namespace sde {

namespace {

std::string lit(double v, bool f32) {
    char buf[64];
    if (std::isnan(v)) return f32 ? "__int_as_float(0x7fffffff)" : "__longlong_as_double(0x7ff8000000000000ll)";
    if (std::isinf(v)) {
        if (f32) return v > 0 ? "__int_as_float(0x7f800000)" : "__int_as_float(0xff800000)";
        return v > 0 ? "__longlong_as_double(0x7ff0000000000000ll)" : "__longlong_as_double(0xfff0000000000000ll)";
    }
    if (f32) std::snprintf(buf, sizeof buf, "%af", (double)(float)v);
    else std::snprintf(buf, sizeof buf, "%a", v);
    std::string s(buf);
    if (s[0] == '-') return "(" + s + ")";
    return s;
}

using VarFn = std::function<std::string(VarKind, int)>;

std::string emit(const ExprP& e, bool f32, const VarFn& var) {
    auto A = [&](int i) { return emit(e->args[i], f32, var); };
    switch (e->op) {
    case Op::Const: return lit(e->value, f32);
    case Op::Var: return var(e->vk, e->idx);
    case Op::Neg: return "(-" + A(0) + ")";
    case Op::Not: return "sde_not(" + A(0) + ")";
    case Op::Add: return "(" + A(0) + " + " + A(1) + ")";
    case Op::Sub: return "(" + A(0) + " - " + A(1) + ")";
    case Op::Mul: return "(" + A(0) + " * " + A(1) + ")";
    case Op::Div: return "(" + A(0) + " / " + A(1) + ")";
    case Op::Mod: return "fmod(" + A(0) + ", " + A(1) + ")";
    case Op::Pow: {
        // x^0.5 is lowered to sqrt (equal to a correctly rounded pow for
        // every x >= 0), x^2 to x*x and x^1 to x.
        const ExprP& b = e->args[1];
        if (b->op == Op::Const && b->value == 0.5) return "sqrt(" + A(0) + ")";
        if (b->op == Op::Const && b->value == 2.0) return "sde_sq(" + A(0) + ")";
        if (b->op == Op::Const && b->value == 1.0) return A(0);
        if (b->op == Op::Const && b->value == -0.5) return "sde_rsqrt(" + A(0) + ")";
        if (b->op == Op::Const && b->value == -1.0) return "(" + lit(1.0, f32) + " / " + A(0) + ")";
        return "pow(" + A(0) + ", " + A(1) + ")";
    }
    case Op::Eq: return "sde_eq(" + A(0) + ", " + A(1) + ")";
    case Op::Ne: return "sde_ne(" + A(0) + ", " + A(1) + ")";
    case Op::Lt: return "sde_lt(" + A(0) + ", " + A(1) + ")";
    case Op::Le: return "sde_le(" + A(0) + ", " + A(1) + ")";
    case Op::Gt: return "sde_gt(" + A(0) + ", " + A(1) + ")";
    case Op::Ge: return "sde_ge(" + A(0) + ", " + A(1) + ")";
    case Op::And: return "sde_and(" + A(0) + ", " + A(1) + ")";
    case Op::Or: return "sde_or(" + A(0) + ", " + A(1) + ")";
    case Op::Call: break;
    }
    const size_t n = e->args.size();
    auto fn1 = [&](const char* f) { return std::string(f) + "(" + A(0) + ")"; };
    switch (e->fn) {
    case Fn::Min: case Fn::Max: {
        std::string m = A(0);
        for (size_t i = 1; i < n; ++i)
            m = std::string(e->fn == Fn::Min ? "fmin(" : "fmax(") + m + ", " + A((int)i) + ")";
        return m;
    }
    case Fn::Abs: return fn1("fabs");
    case Fn::Sign: return fn1("sde_sign");
    case Fn::Int: return fn1("trunc");
    case Fn::Ceil: return fn1("ceil");
    case Fn::Floor: return fn1("floor");
    case Fn::Round: return n == 1 ? fn1("round") : "sde_round2(" + A(0) + ", " + A(1) + ")";
    case Fn::Log: {
        if (n == 1) return fn1("sde_log10");
        // log(e(), x) is the natural log (used by symbolic derivatives)
        if (e->args[0]->op == Op::Call && e->args[0]->fn == Fn::E) return "log(" + A(1) + ")";
        return "sde_logb(" + A(0) + ", " + A(1) + ")";
    }
    case Fn::E: return lit(2.718281828459045, f32);
    case Fn::Pi: return lit(3.141592653589793, f32);
    case Fn::Sin: return fn1("sin");
    case Fn::Cos: return fn1("cos");
    case Fn::Tan: return fn1("tan");
    case Fn::Asin: return fn1("asin");
    case Fn::Acos: return fn1("acos");
    case Fn::Atan: return fn1("atan");
    case Fn::Sinh: return fn1("sinh");
    case Fn::Cosh: return fn1("cosh");
    case Fn::Tanh: return fn1("tanh");
    case Fn::Asinh: return fn1("asinh");
    case Fn::Acosh: return fn1("acosh");
    case Fn::Atanh: return fn1("atanh");
    case Fn::Sqrt: return fn1("sqrt");
    case Fn::Exp: return fn1("exp");
    case Fn::Step: return "sde_b(" + A(0) + " > " + lit(0.0, f32) + ", " + lit(0.0, f32) + ")";
    case Fn::Mul0: return "sde_mul0(" + A(0) + ", " + A(1) + ")";
    case Fn::Sel: return "(" + A(0) + " > " + lit(0.0, f32) + " ? " + A(1) + " : " + A(2) + ")";
    }
    return lit(NAN, f32);
}

struct Out {
    std::ostringstream s;
    int ind = 0;
    void l(const std::string& x) {
        for (int i = 0; i < ind; ++i) s << "  ";
        s << x << "\n";
    }
};

std::string S(int v) { return std::to_string(v); }

// Shared emitter state for one kernel.
struct Gen {
    const Universe& u;
    const KernelSpec& sp;
    bool f32;
    std::string R;
    int P, NI;

    Gen(const Universe& uu, const KernelSpec& s)
        : u(uu), sp(s), f32(s.precision == PREC_FP32), R(f32 ? "float" : "double"),
          P(uu.n_processes()), NI(uu.n_stochastic()) {}

    std::string L(double v) const { return lit(v, f32); }
    std::string T(const char* arr) const { return std::string("__ldg(&a.") + arr + (f32 ? "_f" : "") + "[t])"; }

    // Expression with processes read from the named register set and time
    // from the named variable.
    std::string ex(const ExprP& e, const std::string& procset, const std::string& tvar) const {
        return emit(e, f32, [&](VarKind k, int i) -> std::string {
            if (k == VarKind::Process) return procset + S(i);
            if (k == VarKind::Time) return tvar;
            if (k == VarKind::Param) return "PR" + S(i);
            return "0";
        });
    }
    // Expression with a per-process name function
    std::string exf(const ExprP& e, const std::function<std::string(int)>& proc, const std::string& tvar) const {
        return emit(e, f32, [&](VarKind k, int i) -> std::string {
            if (k == VarKind::Process) return proc(i);
            if (k == VarKind::Time) return tvar;
            if (k == VarKind::Param) return "PR" + S(i);
            return "0";
        });
    }

    int group() const {
        if (NI == 0) return 1;
        if (sp.rng == RNG_SOBOL && sp.scramble == SCRAMBLE_XOR) return 1;
        return 8 / std::gcd(NI, 8);
    }
    bool uses_chacha() const { return NI > 0 && !(sp.rng == RNG_SOBOL && sp.scramble == SCRAMBLE_XOR); }
    bool has_alg() const { return !u.alg.empty(); }

    // ---- uniforms of step t -------------------------------------------
    void uniforms(Out& o, int g, std::vector<bool>& block_done) const {
        for (int k = 0; k < NI; ++k) {
            const std::string K = S(k);
            if (uses_chacha()) {
                int pos = g * NI + k, b = pos / 8, w = (pos % 8) * 2;
                if (!block_done[b]) {
                    o.l("sde_chacha8_block(key, blk0 + " + S(b) + "ull, B" + S(b) + ");");
                    block_done[b] = true;
                }
                o.l("const sde_u64 r" + K + " = sde_pair(B" + S(b) + "[" + S(w) + "], B" + S(b) + "[" + S(w + 1) + "]);");
            }
            if (sp.rng == RNG_PSEUDO) {
                if (!f32) o.l("const double u" + K + " = sde_u64_to_f64(r" + K + ");");
                else o.l("float q" + K + "; bool up" + K + ", gt" + K + "; sde_tail_u53(r" + K + " >> 11, q" + K + ", up" + K + ", gt" + K + ");");
            } else if (sp.scramble == SCRAMBLE_SHIFT) {
                o.l("const sde_u32 x" + K + " = sde_sobol_direct(a.sobol_v, t * " + S(NI) + " + " + K + ", G);");
                if (!f32) {
                    o.l("const double v" + K + " = (double)x" + K + " * 0x1p-32 + sde_u64_to_f64(r" + K + ");");
                    o.l("const double u" + K + " = v" + K + " - trunc(v" + K + ");");
                } else {
                    o.l("float q" + K + "; bool up" + K + ", gt" + K + "; sde_tail_u53(sde_shift_u53(x" + K + ", r" + K + "), q" + K + ", up" + K + ", gt" + K + ");");
                }
            } else {
                o.l("const int d" + K + " = t * " + S(NI) + " + " + K + ";");
                o.l("if ((d" + K + " >> 5) != hchunk) { hchunk = d" + K + " >> 5; hval = sde_sobol_hi(a.sobol_vt, mask_rep, a.sobol_dims, hchunk, H, lane); }");
                o.l("const sde_u32 y" + K + " = __shfl_sync(0xffffffffu, hval, d" + K + " & 31) ^ __ldg(&a.sobol_lo[(sde_u64)d" + K + " * 32u + L]);");
                if (!f32) o.l("const double u" + K + " = ((double)y" + K + " + 0.5) * 0x1p-32;");
                else o.l("float q" + K + "; bool up" + K + ", gt" + K + "; sde_tail_xor(y" + K + ", q" + K + ", up" + K + ", gt" + K + ");");
            }
        }
    }

    // Wiener increments w<k> = sqrt_dt * icdf(u<k>)   (increment.rs:89-97)
    void wiener(Out& o) const {
        for (int k = 0; k < NI; ++k) {
            if (u.token_kind[k] != IncKind::Dw) continue;
            const std::string K = S(k);
            if (!f32) o.l("const double w" + K + " = sdt * sde_icdf_as26(u" + K + ");");
            else o.l("const float w" + K + " = sdt * sde_icdf_as26_q(q" + K + ", up" + K + ");");
        }
    }

    // Poisson increments n<k> (increment.rs:137-148); lambda read through
    // the given register set at time tvar.
    void poisson(Out& o, const std::string& procset, const std::string& tvar) const {
        for (int k = 0; k < NI; ++k) {
            if (u.token_kind[k] != IncKind::Dn) continue;
            ExprP lam;
            for (const auto& p : u.procs)
                for (const auto& t : p.terms)
                    if (t.sidx == k && t.lambda) lam = t.lambda;
            const std::string K = S(k);
            std::string pu = f32 ? "(up" + K + " ? 1.0f - q" + K + " : q" + K + ")" : "u" + K;
            o.l("const " + R + " n" + K + " = sde_poisson(" + pu + ", " + ex(lam, procset, tvar) + " * dt);");
        }
    }

    std::string inc(const Term& t) const {
        if (t.kind == IncKind::Dt) return "dt";
        if (t.kind == IncKind::Dw) return "w" + S(t.sidx);
        return "n" + S(t.sidx);
    }

    std::string sk_expr() const {
        if (!f32) return "(u0 > 0.5 ? 1.0 : -1.0)";
        return "(gt0 ? 1.0f : -1.0f)";
    }

    // ---- one step, reference semantics --------------------------------
    void step_reference(Out& o) const {
        if (sp.scheme == SCHEME_EULER) {
            // cache refresh at t when no algebraic process left it at t
            if (!has_alg())
                for (int p : u.levy) o.l("C" + S(p) + " = X" + S(p) + ";");
            poisson(o, "C", "tc");
            for (int p : u.levy) {
                o.l(R + " N" + S(p) + " = X" + S(p) + ";");
                for (const auto& t : u.procs[p].terms)
                    o.l("N" + S(p) + " = N" + S(p) + " + " + ex(t.coef, "C", "tc") + " * " + inc(t) + ";");
            }
            if (has_alg()) {
                // refresh at t+1 before any algebraic slot of t+1 is written
                for (int p : u.levy) o.l("C" + S(p) + " = N" + S(p) + ";");
                for (int q : u.alg) o.l("C" + S(q) + " = " + L(0.0) + ";");
                for (int q : u.alg) o.l(R + " N" + S(q) + " = " + ex(u.procs[q].alg, "C", "tn") + ";");
            }
        } else {
            o.l("const " + R + " sk = " + sk_expr() + ";");
            poisson(o, "C", "tc");
            for (int p : u.levy) {
                const auto& terms = u.procs[p].terms;
                for (size_t j = 0; j < terms.size(); ++j)
                    o.l("const " + R + " c" + S(p) + "_" + S((int)j) + " = " + ex(terms[j].coef, "C", "tc") + ";");
                o.l(R + " k1_" + S(p) + " = " + L(0.0) + ";");
                for (size_t j = 0; j < terms.size(); ++j)
                    o.l("k1_" + S(p) + " = k1_" + S(p) + " + c" + S(p) + "_" + S((int)j) + " * " + inc(terms[j]) + ";");
                o.l(R + " pe" + S(p) + " = " + L(0.0) + ";");
                for (size_t j = 0; j < terms.size(); ++j)
                    if (terms[j].kind == IncKind::Dw)
                        o.l("pe" + S(p) + " = pe" + S(p) + " + c" + S(p) + "_" + S((int)j) + " * sk * sdt;");
            }
            for (int p : u.levy) o.l("C" + S(p) + " = X" + S(p) + " + k1_" + S(p) + " + pe" + S(p) + ";");
            for (int q : u.alg) o.l("C" + S(q) + " = " + L(0.0) + ";");
            for (int p : u.levy) {
                const auto& terms = u.procs[p].terms;
                o.l(R + " k2_" + S(p) + " = " + L(0.0) + ";");
                for (size_t j = 0; j < terms.size(); ++j)
                    o.l("k2_" + S(p) + " = k2_" + S(p) + " + " + ex(terms[j].coef, "C", "tn") + " * " + inc(terms[j]) + ";");
                o.l(R + " N" + S(p) + " = X" + S(p) + " + " + L(0.5) + " * (k1_" + S(p) + " + k2_" + S(p) + ");");
            }
            for (int q : u.alg) o.l(R + " N" + S(q) + " = " + ex(u.procs[q].alg, "C", "tn") + ";");
        }
        for (int p = 0; p < P; ++p) o.l("X" + S(p) + " = N" + S(p) + ";");
    }

    // ---- one step, textbook semantics ---------------------------------
    void settle_alg_textbook(Out& o) const {
        if (!has_alg()) return;
        for (int q : u.alg) o.l(R + " N" + S(q) + " = X" + S(q) + ";");
        for (int q : u.alg)
            o.l("N" + S(q) + " = " + ex(u.procs[q].alg, "N", "tn") + ";");
    }
    void step_textbook(Out& o) const {
        if (sp.scheme == SCHEME_EULER) {
            poisson(o, "X", "tc");
            for (int p : u.levy) {
                o.l(R + " N" + S(p) + " = X" + S(p) + ";");
                for (const auto& t : u.procs[p].terms)
                    o.l("N" + S(p) + " = N" + S(p) + " + " + ex(t.coef, "X", "tc") + " * " + inc(t) + ";");
            }
            settle_alg_textbook(o);
        } else {
            o.l("const " + R + " sk = " + sk_expr() + ";");
            poisson(o, "X", "tc");
            for (int p : u.levy) {
                const auto& terms = u.procs[p].terms;
                o.l(R + " k1_" + S(p) + " = " + L(0.0) + ";");
                o.l(R + " pe" + S(p) + " = " + L(0.0) + ";");
                for (size_t j = 0; j < terms.size(); ++j) {
                    o.l("const " + R + " c" + S(p) + "_" + S((int)j) + " = " + ex(terms[j].coef, "X", "tc") + ";");
                    o.l("k1_" + S(p) + " = k1_" + S(p) + " + c" + S(p) + "_" + S((int)j) + " * " + inc(terms[j]) + ";");
                    if (terms[j].kind == IncKind::Dw)
                        o.l("pe" + S(p) + " = pe" + S(p) + " + c" + S(p) + "_" + S((int)j) + " * sk * sdt;");
                }
            }
            for (int p = 0; p < P; ++p) {
                if (u.procs[p].levy) o.l("const " + R + " PB" + S(p) + " = X" + S(p) + " + k1_" + S(p) + " + pe" + S(p) + ";");
                else o.l("const " + R + " PB" + S(p) + " = X" + S(p) + ";");
            }
            for (int p : u.levy) {
                const auto& terms = u.procs[p].terms;
                o.l(R + " k2_" + S(p) + " = " + L(0.0) + ";");
                for (size_t j = 0; j < terms.size(); ++j)
                    o.l("k2_" + S(p) + " = k2_" + S(p) + " + " + ex(terms[j].coef, "PB", "tn") + " * " + inc(terms[j]) + ";");
                o.l(R + " N" + S(p) + " = X" + S(p) + " + " + L(0.5) + " * (k1_" + S(p) + " + k2_" + S(p) + ");");
            }
            settle_alg_textbook(o);
        }
        for (int p = 0; p < P; ++p) o.l("X" + S(p) + " = N" + S(p) + ";");
    }

    void store(Out& o, const std::string& tidx) const {
        if (!sp.store_output) return;
        o.l("{ const int slot = __ldg(&a.out_tidx[" + tidx + "]);");
        o.l("  if (slot >= 0 && active) {");
        o.l("    " + R + "* dst = OUT + ((sde_u64)rep * a.n_out + slot) * (sde_u64)" + S(P) + " * a.n_paths + i;");
        for (int p = 0; p < P; ++p)
            o.l("    dst[(sde_u64)" + S(p) + " * a.n_paths] = X" + S(p) + ";");
        o.l("  } }");
    }

    void prologue(Out& o) const {
        o.l("const int lane = threadIdx.x & 31;");
        o.l("const sde_u64 i = (sde_u64)blockIdx.x * blockDim.x + threadIdx.x;");
        o.l("const int rep = blockIdx.y;");
        o.l("const bool active = i < a.n_paths;");
        o.l("const sde_u64 scen = a.path_base + (sde_u64)rep * a.n_paths + i;");
        o.l("const int n_steps = a.T - 1;");
        o.l("(void)lane; (void)scen;");
        for (int k = 0; k < (int)u.params.size(); ++k)
            o.l("const " + R + " PR" + S(k) + " = (" + R + ")__ldg(&a.params[" + S(k) + "]);");
        for (int p = 0; p < P; ++p) o.l(R + " X" + S(p) + " = (" + R + ")__ldg(&a.x0[" + S(p) + "]);");
        for (int p = 0; p < P; ++p) o.l(R + " C" + S(p) + " = X" + S(p) + ";");
        if (sp.store_output) o.l(R + "* OUT = (" + R + "*)a.out;");
        if (uses_chacha()) o.l("sde_u32 key[8]; sde_seed_from_u64(a.seed + scen, key);");
        if (sp.rng == RNG_SOBOL && sp.scramble == SCRAMBLE_SHIFT)
            o.l("const sde_u32 G = sde_gray((sde_u32)(scen + 5ull));");
        if (sp.rng == RNG_SOBOL && sp.scramble == SCRAMBLE_XOR) {
            o.l("const sde_u32 Gx = sde_gray((sde_u32)i);");
            o.l("const sde_u32 L = Gx & 31u, H = Gx >> 5;");
            o.l("const sde_u32* mask_rep = a.masks ? a.masks + (sde_u64)rep * a.mask_stride : nullptr;");
            o.l("int hchunk = -1; sde_u32 hval = 0u;");
        }
    }

    void time_loop(Out& o, bool textbook) const {
        const int U = group();
        const int nblocks = uses_chacha() ? (U * NI) / 8 : 0;
        o.l("for (int t0 = 0; t0 < n_steps; t0 += " + S(U) + ") {");
        o.ind++;
        if (uses_chacha()) {
            o.l("const sde_u64 blk0 = ((sde_u64)t0 * " + S(NI) + "ull) / 8ull;");
            for (int b = 0; b < nblocks; ++b) o.l("sde_u32 B" + S(b) + "[16];");
        }
        std::vector<bool> done(std::max(1, nblocks), false);
        for (int g = 0; g < U; ++g) {
            o.l("{ const int t = t0 + " + S(g) + ";");
            o.l("if (t < n_steps) {");
            o.ind++;
            o.l("const " + R + " tc = " + T("times") + ";");
            o.l("const " + R + " tn = (" + R + ")__ldg(&a.times" + std::string(f32 ? "_f" : "") + "[t + 1]);");
            o.l("const " + R + " dt = " + T("dts") + ";");
            o.l("const " + R + " sdt = " + T("sqrt_dts") + ";");
            o.l("(void)tc; (void)tn; (void)dt; (void)sdt;");
            uniforms(o, g, done);
            wiener(o);
            if (textbook) step_textbook(o);
            else step_reference(o);
            store(o, "t + 1");
            o.ind--;
            o.l("} }");
        }
        o.ind--;
        o.l("}");
    }

    void epilogue(Out& o) const {
        const int K = (int)sp.payoffs.size();
        if (K == 0) return;
        o.l("const " + R + " tT = (" + R + ")__ldg(&a.times[a.T - 1]);");
        o.l("double f[" + S(K) + "];");
        for (int k = 0; k < K; ++k)
            o.l("f[" + S(k) + "] = active ? (double)(" + ex(sp.payoffs[k], "X", "tT") + ") : 0.0;");
        o.l("sde_block_reduce_store<" + S(K) + ">(f, a.partials + (((sde_u64)rep * gridDim.x + blockIdx.x) * " + S(K) + "u) * 4u);");
    }

    // ---- adjoint ---------------------------------------------------------
    // Uniforms by random access (any step order): ChaCha blocks are cached
    // per thread, Sobol points are direct.
    void uniforms_ra(Out& o) const {
        for (int k = 0; k < NI; ++k) {
            const std::string K = S(k);
            if (uses_chacha()) {
                o.l("sde_u64 r" + K + ";");
                o.l("{ const sde_u64 pos = (sde_u64)t * " + S(NI) + "ull + " + K + "ull;");
                o.l("  if ((pos >> 3) != cblk) { cblk = pos >> 3; sde_chacha8_block(key, cblk, CB); }");
                o.l("  const int w = (int)(pos & 7ull) * 2; r" + K + " = sde_pair(CB[w], CB[w + 1]); }");
            }
            if (sp.rng == RNG_PSEUDO) {
                if (!f32) o.l("const double u" + K + " = sde_u64_to_f64(r" + K + ");");
                else o.l("float q" + K + "; bool up" + K + ", gt" + K + "; sde_tail_u53(r" + K + " >> 11, q" + K + ", up" + K + ", gt" + K + ");");
            } else if (sp.scramble == SCRAMBLE_SHIFT) {
                o.l("const sde_u32 x" + K + " = sde_sobol_direct(a.sobol_v, t * " + S(NI) + " + " + K + ", G);");
                if (!f32) {
                    o.l("const double v" + K + " = (double)x" + K + " * 0x1p-32 + sde_u64_to_f64(r" + K + ");");
                    o.l("const double u" + K + " = v" + K + " - trunc(v" + K + ");");
                } else {
                    o.l("float q" + K + "; bool up" + K + ", gt" + K + "; sde_tail_u53(sde_shift_u53(x" + K + ", r" + K + "), q" + K + ", up" + K + ", gt" + K + ");");
                }
            } else {
                o.l("const int d" + K + " = t * " + S(NI) + " + " + K + ";");
                o.l("if ((d" + K + " >> 5) != hchunk) { hchunk = d" + K + " >> 5; hval = sde_sobol_hi(a.sobol_vt, mask_rep, a.sobol_dims, hchunk, H, lane); }");
                o.l("const sde_u32 y" + K + " = __shfl_sync(0xffffffffu, hval, d" + K + " & 31) ^ __ldg(&a.sobol_lo[(sde_u64)d" + K + " * 32u + L]);");
                if (!f32) o.l("const double u" + K + " = ((double)y" + K + " + 0.5) * 0x1p-32;");
                else o.l("float q" + K + "; bool up" + K + ", gt" + K + "; sde_tail_xor(y" + K + ", q" + K + ", up" + K + ", gt" + K + ");");
            }
        }
    }

    void step_header(Out& o) const {
        o.l("const " + R + " tc = " + T("times") + ";");
        o.l("const " + R + " tn = (" + R + ")__ldg(&a.times" + std::string(f32 ? "_f" : "") + "[t + 1]);");
        o.l("const " + R + " dt = " + T("dts") + ";");
        o.l("const " + R + " sdt = " + T("sqrt_dts") + ";");
        o.l("(void)tc; (void)tn; (void)dt; (void)sdt;");
    }

    // increment k of a stochastic index as stored for the reverse sweep
    std::string inc_store_name(int k) const {
        return u.token_kind[k] == IncKind::Dw ? "w" + S(k) : "n" + S(k);
    }

    std::string adjoint(const std::string& name) const {
        // Pathwise adjoint of Euler-Maruyama: X' = X + sum_j c_j(t, X, theta) inc_j,
        // lambda_t = lambda_{t+1} + sum_p lambda_{t+1,p} sum_j dc_pj/dX inc_j,
        // g_theta += sum_p lambda_{t+1,p} sum_j dc_pj/dtheta inc_j.  Increments
        // are held fixed (common random numbers); jump counts are piecewise
        // constant in the parameters.
        const int E = sp.ckpt_every;
        const int K = (int)sp.payoffs.size();
        const int GP = (int)sp.grad_params.size(), GX = (int)sp.grad_x0.size();
        Out o;
        o.l("extern \"C\" __global__ void __launch_bounds__(" + S(sp.block) + ") " + name + "(const sde_args a) {");
        o.ind++;
        prologue(o);
        if (uses_chacha()) o.l("sde_u64 cblk = ~0ull; sde_u32 CB[16];");
        o.l(R + "* CK = (" + R + "*)a.ckpt;");
        o.l("const sde_u64 ckrow = (sde_u64)rep * a.n_ckpt;");
        // forward pass with checkpoints
        o.l("for (int t = 0; t < n_steps; ++t) {");
        o.ind++;
        o.l("if (t % " + S(E) + " == 0 && active) {");
        for (int p = 0; p < P; ++p)
            o.l("  CK[((ckrow + t / " + S(E) + ") * " + S(P) + " + " + S(p) + ") * a.n_paths + i] = X" + S(p) + ";");
        o.l("}");
        step_header(o);
        uniforms_ra(o);
        wiener(o);
        step_reference(o);
        o.ind--;
        o.l("}");
        // payoffs and the terminal adjoint of payoff 0
        o.l("const " + R + " tT = (" + R + ")__ldg(&a.times[a.T - 1]);");
        o.l("double f[" + S(K + GP + GX) + "];");
        for (int k = 0; k < K; ++k)
            o.l("f[" + S(k) + "] = active ? (double)(" + ex(sp.payoffs[k], "X", "tT") + ") : 0.0;");
        for (int p = 0; p < P; ++p)
            o.l(R + " LA" + S(p) + " = " + ex(derivative(sp.payoffs[0], VarKind::Process, p), "X", "tT") + ";");
        for (int m = 0; m < GP; ++m)
            o.l(R + " GP" + S(m) + " = " + ex(derivative(sp.payoffs[0], VarKind::Param, sp.grad_params[m]), "X", "tT") + ";");
        // reverse sweep over segments, recomputing each from its checkpoint
        o.l(R + " LX[" + S(E * std::max(1, P)) + "];");
        o.l(R + " LI[" + S(E * std::max(1, NI)) + "];");
        o.l("const int nseg = (n_steps + " + S(E - 1) + ") / " + S(E) + ";");
        o.l("for (int seg = nseg - 1; seg >= 0; --seg) {");
        o.ind++;
        o.l("const int s0 = seg * " + S(E) + ";");
        o.l("const int s1 = min(s0 + " + S(E) + ", n_steps);");
        for (int p = 0; p < P; ++p)
            o.l("X" + S(p) + " = active ? CK[((ckrow + seg) * " + S(P) + " + " + S(p) + ") * a.n_paths + i] : X" + S(p) + ";");
        o.l("for (int t = s0; t < s1; ++t) {");
        o.ind++;
        o.l("const int s = t - s0;");
        for (int p = 0; p < P; ++p) o.l("LX[s * " + S(P) + " + " + S(p) + "] = X" + S(p) + ";");
        step_header(o);
        uniforms_ra(o);
        wiener(o);
        // record the stochastic increments (jump counts need the cache = X)
        for (int p : u.levy) o.l("C" + S(p) + " = X" + S(p) + ";");
        poisson(o, "C", "tc");
        for (int k = 0; k < NI; ++k) o.l("LI[s * " + S(NI) + " + " + S(k) + "] = " + inc_store_name(k) + ";");
        for (int p : u.levy) {
            o.l(R + " N" + S(p) + " = X" + S(p) + ";");
            for (const auto& tm : u.procs[p].terms)
                o.l("N" + S(p) + " = N" + S(p) + " + " + ex(tm.coef, "C", "tc") + " * " + inc(tm) + ";");
        }
        for (int p : u.levy) o.l("X" + S(p) + " = N" + S(p) + ";");
        o.ind--;
        o.l("}");
        o.l("for (int t = s1 - 1; t >= s0; --t) {");
        o.ind++;
        o.l("const int s = t - s0;");
        o.l("const " + R + " tc = " + T("times") + ";");
        o.l("const " + R + " dt = " + T("dts") + ";");
        o.l("(void)tc; (void)dt;");
        for (int p = 0; p < P; ++p) o.l("const " + R + " Y" + S(p) + " = LX[s * " + S(P) + " + " + S(p) + "];");
        for (int k = 0; k < NI; ++k) o.l("const " + R + " " + inc_store_name(k) + " = LI[s * " + S(NI) + " + " + S(k) + "];");
        for (int q = 0; q < P; ++q) o.l(R + " LN" + S(q) + " = " + L(0.0) + ";");
        for (int p : u.levy) {
            const auto& terms = u.procs[p].terms;
            for (size_t j = 0; j < terms.size(); ++j) {
                const ExprP& c = terms[j].coef;
                const std::string li = "li" + S(p) + "_" + S((int)j);
                o.l("{ const " + R + " " + li + " = LA" + S(p) + " * " + inc(terms[j]) + ";");
                for (int q = 0; q < P; ++q)
                    if (depends_on(c, VarKind::Process, q))
                        o.l("  LN" + S(q) + " += " + li + " * " + ex(derivative(c, VarKind::Process, q), "Y", "tc") + ";");
                for (int m = 0; m < GP; ++m)
                    if (depends_on(c, VarKind::Param, sp.grad_params[m]))
                        o.l("  GP" + S(m) + " += " + li + " * " + ex(derivative(c, VarKind::Param, sp.grad_params[m]), "Y", "tc") + ";");
                o.l("}");
            }
        }
        for (int q = 0; q < P; ++q) o.l("LA" + S(q) + " += LN" + S(q) + ";");
        o.ind--;
        o.l("}");
        o.ind--;
        o.l("}");
        for (int m = 0; m < GP; ++m) o.l("f[" + S(K + m) + "] = active ? (double)GP" + S(m) + " : 0.0;");
        for (int x = 0; x < GX; ++x) o.l("f[" + S(K + GP + x) + "] = active ? (double)LA" + S(sp.grad_x0[x]) + " : 0.0;");
        o.l("sde_block_reduce_store<" + S(K + GP + GX) + ">(f, a.partials + (((sde_u64)rep * gridDim.x + blockIdx.x) * " + S(K + GP + GX) + "u) * 4u);");
        o.ind--;
        o.l("}");
        return o.s.str();
    }

    std::string forward(const std::string& name) const {
        Out o;
        o.l("extern \"C\" __global__ void __launch_bounds__(" + S(sp.block) + ") " + name + "(const sde_args a) {");
        o.ind++;
        prologue(o);
        store(o, "0");
        time_loop(o, sp.semantics == SEM_TEXTBOOK);
        epilogue(o);
        o.ind--;
        o.l("}");
        return o.s.str();
    }
};

}  // namespace

std::string emit_expression(const ExprP& e, bool fp32) {
    return emit(e, fp32, [](VarKind k, int i) -> std::string {
        if (k == VarKind::Process) return "X" + std::to_string(i);
        if (k == VarKind::Time) return "t";
        return "PR" + std::to_string(i);
    });
}

static std::string tag(const KernelSpec& s) {
    std::string r = s.scheme == SCHEME_RK ? "rk" : "euler";
    r += s.precision == PREC_FP32 ? "_fp32" : "_fp64";
    r += s.rng == RNG_PSEUDO ? "_pseudo" : (s.scramble == SCRAMBLE_XOR ? "_sobolxor" : "_sobolshift");
    return r;
}

std::string forward_kernel_name(const KernelSpec& s) { return "sde_step_" + tag(s); }
std::string adjoint_kernel_name(const KernelSpec& s) { return "sde_adjoint_" + tag(s); }

std::string generate_source(const Universe& u, const KernelSpec& s) {
    Gen g(u, s);
    std::string src;
    src += g.forward(forward_kernel_name(s));
    if (s.adjoint) src += "\n" + g.adjoint(adjoint_kernel_name(s));
    return src;
}

}  // namespace sde
