// codegen.cpp -- lowers a process universe to CUDA kernels.
//
// A thread owns PPT paths (lanes j = 0..PPT-1) for the whole time loop
// (src/sim/mod.rs:41-87 is the reference's loop over scenarios and steps).
// Every coefficient is an inline expression, so the step loop interprets
// nothing.  The step body follows euler_iteration (src/sim/euler.rs:5-37) or
// runge_kutta_iteration (src/sim/runge_kutta.rs:5-107), including the
// reference's name->value cache (src/func.rs:32-42, src/filtration.rs:70-79),
// which the lowered code keeps in registers C<p> and refreshes exactly where
// the reference refreshes it.
//
// Three kernels come out of the same emitters:
//   forward  -- one plan, grid over (paths / (block*PPT), replicates)
//   adjoint  -- forward with checkpoints, then a pathwise reverse sweep
//   batch    -- per-template device functions called from a persistent
//               work-queue kernel over many instances
#include "codegen.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
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
        // every x >= 0), x^2 to x*x, x^1 to x, x^-0.5 to rsqrt, x^-1 to 1/x.
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

// IEEE binary16 from binary32, round to nearest even (subnormals kept).
uint16_t f32_to_f16(float f) {
    uint32_t x;
    std::memcpy(&x, &f, 4);
    const uint16_t sign = (uint16_t)((x >> 16) & 0x8000u);
    const uint32_t ax = x & 0x7FFFFFFFu;
    if (ax >= 0x7F800000u) return sign | (ax > 0x7F800000u ? 0x7E00u : 0x7C00u);
    if (ax >= 0x477FF000u) return sign | 0x7C00u;  // 65520 and up round to infinity
    if (ax >= 0x38800000u) {                        // normal: rebias, round 23 -> 10 bits
        const uint32_t m = ax - 0x38000000u;
        return sign | (uint16_t)((m + 0xFFFu + ((m >> 13) & 1u)) >> 13);
    }
    if (ax < 0x33000000u) return sign;              // below 2^-25: zero
    const int e = (int)(ax >> 23);
    const uint32_t mant = (ax & 0x7FFFFFu) | 0x800000u;
    const int shift = 126 - e;                      // value * 2^24 = mant >> shift
    uint32_t q = mant >> shift;
    const uint32_t rem = mant & ((1u << shift) - 1u), half = 1u << (shift - 1);
    if (rem > half || (rem == half && (q & 1u))) ++q;
    return sign | (uint16_t)q;
}

float f16_to_f32(uint16_t h) {
    const int e = (h >> 10) & 0x1F, m = h & 0x3FF;
    float v;
    if (e == 0) v = std::ldexp((float)m, -24);
    else if (e == 31) v = m ? NAN : INFINITY;
    else v = std::ldexp((float)(m | 0x400), e - 25);
    return (h & 0x8000u) ? -v : v;
}

// Value of an expression that reads no variable (plain f64 arithmetic, as
// fasteval evaluates it); false if it reads one or uses an unfolded call.
bool fold_const(const ExprP& e, double& v) {
    double a = 0.0, b = 0.0;
    switch (e->op) {
    case Op::Const: v = e->value; return true;
    case Op::Var: return false;
    case Op::Neg: if (!fold_const(e->args[0], a)) return false; v = -a; return true;
    case Op::Add: case Op::Sub: case Op::Mul: case Op::Div: case Op::Pow:
        if (!fold_const(e->args[0], a) || !fold_const(e->args[1], b)) return false;
        v = e->op == Op::Add ? a + b : e->op == Op::Sub ? a - b : e->op == Op::Mul ? a * b
          : e->op == Op::Div ? a / b : std::pow(a, b);
        return true;
    case Op::Call:
        if (e->args.size() != 1 || !fold_const(e->args[0], a)) return false;
        if (e->fn == Fn::Sqrt) { v = std::sqrt(a); return true; }
        if (e->fn == Fn::Exp) { v = std::exp(a); return true; }
        if (e->fn == Fn::Abs) { v = std::fabs(a); return true; }
        return false;
    default: return false;
    }
}

// coefficient k * X_q (or X_q * k) -> (k, q)
bool split_linear_coef(const ExprP& c, ExprP& k, int& q) {
    if (c->op == Op::Var && c->vk == VarKind::Process) {
        k = mk_const(1.0);
        q = c->idx;
        return true;
    }
    if (c->op != Op::Mul) return false;
    const ExprP& a = c->args[0];
    const ExprP& b = c->args[1];
    if (b->op == Op::Var && b->vk == VarKind::Process) { k = a; q = b->idx; return true; }
    if (a->op == Op::Var && a->vk == VarKind::Process) { k = b; q = a->idx; return true; }
    return false;
}

// Constant diffusion matrix K[p][j] (process p, Wiener index j) of a
// universe whose every dW term is constant * own process; false otherwise.
bool diffusion_matrix(const Universe& u, std::vector<std::vector<double>>& K) {
    const int P = u.n_processes(), NI = u.n_stochastic();
    K.assign(P, std::vector<double>(NI, 0.0));
    bool any = false;
    for (int p = 0; p < P; ++p)
        for (const auto& t : u.procs[p].terms) {
            if (t.kind != IncKind::Dw) continue;
            ExprP k;
            int q = -1;
            double v = 0.0;
            if (!split_linear_coef(t.coef, k, q) || q != p || !fold_const(k, v)) return false;
            K[p][t.sidx] += v;
            any = true;
        }
    return any;
}

// Every term of process p but its dW terms is (constant * X_p) * dt; c gets
// the sum of those constants.
bool linear_drift_of(const Universe& u, int p, double& c) {
    c = 0.0;
    for (const auto& t : u.procs[p].terms) {
        if (t.kind == IncKind::Dw) continue;
        ExprP k;
        int q = -1;
        double v = 0.0;
        if (t.kind != IncKind::Dt || !split_linear_coef(t.coef, k, q) || q != p || !fold_const(k, v)) return false;
        c += v;
    }
    return true;
}

enum class Mode { Forward, Batch };

struct Gen {
    const Universe& u;
    const KernelSpec& sp;
    bool f32;
    std::string R;
    int P, NI;
    Mode mode = Mode::Forward;
    int ppt = 1;
    std::string sfx;  // per-lane suffix of per-path names

    Gen(const Universe& uu, const KernelSpec& s)
        : u(uu), sp(s), f32(s.precision == PREC_FP32), R(f32 ? "float" : "double"),
          P(uu.n_processes()), NI(uu.n_stochastic()), ppt(std::max(1, s.ppt)) {}

    std::string L(double v) const { return lit(v, f32); }
    // per-path (per-lane) names
    std::string V(const std::string& b, int i) const { return b + S(i) + sfx; }
    std::string V(const std::string& b) const { return b + sfx; }
    void lane(int j) { sfx = ppt > 1 ? "_" + S(j) : ""; }

    std::string T(const char* arr, const char* idx = "t") const {
        return std::string("__ldg(&a.") + arr + (f32 ? "_f" : "") + "[" + idx + "])";
    }

    // Expression with processes read from the named per-lane register set.
    std::string ex(const ExprP& e, const std::string& procset, const std::string& tvar) const {
        return emit(e, f32, [&](VarKind k, int i) -> std::string {
            if (k == VarKind::Process) return V(procset, i);
            if (k == VarKind::Time) return tvar;
            if (k == VarKind::Param) return "PR" + S(i);
            return "0";
        });
    }

    bool xorm() const { return sp.rng == RNG_SOBOL && sp.scramble == SCRAMBLE_XOR; }
    bool shiftm() const { return sp.rng == RNG_SOBOL && sp.scramble == SCRAMBLE_SHIFT; }
    // Steps per unrolled group: whole ChaCha blocks (8 u64) for the pseudo /
    // shift streams, whole 32-dimension Sobol chunks for the XOR mode, so
    // every block word and every shuffle lane is a compile-time constant.
    int group() const {
        if (NI == 0) return 1;
        if (xorm()) return 32 / std::gcd(NI, 32);
        return 8 / std::gcd(NI, 8);
    }
    // The FP32 forward CUDA-core kernel on the reference's shifted Sobol
    // points, with a power-of-two number of stochastic indices up to 32: an
    // outer loop over 32-dimension chunks (32 / NI steps) fetches the warp's
    // two high parts once per chunk, and the inner step groups (whole
    // ChaCha8 blocks, a rolled loop) find their shuffle lanes and LO words
    // at an offset eo from the chunk's start.  Other kernels check per
    // dimension whether the chunk changed.
    bool grp_shift = false;
    bool grp_shift_eligible() const {
        return shiftm() && f32 && !mma && NI > 0 && NI <= 32 && (NI & (NI - 1)) == 0;
    }
    // the FP32 XOR path goes straight from the scrambled word to a normal;
    // q / up / gt are formed only where a jump count or RK's sign needs them
    bool needs_tail(int k) const {
        return u.token_kind[k] == IncKind::Dn || (sp.scheme == SCHEME_RK && k == 0) || sp.icdf != 0;
    }
    bool uses_chacha() const { return NI > 0 && !xorm(); }
    // XOR mode: dimensions per LO load, the largest of 4, 2, 1 dividing NI
    // (a step's first dimension is then aligned to it)
    int lo_width() const { return NI % 4 == 0 ? 4 : NI % 2 == 0 ? 2 : 1; }
    // the tensor-core step reads its LO words from shared memory, where
    // thread 0 bulk-copies each step's NI * 128 bytes two steps ahead
    bool lo_tma() const { return mma && mma->lo_off > 0 && xorm() && mode == Mode::Forward; }
    // thread 0: the bulk copy of step s's LO words into buffer s & 1
    void lo_issue(Out& o, const std::string& pad, const std::string& s) const {
        const std::string B = S(mma->lo_step_bytes) + "u";
        o.l(pad + "if ((" + s + ") < a.T - 1) {");
        o.l(pad + "  const sde_u32 b_ = (sde_u32)(" + s + ") & 1u;");
        o.l(pad + "  sde_fence_async_smem();");
        o.l(pad + "  sde_mbar_arrive_expect_tx(LBAR0 + 8u * b_, " + B + ");");
        o.l(pad + "  sde_bulk_g2s(LOBA + b_ * " + B + ", a.sobol_lo + (sde_u64)(" + s + ") * " + S(NI * 32) + "ull, " + B +
            ", LBAR0 + 8u * b_);");
        o.l(pad + "  lb_issued = " + s + ";");
        o.l(pad + "}");
    }
    bool has_alg() const { return !u.alg.empty(); }

    // ---- uniforms of step t for the current lane ------------------------
    // Forward / batch kernels: step groups of U steps hold whole ChaCha
    // blocks in registers (indices known at compile time).
    void uniform_from(Out& o, int k, int g = -1) const {
        const std::string K = S(k);
        // FP32: the 53-bit uniform U (p = U 2^-53); the tail q / up / gt
        // only where a jump count, RK's sign or the accurate icdf reads it
        auto tail53 = [&]() {
            if (needs_tail(k))
                o.l("float " + V("q", k) + "; bool " + V("up", k) + ", " + V("gt", k) + "; sde_tail_u53(" + V("U", k) +
                    ", " + V("q", k) + ", " + V("up", k) + ", " + V("gt", k) + ");");
        };
        if (sp.rng == RNG_PSEUDO) {
            if (!f32) {
                o.l("const double " + V("u", k) + " = sde_u64_to_f64(" + V("r", k) + ");");
            } else {
                o.l("const sde_u64 " + V("U", k) + " = " + V("r", k) + " >> 11;");
                tail53();
            }
        } else if (shiftm() && grp_shift && g >= 0) {
            // dimension t*NI + k = chunk start + eo + e (eo: the step
            // group's offset in the chunk, a multiple of 4 or of the group's
            // dimensions): the chunk's high parts and this lane's LO words
            // in loads of lo_width() dimensions
            const int e = g * NI + k;
            const int lw = lo_width(), e0 = e - e % lw;
            const std::string at = S((e0 / 4) * 128 + e0 % 4);
            std::string word;
            if (lw == 1) {
                word = "__ldg(" + V("LOp") + " + " + at + ")";
            } else {
                if (e % lw == 0)
                    o.l("const uint" + S(lw) + " " + V("LW", e) + " = __ldg((const uint" + S(lw) + "*)(" + V("LOp") + " + " +
                        at + "));");
                static const char* const comp[4] = {"x", "y", "z", "w"};
                word = V("LW", e0) + "." + comp[e % lw];
            }
            o.l("const sde_u32 " + V("sa", k) + " = __shfl_sync(0xffffffffu, " + V("sh0") + ", eo + " + S(e) + ");");
            o.l("const sde_u32 " + V("sb", k) + " = __shfl_sync(0xffffffffu, " + V("sh1") + ", eo + " + S(e) + ");");
            o.l("const sde_u32 " + V("x", k) + " = (" + V("shi1") + " ? " + V("sb", k) + " : " + V("sa", k) + ") ^ " + word +
                ";");
            // U = uh 2^21 + ul in 32-bit pieces (the 64-bit U only where a
            // single normal, a jump count or RK's sign reads it)
            o.l("sde_u32 " + V("uh", k) + ", " + V("ul", k) + "; sde_shift_split(" + V("x", k) + ", " + V("r", k) + ", &" +
                V("uh", k) + ", &" + V("ul", k) + ");");
            o.l("const sde_u64 " + V("U", k) + " = ((sde_u64)" + V("uh", k) + " << 21) | " + V("ul", k) + ";");
            tail53();
        } else if (shiftm()) {
            // the dimension's point from the warp's two high parts (fetched
            // once per 32 dimensions) and this lane's low part
            o.l("const int " + V("sd", k) + " = t * " + S(NI) + " + " + K + ";");
            o.l("if ((" + V("sd", k) + " >> 5) != " + V("shc") + ") { " + V("shc") + " = " + V("sd", k) + " >> 5; " +
                V("shv0") + " = sde_sobol_hi_unrolled(a.sobol_vt, nullptr, a.sobol_dims, " + V("shc") + ", " +
                V("sH0") + ", lane); " + V("shv1") + " = sde_sobol_hi_unrolled(a.sobol_vt, nullptr, a.sobol_dims, " +
                V("shc") + ", " + V("sH1") + ", lane); }");
            o.l("const sde_u32 " + V("sa", k) + " = __shfl_sync(0xffffffffu, " + V("shv0") + ", " + V("sd", k) + " & 31);");
            o.l("const sde_u32 " + V("sb", k) + " = __shfl_sync(0xffffffffu, " + V("shv1") + ", " + V("sd", k) + " & 31);");
            o.l("const sde_u32 " + V("x", k) + " = (" + V("shi1") + " ? " + V("sb", k) + " : " + V("sa", k) +
                ") ^ __ldg(&a.sobol_lo[(sde_u64)(" + V("sd", k) + " >> 2) * 128u + " + V("sL") + " * 4u + (" +
                V("sd", k) + " & 3)]);");
            if (!f32) {
                o.l("const double " + V("v", k) + " = (double)" + V("x", k) + " * 0x1p-32 + sde_u64_to_f64(" + V("r", k) + ");");
                o.l("const double " + V("u", k) + " = " + V("v", k) + " - trunc(" + V("v", k) + ");");
            } else {
                o.l("const sde_u64 " + V("U", k) + " = sde_shift_u53(" + V("x", k) + ", " + V("r", k) + ");");
                tail53();
            }
        } else {
            o.l("const int " + V("d", k) + " = t * " + S(NI) + " + " + K + ";");
            o.l("if ((" + V("d", k) + " >> 5) != " + V("hchunk") + ") { " + V("hchunk") + " = " + V("d", k) +
                " >> 5; " + V("hval") + " = sde_sobol_hi(a.sobol_vt, mask_rep, a.sobol_dims, " + V("hchunk") +
                ", " + V("H") + ", lane); }");
            o.l("const sde_u32 " + V("y", k) + " = __shfl_sync(0xffffffffu, " + V("hval") + ", " + V("d", k) +
                " & 31) ^ __ldg(&a.sobol_lo[(sde_u64)(" + V("d", k) + " >> 2) * 128u + " + V("L") + " * 4u + (" +
                V("d", k) + " & 3)]);");
            if (!f32) o.l("const double " + V("u", k) + " = ((double)" + V("y", k) + " + 0.5) * 0x1p-32;");
            else o.l("float " + V("q", k) + "; bool " + V("up", k) + ", " + V("gt", k) + "; sde_tail_xor(" + V("y", k) +
                     ", " + V("q", k) + ", " + V("up", k) + ", " + V("gt", k) + ");");
        }
    }

    // uniforms of Wiener / jump indices k0 <= k < k1 (all by default)
    void uniforms(Out& o, int g, std::vector<bool>& block_done, int k0 = 0, int k1 = -1) const {
        if (k1 < 0) k1 = NI;
        for (int k = k0; k < k1; ++k) {
            if (xorm()) {
                // dimension t*NI + k = group base (a multiple of 32) + e
                const int e = g * NI + k, c = e / 32, l = e % 32;
                if (!block_done[c]) {
                    // forward kernels took it from the one-group-ahead fetch
                    if (!hv_pf())
                        o.l(V("hv", c) + " = sde_sobol_hi(a.sobol_vt, mask_rep, a.sobol_dims, chunk0 + " + S(c) +
                            ", " + V("H") + ", lane);");
                    block_done[c] = true;
                }
                // this lane's LO words come lw dimensions per load (16 or 8
                // bytes); lw divides NI, so a load never spans two steps and
                // every call draws whole loads (chunks of 8 in the
                // tensor-core step)
                const int lw = lo_width(), e0 = e - e % lw;
                const std::string at = S((e0 / 4) * 128 + e0 % 4);
                std::string word;
                if (lo_tma()) {
                    // from the step's shared-memory buffer (k: the index in the step)
                    const int k0q = k - k % 4;
                    if (k % 4 == 0)
                        o.l("const uint4 " + V("LW", k) + " = *(const uint4*)(" + V("LOS") + " + " + S(k0q / 4 * 512) + ");");
                    static const char* const cq[4] = {"x", "y", "z", "w"};
                    word = V("LW", k0q) + "." + cq[k % 4];
                } else if (lw == 1) {
                    word = "__ldg(" + V("LOp") + " + " + at + ")";
                } else {
                    if (e % lw == 0)
                        o.l("const uint" + S(lw) + " " + V("LW", e) + " = __ldg((const uint" + S(lw) + "*)(" + V("LOp") +
                            " + " + at + "));");
                    static const char* const comp[4] = {"x", "y", "z", "w"};
                    word = V("LW", e0) + "." + comp[e % lw];
                }
                o.l("const sde_u32 " + V("y", k) + " = __shfl_sync(0xffffffffu, " + V("hv", c) + ", " + S(l) +
                    ") ^ " + word + ";");
                if (!f32) o.l("const double " + V("u", k) + " = ((double)" + V("y", k) + " + 0.5) * 0x1p-32;");
                else if (needs_tail(k))
                    o.l("float " + V("q", k) + "; bool " + V("up", k) + ", " + V("gt", k) + "; sde_tail_xor(" +
                        V("y", k) + ", " + V("q", k) + ", " + V("up", k) + ", " + V("gt", k) + ");");
                continue;
            }
            if (uses_chacha()) {
                int pos = g * NI + k, b = pos / 8, w = (pos % 8) * 2;
                if (!block_done[b]) {
                    o.l("sde_chacha8_block(" + V("key") + ", blk0 + " + S(b) + "ull, " + V("B", b) + ");");
                    block_done[b] = true;
                }
                o.l("const sde_u64 " + V("r", k) + " = sde_pair(" + V("B", b) + "[" + S(w) + "], " + V("B", b) + "[" +
                    S(w + 1) + "]);");
            }
            uniform_from(o, k, g);
        }
    }

    // Random access by step (adjoint): ChaCha blocks cached per thread.
    void uniforms_ra(Out& o) const {
        for (int k = 0; k < NI; ++k) {
            if (uses_chacha()) {
                o.l("sde_u64 " + V("r", k) + ";");
                o.l("{ const sde_u64 pos = (sde_u64)t * " + S(NI) + "ull + " + S(k) + "ull;");
                o.l("  if ((pos >> 3) != cblk) { cblk = pos >> 3; sde_chacha8_block(" + V("key") + ", cblk, CB); }");
                o.l("  const int w = (int)(pos & 7ull) * 2; " + V("r", k) + " = sde_pair(CB[w], CB[w + 1]); }");
            }
            uniform_from(o, k);
        }
    }

    // Wiener increments w<k> = sqrt_dt * icdf(u<k>)   (increment.rs:89-97)
    // for k0 <= k < k1; mult replaces sqrt_dt (the tensor-core step writes
    // scaled standard normals and applies sqrt_dt to the product)
    void wiener(Out& o, bool from_words = false, const std::string& mult = "sdt", int k0 = 0, int k1 = -1) const {
        if (k1 < 0) k1 = NI;
        const bool acc = sp.icdf != 0;
        // FP32 with the AS 26.2.23 normal: pairs of Wiener indices share
        // paired FP32 arithmetic (fma.f32x2)
        // (wide universes -- dozens of normals per step feeding long FMA
        // chains -- are register-bound already; pairing is kept to <= 16,
        // except where the normals stream into shared memory)
        std::vector<int> paired;
        if (f32 && !acc && (from_words || !xorm()) && (NI <= 16 || mma)) {
            std::vector<int> ks;
            for (int k = k0; k < k1; ++k)
                if (u.token_kind[k] == IncKind::Dw) ks.push_back(k);
            for (size_t i = 0; i + 1 < ks.size(); i += 2) {
                const int ka = ks[i], kb = ks[i + 1];
                const std::string pr = V("wp" + S(ka) + "_", kb);
                // one reciprocal for the pair where the SFU pipe is the
                // bound (the CUDA-core kernels); one each in the tensor-core
                // step, which is bound by issue (measured both ways)
                const std::string tpl = mma ? "<false>(" : shiftm() ? "<true, true>(" : "(";
                const std::string src = xorm() ? "sde_normal_xor2" + tpl + V("y", ka) + ", " + V("y", kb) + ")"
                                        : grp_shift ? "sde_normal_split2(" + V("uh", ka) + ", " + V("ul", ka) + ", " +
                                                          V("uh", kb) + ", " + V("ul", kb) + ")"
                                                    : "sde_normal_u53_2" + tpl + V("U", ka) + ", " + V("U", kb) + ")";
                o.l("const float2 " + pr + " = __fmul2_rn(make_float2(" + mult + ", " + mult + "), " + src + ");");
                o.l("const float " + V("w", ka) + " = " + pr + ".x;");
                o.l("const float " + V("w", kb) + " = " + pr + ".y;");
                paired.push_back(ka);
                paired.push_back(kb);
            }
        }
        for (int k = k0; k < k1; ++k) {
            if (u.token_kind[k] != IncKind::Dw) continue;
            if (std::find(paired.begin(), paired.end(), k) != paired.end()) continue;
            if (!f32)
                o.l("const double " + V("w", k) + " = " + mult + " * " + (acc ? "sde_icdf_accurate(" : "sde_icdf_as26(") +
                    V("u", k) + ");");
            else if (from_words && !acc)
                o.l("const float " + V("w", k) + " = " + mult + " * sde_normal_xor(" + V("y", k) + ");");
            else if (!xorm() && !acc)
                o.l("const float " + V("w", k) + " = " + mult + " * sde_normal_u53(" + V("U", k) + ");");
            else
                o.l("const float " + V("w", k) + " = " + mult + " * " + (acc ? "sde_icdf_accurate_q(" : "sde_icdf_as26_q(") +
                    V("q", k) + ", " + V("up", k) + ");");
        }
    }

    // Poisson increments n<k> (increment.rs:137-148); the intensity is read
    // through the given register set at time tvar.
    void poisson(Out& o, const std::string& procset, const std::string& tvar) const {
        for (int k = 0; k < NI; ++k) {
            if (u.token_kind[k] != IncKind::Dn) continue;
            ExprP lam;
            for (const auto& p : u.procs)
                for (const auto& t : p.terms)
                    if (t.sidx == k && t.lambda) lam = t.lambda;
            std::string pu = f32 ? "(" + V("up", k) + " ? 1.0f - " + V("q", k) + " : " + V("q", k) + ")" : V("u", k);
            o.l("const " + R + " " + V("n", k) + " = sde_poisson(" + pu + ", " + ex(lam, "C", tvar) + " * dt);");
            (void)procset;
        }
    }

    std::string inc(const Term& t) const {
        if (t.kind == IncKind::Dt) return "dt";
        if (t.kind == IncKind::Dw) return V("w", t.sidx);
        return V("n", t.sidx);
    }

    std::string sk_expr() const {
        // with no stochastic index the reference panics at the first step
        // (src/rng/pseudo.rs:53-57); runs with steps are refused on the host
        if (NI == 0) return L(1.0);
        if (!f32) return "(" + V("u", 0) + " > 0.5 ? 1.0 : -1.0)";
        return "(" + V("gt", 0) + " ? 1.0f : -1.0f)";
    }

    // coefficient k * X_q (or X_q * k) -> (k, q); k may be any expression:
    // sum_j (k_j X_q) inc_j = X_q sum_j k_j inc_j holds whatever k_j is
    static bool split_linear(const ExprP& c, ExprP& k, int& q) { return split_linear_coef(c, k, q); }

    // Euler update of process p.  FP64 keeps the reference's term order
    // (val += c * inc per term).  FP32 factors coefficients k_j * X_q out of
    // the sum: X_q * (sum_j k_j inc_j), one FMA per term instead of two
    // operations; the value changes only by rounding.  With mma_d set, the
    // dW terms are already summed in mma_d (sum_j K_pj w_j from the tensor
    // cores) and join the group of X_p.
    void euler_update(Out& o, int p, const std::string& procset, const std::string& mma_d = "") const {
        o.l(R + " " + V("N", p) + " = " + V("X", p) + ";");
        const auto& terms = u.procs[p].terms;
        if (!f32) {
            for (const auto& t : terms)
                o.l(V("N", p) + " = " + V("N", p) + " + " + ex(t.coef, procset, "tc") + " * " + inc(t) + ";");
            return;
        }
        std::vector<int> groups;
        std::vector<std::vector<std::pair<ExprP, std::string>>> gterms;
        if (!mma_d.empty()) {
            groups.push_back(p);
            gterms.emplace_back();
        }
        for (const auto& t : terms) {
            ExprP k;
            int q;
            if (!mma_d.empty() && t.kind == IncKind::Dw) continue;
            if (split_linear(t.coef, k, q)) {
                auto it = std::find(groups.begin(), groups.end(), q);
                size_t gi = it - groups.begin();
                if (it == groups.end()) { groups.push_back(q); gterms.emplace_back(); }
                gterms[gi].push_back({k, inc(t)});
            } else {
                o.l(V("N", p) + " = " + V("N", p) + " + " + ex(t.coef, procset, "tc") + " * " + inc(t) + ";");
            }
        }
        for (size_t g = 0; g < groups.size(); ++g) {
            const std::string acc = V("acc" + S(p) + "_", (int)g);
            o.l(R + " " + acc + " = " + (!mma_d.empty() && g == 0 ? mma_d : L(0.0)) + ";");
            for (const auto& kt : gterms[g]) o.l(acc + " = " + acc + " + " + ex(kt.first, procset, "tc") + " * " + kt.second + ";");
            o.l(V("N", p) + " = " + V("N", p) + " + " + V(procset, groups[g]) + " * " + acc + ";");
        }
    }

    // ---- one step, reference semantics ---------------------------------
    void step_reference(Out& o) const {
        if (sp.scheme == SCHEME_EULER) {
            // cache refresh at t when no algebraic process left it at t
            if (!has_alg())
                for (int p : u.levy) o.l(V("C", p) + " = " + V("X", p) + ";");
            poisson(o, "C", "tc");
            for (int p : u.levy) euler_update(o, p, "C");
            if (has_alg()) {
                // refresh at t+1 before any algebraic slot of t+1 is written
                for (int p : u.levy) o.l(V("C", p) + " = " + V("N", p) + ";");
                for (int q : u.alg) o.l(V("C", q) + " = " + L(0.0) + ";");
                for (int q : u.alg) o.l(R + " " + V("N", q) + " = " + ex(u.procs[q].alg, "C", "tn") + ";");
            }
        } else {
            o.l("const " + R + " " + V("sk") + " = " + sk_expr() + ";");
            poisson(o, "C", "tc");
            for (int p : u.levy) {
                const auto& terms = u.procs[p].terms;
                const std::string cp = "c" + S(p) + "_";
                for (size_t j = 0; j < terms.size(); ++j)
                    o.l("const " + R + " " + V(cp, (int)j) + " = " + ex(terms[j].coef, "C", "tc") + ";");
                o.l(R + " " + V("k1_", p) + " = " + L(0.0) + ";");
                for (size_t j = 0; j < terms.size(); ++j)
                    o.l(V("k1_", p) + " = " + V("k1_", p) + " + " + V(cp, (int)j) + " * " + inc(terms[j]) + ";");
                o.l(R + " " + V("pe", p) + " = " + L(0.0) + ";");
                for (size_t j = 0; j < terms.size(); ++j)
                    if (terms[j].kind == IncKind::Dw)
                        o.l(V("pe", p) + " = " + V("pe", p) + " + " + V(cp, (int)j) + " * " + V("sk") + " * sdt;");
            }
            for (int p : u.levy)
                o.l(V("C", p) + " = " + V("X", p) + " + " + V("k1_", p) + " + " + V("pe", p) + ";");
            for (int q : u.alg) o.l(V("C", q) + " = " + L(0.0) + ";");
            for (int p : u.levy) {
                const auto& terms = u.procs[p].terms;
                o.l(R + " " + V("k2_", p) + " = " + L(0.0) + ";");
                for (size_t j = 0; j < terms.size(); ++j)
                    o.l(V("k2_", p) + " = " + V("k2_", p) + " + " + ex(terms[j].coef, "C", "tn") + " * " + inc(terms[j]) + ";");
                o.l(R + " " + V("N", p) + " = " + V("X", p) + " + " + L(0.5) + " * (" + V("k1_", p) + " + " + V("k2_", p) + ");");
            }
            for (int q : u.alg) o.l(R + " " + V("N", q) + " = " + ex(u.procs[q].alg, "C", "tn") + ";");
        }
        for (int p = 0; p < P; ++p) o.l(V("X", p) + " = " + V("N", p) + ";");
    }

    // ---- one step, textbook semantics ---------------------------------
    void settle_alg_textbook(Out& o) const {
        if (!has_alg()) return;
        for (int q : u.alg) o.l(R + " " + V("N", q) + " = " + V("X", q) + ";");
        for (int q : u.alg) o.l(V("N", q) + " = " + ex(u.procs[q].alg, "N", "tn") + ";");
    }
    void step_textbook(Out& o) const {
        // the Poisson intensity reads C, which is the true state here
        for (int p = 0; p < P; ++p) o.l(V("C", p) + " = " + V("X", p) + ";");
        if (sp.scheme == SCHEME_EULER) {
            poisson(o, "C", "tc");
            for (int p : u.levy) euler_update(o, p, "X");
            settle_alg_textbook(o);
        } else {
            o.l("const " + R + " " + V("sk") + " = " + sk_expr() + ";");
            poisson(o, "C", "tc");
            for (int p : u.levy) {
                const auto& terms = u.procs[p].terms;
                const std::string cp = "c" + S(p) + "_";
                o.l(R + " " + V("k1_", p) + " = " + L(0.0) + ";");
                o.l(R + " " + V("pe", p) + " = " + L(0.0) + ";");
                for (size_t j = 0; j < terms.size(); ++j) {
                    o.l("const " + R + " " + V(cp, (int)j) + " = " + ex(terms[j].coef, "X", "tc") + ";");
                    o.l(V("k1_", p) + " = " + V("k1_", p) + " + " + V(cp, (int)j) + " * " + inc(terms[j]) + ";");
                    if (terms[j].kind == IncKind::Dw)
                        o.l(V("pe", p) + " = " + V("pe", p) + " + " + V(cp, (int)j) + " * " + V("sk") + " * sdt;");
                }
            }
            for (int p = 0; p < P; ++p) {
                if (u.procs[p].levy)
                    o.l("const " + R + " " + V("PB", p) + " = " + V("X", p) + " + " + V("k1_", p) + " + " + V("pe", p) + ";");
                else
                    o.l("const " + R + " " + V("PB", p) + " = " + V("X", p) + ";");
            }
            for (int p : u.levy) {
                const auto& terms = u.procs[p].terms;
                o.l(R + " " + V("k2_", p) + " = " + L(0.0) + ";");
                for (size_t j = 0; j < terms.size(); ++j)
                    o.l(V("k2_", p) + " = " + V("k2_", p) + " + " + ex(terms[j].coef, "PB", "tn") + " * " + inc(terms[j]) + ";");
                o.l(R + " " + V("N", p) + " = " + V("X", p) + " + " + L(0.5) + " * (" + V("k1_", p) + " + " + V("k2_", p) + ");");
            }
            settle_alg_textbook(o);
        }
        for (int p = 0; p < P; ++p) o.l(V("X", p) + " = " + V("N", p) + ";");
    }

    void step(Out& o) const {
        if (sp.semantics == SEM_TEXTBOOK) step_textbook(o);
        else step_reference(o);
    }

    // ---- one Euler step with the dW terms on the tensor cores -------------
    // Eligible universes have no algebraic process, so the reference's cache
    // equals the state at t under both semantics (euler.rs:5-37).  The CTA's
    // 128 paths write their standard normals z (times 2^12, split into FP16
    // hi + lo) as rows of A, eight indices at a time as they are drawn; one
    // thread issues D = A_hi B_hi + A_hi B_lo + A_lo B_hi (3 FP16 products,
    // about FP32 accuracy; B = K with each row scaled by a power of two)
    // into tensor memory; each thread reads back its row and finishes the
    // update in FP32 with d_p = D_p sqrt_dt 2^-(12 + e_p) = sum_j K_pj w_j.
    const MmaShape* mma = nullptr;
    std::vector<int> row_e;   // B row p is K_p * 2^row_e[p]

    bool linear_drift(int p, double& c) const { return linear_drift_of(u, p, c); }

    // With S = mma->split threads per path (2 or 4), the thread of part h
    // (`half`) draws the normals of A columns [h KP/S, (h+1) KP/S), reads D
    // columns [h NP/S, (h+1) NP/S) and steps those processes.
    int half = 0;
    int kcols() const { return mma->kpad / mma->split; }
    int pcols() const { return mma->npad / mma->split; }
    // 32-dimension Sobol chunks of a group that this thread's indices touch
    std::vector<bool> own_chunks() const {
        const int nb = (group() * NI) / 32;
        const int k0 = mma ? half * kcols() : 0, k1 = mma ? std::min(NI, (half + 1) * kcols()) : NI;
        std::vector<bool> need(std::max(1, nb), false);
        for (int g = 0; g < group(); ++g)
            for (int k = k0; k < k1; ++k) need[(g * NI + k) / 32] = true;
        return need;
    }

    void step_mma(Out& o, int g, std::vector<bool>& done) const {
        const int KH = kcols(), PH = pcols();
        if (lo_tma()) {
            // this step's LO words, bulk-copied two steps ago
            o.l("if (!sde_mbar_wait_bounded(LBAR0 + 8u * (sde_u32)(t & 1), (sde_u32)(t >> 1) & 1u)) tc_ok = 0;");
            o.l("lb_waited = t;");
            o.l("const unsigned char* const " + V("LOS") + " = LOB + (t & 1) * " + S(mma->lo_step_bytes) + " + " + V("L") +
                " * 16u;");
        }
        for (int k8 = half * KH; k8 < (half + 1) * KH; k8 += 8) {
            if (k8 < NI) {
                uniforms(o, g, done, k8, std::min(k8 + 8, NI));
                wiener(o, xorm() && f32, "0x1p12f", k8, std::min(k8 + 8, NI));
            }
            std::string e[8];
            bool any = false;
            for (int i = 0; i < 8; ++i) {
                const int k = k8 + i;
                const bool dw = k < NI && u.token_kind[k] == IncKind::Dw;
                e[i] = dw ? V("w", k) : "0.0f";
                any = any || dw;
            }
            if (!any) continue;  // stays zero from the prologue
            const std::string off = S(k8 / 8 * 128);
            o.l("{ sde_u32 h0, h1, h2, h3, l0, l1, l2, l3;");
            for (int i = 0; i < 4; ++i)
                o.l("  sde_split_f16x2(" + e[2 * i] + ", " + e[2 * i + 1] + ", h" + S(i) + ", l" + S(i) + ");");
            o.l("  *(uint4*)(ARH + " + off + ") = make_uint4(h0, h1, h2, h3);");
            o.l("  *(uint4*)(ARL + " + off + ") = make_uint4(l0, l1, l2, l3); }");
        }
        // A ready: a CTA barrier whose vote also ends the loop together;
        // then thread 0 issues the product and commits it to DBAR.
        o.l("sde_fence_async_smem();");
        o.l("sde_tc_fence_before();");
        auto issue = [&](const std::string& pad) {
            for (int c = 0; c < mma->kpad / 16; ++c) {
                const std::string dc = S(c * 16) + "ull";  // 256 bytes further along K, in 16-byte units
                o.l(pad + "sde_mma_f16(tmem, ADH + " + dc + ", BDH + " + dc + ", IDESC, " + (c ? "1u" : "0u") + ");");
                o.l(pad + "sde_mma_f16(tmem, ADH + " + dc + ", BDL + " + dc + ", IDESC, 1u);");
                o.l(pad + "sde_mma_f16(tmem, ADL + " + dc + ", BDH + " + dc + ", IDESC, 1u);");
            }
            o.l(pad + "sde_mma_commit(DBAR);");
            // every thread has read this step's LO buffer (the A barrier):
            // refill it with the words of step t + 2
            if (lo_tma()) lo_issue(o, pad, "t + 2");
        };
        if (mma->split == 1) {
            // one thread per path: a CTA vote, the loop's only exit, so every
            // warp takes the same votes
            o.l("if (!__syncthreads_and(tc_ok)) break;");
            o.l("sde_tc_fence_after();");
            o.l("if (threadIdx.x == 0) {");
            issue("  ");
            o.l("}");
        } else {
            // several threads per path (separate copies of the loop): every
            // thread arrives on ABAR; warp 0 waits as a whole, so lane 0 never
            // waits behind lanes of its own warp suspended on DBAR
            o.l("sde_mbar_arrive(ABAR);");
            if (half == 0) {
                o.l("if (threadIdx.x < 32) {");
                o.l("  const bool a_ready = sde_mbar_wait_budget(ABAR, tc_phase, a.tc_wait_cycles);");
                o.l("  if (!a_ready) tc_ok = 0;");
                o.l("  if (threadIdx.x == 0 && a_ready) {");
                o.l("    sde_tc_fence_after();");
                issue("    ");
                o.l("  }");
                o.l("}");
            }
        }
        // lanes 1..31 of warp 0 must not suspend on DBAR before lane 0 has
        // issued
        if (half == 0) o.l("__syncwarp();");
        // while the MMA runs: the next group's Sobol high parts
        if (xorm() && g == group() - 1) hv_prefetch(o, "chunk0 + " + S((group() * NI) / 32));
        o.l("if (!sde_mbar_wait_bounded(DBAR, tc_phase)) tc_ok = 0;");
        o.l("tc_phase ^= 1u;");
        if (mma->split == 1)  // a timed-out thread carries on; the next vote ends the loop for all
            o.l("__syncwarp();");
        else  // a warp leaves together (tcgen05.ld below is warp-collective)
            o.l("if (!__all_sync(0xffffffffu, tc_ok)) break;");
        o.l("sde_tc_fence_after();");
        o.l("float DM[" + S(PH) + "];");
        // 16 columns per load: a block of D is consumed before the next one
        // is loaded, so D and the state need not be live in full at once
        // (one 32-column load was measured: no faster, more spills)
        for (int c = 0; c < PH; c += 16) o.l("sde_tmem_ld16_wait(TROW + " + S(c) + "u, DM + " + S(c) + ");");
        o.l("const float sdz = sdt * 0x1p-12f;");
        for (int p : u.levy)
            if (p >= plo && p < pend()) o.l(V("C", p) + " = " + V("X", p) + ";");
        poisson(o, "C", "tc");
        for (int p : u.levy) {
            if (p < plo || p >= pend()) continue;
            const std::string d = "DM[" + S(p - half * PH) + "]";
            const std::string f = row_e[p] == 0 ? "sdz" : "(sdz * " + lit(std::ldexp(1.0, -row_e[p]), true) + ")";
            double c = 0.0;
            // N = X + X (c dt + d): two FMAs (c dt is shared by equal c).  Not
            // X (1 + c dt + d): 1 + c dt would round the same way every step
            // and bias the paths coherently
            if (linear_drift(p, c))
                o.l("const float " + V("N", p) + " = fmaf(" + V("X", p) + ", fmaf(" + d + ", " + f + ", " + lit(c, true) +
                    " * dt), " + V("X", p) + ");");
            else
                euler_update(o, p, "C", d + " * " + f);
        }
        for (int p = plo; p < pend(); ++p) o.l(V("X", p) + " = " + V("N", p) + ";");
    }

    // Forward kernel on the tensor cores (one path per thread, 128 paths per
    // CTA = the MMA's M).  Shared memory: A_hi, A_lo [128 x KP], B_hi, B_lo
    // [NP x KP] FP16, all in the no-swizzle K-major core-matrix layout
    // (8 rows x 16 bytes per core matrix); element (r, k) at half
    // (r/8)*(8 KP) + (k/8)*64 + (r%8)*8 + k%8.  D [128 x NP] FP32 in tensor
    // memory.  Every wait is bounded: on a timeout the CTA stops stepping,
    // frees its tensor memory and sets *a.status.
    std::string forward_mma(const std::string& name, const std::vector<std::vector<double>>& K) {
        mode = Mode::Forward;
        lane(0);
        const int KP = mma->kpad, NP = mma->npad;
        const int NPAY = (int)sp.payoffs.size();
        Out o;
        // per-row power-of-two scale: the largest |K_pj 2^e_p| lies in
        // [2^12, 2^13), so FP16 holds B_hi and the B_lo remainders
        row_e.assign(P, 0);
        for (int n = 0; n < P; ++n) {
            double mx = 0.0;
            for (int k = 0; k < NI; ++k) mx = std::max(mx, std::fabs(K[n][k]));
            if (mx > 0.0) {
                int ex = 0;
                std::frexp(mx, &ex);  // mx < 2^ex
                row_e[n] = std::max(-100, std::min(100, 13 - ex));
            }
        }
        // B_hi then B_lo as one shared-memory image
        std::vector<uint16_t> img(2 * (size_t)NP * KP, 0);
        for (int n = 0; n < P; ++n)
            for (int k = 0; k < NI; ++k) {
                const float kf = (float)std::ldexp(K[n][k], row_e[n]);
                const uint16_t hi = f32_to_f16(kf);
                const uint16_t lo = f32_to_f16(kf - f16_to_f32(hi));
                const size_t at = (size_t)(n / 8) * (8 * KP) + (k / 8) * 64 + (n % 8) * 8 + k % 8;
                img[at] = hi;
                img[(size_t)NP * KP + at] = lo;
            }
        o.l("static __device__ __align__(16) const unsigned short " + name + "_kmat[" + S((int)img.size()) + "] = {");
        for (size_t i = 0; i < img.size(); i += 16) {
            std::string row = "  ";
            for (size_t j = i; j < std::min(img.size(), i + 16); ++j) {
                char b[16];
                std::snprintf(b, sizeof b, "0x%04x, ", img[j]);
                row += b;
            }
            o.l(row);
        }
        o.l("};");
        const int TH = 128 * mma->split;  // threads per CTA
        o.l("extern \"C\" __global__ void __launch_bounds__(" + S(TH) + ", " + S(mma->min_blocks) + ") " + name +
            "(const sde_args a) {");
        o.ind++;
        o.l("extern __shared__ __align__(1024) unsigned char sde_smem[];");
        o.l("unsigned char* const SAH = sde_smem;");
        o.l("unsigned char* const SAL = SAH + " + S(128 * KP * 2) + ";");
        o.l("unsigned char* const SBH = SAL + " + S(128 * KP * 2) + ";");
        o.l("unsigned char* const SBL = SBH + " + S(NP * KP * 2) + ";");
        o.l("sde_u64* const MBP = (sde_u64*)(SBL + " + S(NP * KP * 2) + ");");
        o.l("sde_u32* const TSLOT = (sde_u32*)(MBP + 4);");
        // ABAR: A written (several threads per path: every thread arrives);
        // DBAR: the step's product committed (one arrival, tcgen05.commit);
        // LBAR0 / LBAR0 + 8: the two LO step buffers filled
        o.l("const sde_u32 ABAR = sde_smem_addr(MBP), DBAR = sde_smem_addr(MBP + 1), LBAR0 = sde_smem_addr(MBP + 2);");
        o.l("(void)ABAR; (void)LBAR0;");
        o.l("int lb_issued = -1, lb_waited = -1;");
        o.l("(void)lb_issued; (void)lb_waited;");
        if (lo_tma()) {
            o.l("const unsigned char* const LOB = sde_smem + " + S(mma->lo_off) + ";");
            o.l("const sde_u32 LOBA = sde_smem_addr(LOB);");
        }
        o.l("for (int e = threadIdx.x; e < " + S(2 * 128 * KP * 2 / 16) + "; e += " + S(TH) +
            ") ((uint4*)SAH)[e] = make_uint4(0u, 0u, 0u, 0u);");
        o.l("for (int e = threadIdx.x; e < " + S(2 * NP * KP * 2 / 16) + "; e += " + S(TH) +
            ") ((uint4*)SBH)[e] = ((const uint4*)" + name + "_kmat)[e];");
        o.l("if (threadIdx.x == 0) {");
        o.l("  sde_mbar_init(ABAR, " + S(TH) + "u); sde_mbar_init(DBAR, 1u);");
        if (lo_tma()) o.l("  sde_mbar_init(LBAR0, 1u); sde_mbar_init(LBAR0 + 8u, 1u);");
        o.l("  sde_fence_mbar_init();");
        if (lo_tma()) {
            lo_issue(o, "  ", "0");
            lo_issue(o, "  ", "1");
        }
        o.l("}");
        o.l("__syncwarp();");
        o.l("if (threadIdx.x < 32) sde_tmem_alloc(sde_smem_addr(TSLOT), " + S(mma->ncols) + "u);");
        o.l("sde_fence_async_smem();");
        o.l("sde_tc_fence_before();");
        o.l("__syncthreads();");
        o.l("sde_tc_fence_after();");
        o.l("const sde_u32 tmem = *TSLOT;");
        // the thread's path in the tile (its A row and TMEM lane) and half
        o.l("const int r = threadIdx.x & 127;");
        o.l("const int half = threadIdx.x >> 7;");
        o.l("(void)half;");
        // warps w and w + 4 reach lanes 32 (w % 4) ..; half h reads D columns from h NP / split
        o.l("const sde_u32 TROW = tmem + ((sde_u32)(r & ~31) << 16) + (sde_u32)half * " + S(pcols()) + "u;");
        // LBO: the two core matrices of one MMA's K slice; SBO: 8-row groups
        o.l("const sde_u32 IDESC = sde_idesc_f16(128, " + S(NP) + ");");
        o.l("const sde_u64 ADH = sde_smem_desc(sde_smem_addr(SAH), 128u, " + S(KP * 16) + "u);");
        o.l("const sde_u64 ADL = sde_smem_desc(sde_smem_addr(SAL), 128u, " + S(KP * 16) + "u);");
        o.l("const sde_u64 BDH = sde_smem_desc(sde_smem_addr(SBH), 128u, " + S(KP * 16) + "u);");
        o.l("const sde_u64 BDL = sde_smem_desc(sde_smem_addr(SBL), 128u, " + S(KP * 16) + "u);");
        o.l("(void)ADH; (void)ADL; (void)BDH; (void)BDL; (void)IDESC;");
        o.l("unsigned char* const ARH = SAH + (r >> 3) * " + S(16 * KP) + " + (r & 7) * 16;");
        o.l("unsigned char* const ARL = ARH + " + S(128 * KP * 2) + ";");
        o.l("int tc_ok = 1;");
        o.l("sde_u32 tc_phase = 0u;");
        row = "r";
        cta = "128";
        shared_prologue(o);
        if (mma->split == 1) {
            lane_prologue(o);
            store(o, "0");
            time_loop(o);
        } else {
            // each part steps its own processes in its own copy of the loop
            // (its registers hold only those); the parts meet only at the
            // mbarriers, whose waits are bounded
            for (int h = 0; h < mma->split; ++h) {
                half = h;
                plo = h * pcols();
                phi = std::min(P, (h + 1) * pcols());
                o.l(h == 0 ? "if (half == 0) {"
                           : h + 1 < mma->split ? "} else if (half == " + S(h) + ") {" : "} else {");
                o.ind++;
                lane_prologue(o);
                store(o, "0");
                time_loop(o);
                // the state goes to shared memory (the operand area, free
                // now) for the payoffs
                for (int p = plo; p < pend(); ++p) o.l("((float*)sde_smem)[" + S(p * 128) + " + r] = " + V("X", p) + ";");
                o.ind--;
            }
            o.l("}");
            half = 0;
            plo = 0;
            phi = -1;
        }
        // teardown: every thread arrives here (one thread per path: after the
        // same votes; several: the loops hold no CTA barrier).  A loop left
        // early may leave LO copies in flight: thread 0 waits for them
        if (lo_tma())
            o.l("if (threadIdx.x == 0) for (int s_ = lb_waited + 1; s_ <= lb_issued; ++s_) "
                "(void)sde_mbar_wait_bounded(LBAR0 + 8u * (sde_u32)(s_ & 1), (sde_u32)(s_ >> 1) & 1u);");
        o.l("sde_tc_fence_before();");
        o.l("const int tc_all = __syncthreads_and(tc_ok);");
        o.l("sde_tc_fence_after();");
        o.l("if (threadIdx.x < 32) {");
        o.l("  if (!tc_all) (void)sde_mbar_wait_bounded(DBAR, tc_phase ^ 1u);");
        o.l("  __syncwarp();");
        o.l("  sde_tmem_dealloc(tmem, " + S(mma->ncols) + "u);");
        o.l("}");
        o.l("if (!tc_all && threadIdx.x == 0 && a.status) atomicOr(a.status, 1);");
        if (NPAY > 0) {
            o.l("double fs[" + S(NPAY) + "] = {}, fq[" + S(NPAY) + "] = {};");
            if (mma->split == 1) {
                payoffs(o, NPAY);
            } else {
                o.l("if (half == 0) {");
                o.ind++;
                o.l("const bool active = base + r < a.n_paths;");
                for (int p = 0; p < P; ++p) o.l("const float X" + S(p) + " = ((const float*)sde_smem)[" + S(p * 128) + " + r];");
                payoffs(o, NPAY);
                o.ind--;
                o.l("}");
            }
            o.l("sde_block_reduce_store<" + S(NPAY) + ">(fs, fq, a.partials + (((sde_u64)rep * gridDim.x + blockIdx.x) * " +
                S(NPAY) + "u) * 4u);");
        }
        row = "threadIdx.x";
        cta = "blockDim.x";
        o.ind--;
        o.l("}");
        return o.s.str();
    }

    void store(Out& o, const std::string& tidx) const {
        if (!sp.store_output || mode != Mode::Forward) return;
        o.l("{ const int slot = __ldg(&a.out_tidx[" + tidx + "]);");
        o.l("  if (slot >= 0 && " + V("active") + ") {");
        o.l("    " + R + "* dst = OUT + ((sde_u64)rep * a.n_out + slot) * (sde_u64)" + S(P) + " * a.n_paths + " + V("i") + ";");
        for (int p = plo; p < pend(); ++p)
            o.l("    dst[(sde_u64)" + S(p) + " * a.n_paths] = " + V("X", p) + ";");
        o.l("  } }");
    }

    // Processes [plo, pend()) are this thread's (all but in the tensor-core
    // kernel with several threads per path); `row` is the thread's path within
    // the CTA and `cta` the CTA's paths per lane.
    int plo = 0, phi = -1;
    int pend() const { return phi < 0 ? P : phi; }
    std::string row = "threadIdx.x", cta = "blockDim.x";

    // ---- per-lane state --------------------------------------------------
    void lane_prologue(Out& o) const {
        if (mode == Mode::Forward) {
            o.l("const sde_u64 " + V("i") + " = base + " + S(0) + "ull + (sde_u64)" + (sfx.empty() ? "0" : sfx.substr(1)) +
                " * " + cta + " + " + row + ";");
            o.l("const bool " + V("active") + " = " + V("i") + " < a.n_paths;");
            o.l("const sde_u64 " + V("scen") + " = a.path_base + (sde_u64)rep * a.n_paths + " + V("i") + ";");
            for (int p = plo; p < pend(); ++p) o.l(R + " " + V("X", p) + " = (" + R + ")__ldg(&a.x0[" + S(p) + "]);");
        } else {
            o.l("const sde_u64 " + V("i") + " = first + (sde_u64)" + (sfx.empty() ? "0" : sfx.substr(1)) +
                " * blockDim.x + threadIdx.x;");
            o.l("const bool " + V("active") + " = " + V("i") + " < in.n_paths;");
            o.l("const sde_u64 " + V("scen") + " = " + V("i") + ";");
            for (int p = 0; p < P; ++p) o.l(R + " " + V("X", p) + " = (" + R + ")__ldg(&a.x0[in.x0_off + " + S(p) + "]);");
        }
        o.l("(void)" + V("scen") + ";");
        for (int p = plo; p < pend(); ++p) o.l(R + " " + V("C", p) + " = " + V("X", p) + ";");
        const std::string seed = mode == Mode::Forward ? "a.seed" : "in.seed";
        if (uses_chacha()) o.l("sde_u32 " + V("key") + "[8]; sde_seed_from_u64(" + seed + " + " + V("scen") + ", " + V("key") + ");");
        if (shiftm()) {
            // point n = scenario + 5 (the reference's skip(5)); gray(n) >> 5 ==
            // gray(n >> 5), and a warp's 32 consecutive points fall in two
            // groups of 32, W0 = lane 0's n >> 5 and W0 + 1.  The warp
            // evaluates both groups' high parts for 32 dimensions at a time
            // (sde_sobol_hi_unrolled); the low five bits of gray(n) index LO.
            // Lanes past the last point may wrap n; they are inactive, and
            // W0 + 1 beyond the table's 27 high bits reads nothing.
            o.l("const sde_u32 " + V("sn") + " = (sde_u32)(" + V("scen") + " + 5ull);");
            o.l("const sde_u32 " + V("sL") + " = sde_gray(" + V("sn") + ") & 31u;");
            o.l("const sde_u32 " + V("sW0") + " = __shfl_sync(0xffffffffu, " + V("sn") + " >> 5, 0);");
            o.l("const bool " + V("shi1") + " = (" + V("sn") + " >> 5) != " + V("sW0") + ";");
            o.l("const sde_u32 " + V("sH0") + " = sde_gray(" + V("sW0") + ");");
            o.l("const sde_u32 " + V("sH1") + " = " + V("sW0") + " + 1u < (1u << 27) ? sde_gray(" + V("sW0") +
                " + 1u) : 0u;");
            o.l("int " + V("shc") + " = -1; sde_u32 " + V("shv0") + " = 0u, " + V("shv1") + " = 0u;");
        }
        if (xorm()) {
            o.l("const sde_u32 " + V("Gx") + " = sde_gray((sde_u32)" + V("i") + ");");
            o.l("const sde_u32 " + V("L") + " = " + V("Gx") + " & 31u, " + V("H") + " = " + V("Gx") + " >> 5;");
            o.l("int " + V("hchunk") + " = -1; sde_u32 " + V("hval") + " = 0u;");
        }
    }

    void shared_prologue(Out& o) const {
        o.l("const int lane = threadIdx.x & 31;");
        o.l("(void)lane;");
        if (mode == Mode::Forward) {
            o.l("const int rep = blockIdx.y;");
            o.l("const sde_u64 base = (sde_u64)blockIdx.x * " + cta + " * " + S(ppt) + "ull;");
            o.l("const int n_steps = a.T - 1;");
            for (int k = 0; k < (int)u.params.size(); ++k)
                o.l("const " + R + " PR" + S(k) + " = (" + R + ")__ldg(&a.params[" + S(k) + "]);");
            if (sp.store_output) o.l(R + "* OUT = (" + R + "*)a.out;");
            if (xorm()) o.l("const sde_u32* mask_rep = a.masks ? a.masks + (sde_u64)rep * a.mask_stride : nullptr;");
        } else {
            o.l("const int n_steps = in.n_steps;");
            o.l("const " + R + " bdt = (" + R + ")in.dt" + (f32 ? "_f" : "") + ";");
            o.l("const " + R + " bsdt = (" + R + ")in.sdt" + (f32 ? "_f" : "") + ";");
            for (int k = 0; k < (int)u.params.size(); ++k)
                o.l("const " + R + " PR" + S(k) + " = (" + R + ")__ldg(&a.params[in.par_off + " + S(k) + "]);");
        }
    }

    void step_header(Out& o) const {
        if (mode == Mode::Forward) {
            o.l("const " + R + " tc = " + T("times") + ";");
            o.l("const " + R + " tn = " + T("times", "t + 1") + ";");
            if (sp.ugrid && f32) {
                o.l("const " + R + " dt = a.udt_f;");
                o.l("const " + R + " sdt = a.usdt_f;");
            } else {
                o.l("const " + R + " dt = " + T("dts") + ";");
                o.l("const " + R + " sdt = " + T("sqrt_dts") + ";");
            }
        } else {
            o.l("const " + R + " tc = (" + R + ")t * bdt;");
            o.l("const " + R + " tn = (" + R + ")(t + 1) * bdt;");
            o.l("const " + R + " dt = bdt;");
            o.l("const " + R + " sdt = bsdt;");
        }
        o.l("(void)tc; (void)tn; (void)dt; (void)sdt;");
    }

    // Sobol high parts of the 32-dimension chunks of the group starting at
    // chunk `first` (an expression), fetched a group ahead; chunks past the
    // last step's dimensions are not read (the scramble-mask rows end
    // there).  The tensor-core step with one thread per path issues the
    // loads eight bits of H at a time (sde_sobol_hi_unrolled); the others
    // loop over H's set bits, fewer instructions now that the fetch runs a
    // group ahead (Heston 7.95 -> 7.81 ms, FP32 GBM 1.08 -> 1.01 ms; the
    // 64-dim basket with two threads per path 22.14 -> 21.26 ms, while one
    // thread per path slowed from 25.45 to 28.86 ms with the loop)
    void hv_prefetch(Out& o, const std::string& first) const {
        const std::vector<bool> need = own_chunks();
        for (int c = 0; c < (int)need.size(); ++c)
            if (need[c])
                o.l("if (32 * (" + first + " + " + S(c) + ") < n_steps * " + S(NI) + ") " + V("hvn", c) +
                " = " + (mma && mma->split == 1 ? "sde_sobol_hi_unrolled" : "sde_sobol_hi") +
                "(a.sobol_vt, mask_rep, a.sobol_dims, " + first + " + " + S(c) + ", " +
                V("H") + ", lane);");
    }

    // forward kernels on XOR-scrambled Sobol fetch each group's high parts
    // one group ahead, so the direction-number loads are never waited for
    // (CUDA-core kernels only where a group spans several steps: with one
    // step per group the fetch lands no earlier and costs registers)
    bool hv_pf() const { return xorm() && mode == Mode::Forward && (mma || group() >= 2); }

    void time_loop(Out& o) {
        const int U = group();
        const int nblocks = uses_chacha() ? (U * NI) / 8 : (xorm() ? (U * NI) / 32 : 0);
        const std::vector<bool> need = hv_pf() ? own_chunks() : std::vector<bool>();
        if (hv_pf()) {
            for (int j = 0; j < ppt; ++j) {
                lane(j);
                for (int c = 0; c < nblocks; ++c)
                    if (need[c]) o.l("sde_u32 " + V("hvn", c) + " = 0u;");
                hv_prefetch(o, "0");
            }
            lane(0);
        }
        if (grp_shift) {
            // a 32-dimension chunk: its high parts for the warp's two point
            // groups, then its step groups in a rolled loop
            const int OS = 32 / NI;
            o.l("for (int t1 = 0; t1 < n_steps; t1 += " + S(OS) + ") {");
            o.ind++;
            o.l("const int chunk0 = (t1 * " + S(NI) + ") >> 5;");
            for (int j = 0; j < ppt; ++j) {
                lane(j);
                o.l("const sde_u32 " + V("sh0") + " = sde_sobol_hi_unrolled(a.sobol_vt, nullptr, a.sobol_dims, chunk0, " +
                    V("sH0") + ", lane);");
                o.l("const sde_u32 " + V("sh1") + " = sde_sobol_hi_unrolled(a.sobol_vt, nullptr, a.sobol_dims, chunk0, " +
                    V("sH1") + ", lane);");
                o.l("const sde_u32* " + V("LOp1") + " = a.sobol_lo + (sde_u64)t1 * " + S(NI * 32) + "u + " + V("sL") +
                    " * 4u;");
            }
            lane(0);
            o.l("#pragma unroll 1");
            o.l("for (int t0 = t1; t0 < min(t1 + " + S(OS) + ", n_steps); t0 += " + S(U) + ") {");
        } else {
            o.l("for (int t0 = 0; t0 < n_steps; t0 += " + S(U) + ") {");
        }
        o.ind++;
        if (uses_chacha()) {
            o.l("const sde_u64 blk0 = ((sde_u64)t0 * " + S(NI) + "ull) / 8ull;");
            for (int j = 0; j < ppt; ++j) {
                lane(j);
                for (int b = 0; b < nblocks; ++b) o.l("sde_u32 " + V("B", b) + "[16];");
            }
        }
        if (xorm()) {
            // the group starts at dimension t0*NI, a multiple of 32
            o.l("const int chunk0 = (t0 * " + S(NI) + ") >> 5;");
            for (int j = 0; j < ppt; ++j) {
                lane(j);
                // the group starts at dimension t0*NI, a multiple of 32
                o.l("const sde_u32* " + V("LOp") + " = a.sobol_lo + (sde_u64)t0 * " + S(NI * 32) + "u + " + V("L") +
                    " * 4u;");
                for (int c = 0; c < nblocks; ++c)
                    o.l("sde_u32 " + V("hv", c) + (hv_pf() && need[c] ? " = " + V("hvn", c) : "") + ";");
                // the next group's, now; the tensor-core step issues its own
                // while the product runs
                if (hv_pf() && !mma) hv_prefetch(o, "chunk0 + " + S(nblocks));
            }
        }
        if (grp_shift) {
            // the step group's dimensions from offset eo of the chunk
            o.l("const int eo = (t0 - t1) * " + S(NI) + ";");
            for (int j = 0; j < ppt; ++j) {
                lane(j);
                o.l("const sde_u32* " + V("LOp") + " = " + V("LOp1") + " + (eo >> 2) * 128;");
            }
            lane(0);
        }
        // a full group (every group but perhaps the last) runs its steps
        // without the per-step bound check: forward CUDA-core kernels on
        // Sobol points.  (Measured on GB300: FP32 GBM 1.13 -> 1.08 ms on XOR
        // scrambles and 4.80 -> 4.44 ms shifted, Heston XOR unchanged; the
        // ChaCha8 kernels and the batched kernel, which carries every
        // template, slowed with the larger code: batched 54.5 -> 60.4 ms)
        const bool full_copy = !mma && U > 1 && mode == Mode::Forward && sp.rng == RNG_SOBOL;
        const std::vector<std::vector<bool>> done0(ppt, std::vector<bool>(std::max(1, nblocks), false));
        for (int copy = full_copy ? 0 : 1; copy < 2; ++copy) {
        if (full_copy) o.l(copy == 0 ? "if (t0 + " + S(U) + " <= n_steps) {" : "} else {");
        std::vector<std::vector<bool>> done = done0;
        for (int g = 0; g < U; ++g) {
            o.l("{ const int t = t0 + " + S(g) + ";");
            o.l(copy == 0 ? "{" : "if (t < n_steps) {");
            o.ind++;
            step_header(o);
            for (int j = 0; j < ppt; ++j) {
                lane(j);
                o.l("{");
                o.ind++;
                if (mma) {
                    step_mma(o, g, done[j]);
                } else {
                    uniforms(o, g, done[j]);
                    wiener(o, xorm() && f32);
                    step(o);
                }
                store(o, "t + 1");
                o.ind--;
                o.l("}");
            }
            o.ind--;
            o.l("} }");
        }
        }
        if (full_copy) o.l("}");
        o.ind--;
        o.l("}");
        if (grp_shift) {
            o.ind--;
            o.l("}");
        }
        lane(0);
    }

    // payoff sums: fs[k], fq[k] (this thread's lanes)
    void payoffs(Out& o, int K) {
        const std::string tT = mode == Mode::Forward ? "(" + R + ")__ldg(&a.times[a.T - 1])"
                                                     : "(" + R + ")n_steps * bdt";
        o.l("const " + R + " tT = " + tT + "; (void)tT;");
        for (int j = 0; j < ppt; ++j) {
            lane(j);
            for (int k = 0; k < (int)sp.payoffs.size(); ++k) {
                o.l("{ const double v = " + V("active") + " ? (double)(" + ex(sp.payoffs[k], "X", "tT") + ") : 0.0;");
                o.l("  fs[" + S(k) + "] += v; fq[" + S(k) + "] += v * v; }");
            }
        }
        lane(0);
        (void)K;
    }

    std::string forward(const std::string& name) {
        mode = Mode::Forward;
        grp_shift = grp_shift_eligible();
        const int K = (int)sp.payoffs.size();
        Out o;
        o.l("extern \"C\" __global__ void __launch_bounds__(" + S(sp.block) + ") " + name + "(const sde_args a) {");
        o.ind++;
        shared_prologue(o);
        for (int j = 0; j < ppt; ++j) {
            lane(j);
            lane_prologue(o);
            store(o, "0");
        }
        lane(0);
        time_loop(o);
        if (K > 0) {
            o.l("double fs[" + S(K) + "] = {}, fq[" + S(K) + "] = {};");
            payoffs(o, K);
            o.l("sde_block_reduce_store<" + S(K) + ">(fs, fq, a.partials + (((sde_u64)rep * gridDim.x + blockIdx.x) * " +
                S(K) + "u) * 4u);");
        }
        o.ind--;
        o.l("}");
        grp_shift = false;
        return o.s.str();
    }

    // Forward kernel for runs with few paths (the reference's 10,000): one
    // thread per path leaves most of the GPU idle and each thread runs a
    // long chain of FP64 inverse CDFs.  Here a CTA of 8 warps owns 32 paths
    // and walks the steps in chunks of 8 step groups.  Phase A: warp w draws
    // group w of the chunk for all 32 paths (its ChaCha blocks, the FP64
    // inverse CDFs) into shared memory.  Phase B: warp 0 steps the 32 paths
    // through the chunk with the same step code as the one-thread-per-path
    // kernel, reading the increments back, and stores the filtration.  The
    // arithmetic is unchanged, so the paths are the same bit for bit.
    // (NI dividing 8: a step group is one ChaCha block, and the two chunk
    // buffers take 32 KB of static shared memory)
    static bool chunked_eligible(const Universe& u, const KernelSpec& s) {
        const int NI = u.n_stochastic();
        return s.precision == PREC_FP64 && !s.adjoint && s.ppt == 1 && !s.tensor_cores &&
               (s.rng == RNG_PSEUDO || s.scramble == SCRAMBLE_SHIFT) && NI > 0 && 8 % NI == 0;
    }
    std::string forward_chunked(const std::string& name) {
        mode = Mode::Forward;
        lane(0);
        const int U = group(), CH = 8 * U;
        const int NPAY = (int)sp.payoffs.size();
        Out o;
        o.l("extern \"C\" __global__ void __launch_bounds__(256) " + name + "(const sde_args a) {");
        o.ind++;
        // increments and uniforms of one chunk: [step][index][path]
        o.l("__shared__ double SW[" + S(CH * NI * 32) + "];");
        o.l("__shared__ double SU[" + S(CH * NI * 32) + "];");
        o.l("const int warp = threadIdx.x >> 5;");
        row = "lane";
        cta = "32";
        shared_prologue(o);
        lane_prologue(o);
        o.l("if (warp == 0) {");
        store(o, "0");
        o.l("}");
        o.l("for (int c0 = 0; c0 < n_steps; c0 += " + S(CH) + ") {");
        o.ind++;
        // phase A: this warp's step group
        o.l("{ const int t0 = c0 + warp * " + S(U) + ";");
        o.ind++;
        o.l("const sde_u64 blk0 = ((sde_u64)t0 * " + S(NI) + "ull) / 8ull;");
        const int nblocks = (U * NI) / 8;
        for (int b = 0; b < nblocks; ++b) o.l("sde_u32 " + V("B", b) + "[16];");
        std::vector<bool> done(std::max(1, nblocks), false);
        for (int g = 0; g < U; ++g) {
            o.l("{ const int t = t0 + " + S(g) + ";");
            o.l("if (t < n_steps) {");
            o.ind++;
            step_header(o);
            uniforms(o, g, done);
            wiener(o);
            for (int k = 0; k < NI; ++k) {
                const std::string at = "((warp * " + S(U) + " + " + S(g) + ") * " + S(NI) + " + " + S(k) + ") * 32 + lane";
                if (u.token_kind[k] == IncKind::Dw) o.l("SW[" + at + "] = " + V("w", k) + ";");
                o.l("SU[" + at + "] = " + V("u", k) + ";");
            }
            o.ind--;
            o.l("} }");
        }
        o.ind--;
        o.l("}");
        o.l("__syncthreads();");
        // phase B: warp 0 steps its 32 paths through the chunk
        o.l("if (warp == 0) {");
        o.ind++;
        o.l("const int cend = min(" + S(CH) + ", n_steps - c0);");
        o.l("for (int s = 0; s < cend; ++s) {");
        o.ind++;
        o.l("const int t = c0 + s;");
        step_header(o);
        for (int k = 0; k < NI; ++k) {
            const std::string at = "(s * " + S(NI) + " + " + S(k) + ") * 32 + lane";
            if (u.token_kind[k] == IncKind::Dw) o.l("const double " + V("w", k) + " = SW[" + at + "];");
            o.l("const double " + V("u", k) + " = SU[" + at + "];");
            o.l("(void)" + V("u", k) + ";");
        }
        step(o);
        store(o, "t + 1");
        o.ind--;
        o.l("}");
        o.ind--;
        o.l("}");
        o.l("__syncthreads();");
        o.ind--;
        o.l("}");
        if (NPAY > 0) {
            o.l("double fs[" + S(NPAY) + "] = {}, fq[" + S(NPAY) + "] = {};");
            o.l("if (warp == 0) {");
            o.ind++;
            payoffs(o, NPAY);
            o.ind--;
            o.l("}");
            o.l("sde_block_reduce_store<" + S(NPAY) + ">(fs, fq, a.partials + (((sde_u64)rep * gridDim.x + blockIdx.x) * " +
                S(NPAY) + "u) * 4u);");
        }
        row = "threadIdx.x";
        cta = "blockDim.x";
        o.ind--;
        o.l("}");
        return o.s.str();
    }

    // Device function of one template for the batched kernel.
    std::string batch_template(const std::string& name, int K) {
        mode = Mode::Batch;
        Out o;
        o.l("static __device__ __forceinline__ void " + name +
            "(const sde_batch_inst& in, sde_u64 first, const sde_batch_args& a, double (&fs)[" + S(K) +
            "], double (&fq)[" + S(K) + "]) {");
        o.ind++;
        shared_prologue(o);
        for (int j = 0; j < ppt; ++j) {
            lane(j);
            lane_prologue(o);
        }
        lane(0);
        time_loop(o);
        payoffs(o, K);
        o.ind--;
        o.l("}");
        return o.s.str();
    }

    // ---- adjoint ---------------------------------------------------------
    std::string inc_store_name(int k) const {
        return u.token_kind[k] == IncKind::Dw ? V("w", k) : V("n", k);
    }

    // One step's increments at local slot s of the segment buffers (LI, and
    // LS for Runge-Kutta's sign) as named values.
    void adj_load_incs(Out& o, bool rk) const {
        for (int k = 0; k < NI; ++k) o.l("const " + R + " " + inc_store_name(k) + " = LI[s * " + S(NI) + " + " + S(k) + "];");
        if (rk) o.l("const " + R + " sk = LS[s];");
    }

    // Adjoint of one coefficient evaluation c(Zset, tvar) weighted by the
    // adjoint `w` of its value: the process adjoints `lset<q>` and the
    // parameter gradients GP<m> take w * dc/dX_q and w * dc/dtheta_m.
    void adj_coef(Out& o, const ExprP& c, const std::string& w, const std::string& zset, const std::string& tvar,
                  const std::string& lset) const {
        const int GP = (int)sp.grad_params.size();
        for (int q = 0; q < P; ++q)
            if (depends_on(c, VarKind::Process, q))
                o.l("  " + lset + S(q) + " += " + w + " * " + ex(derivative(c, VarKind::Process, q), zset, tvar) + ";");
        for (int m = 0; m < GP; ++m)
            if (depends_on(c, VarKind::Param, sp.grad_params[m]))
                o.l("  GP" + S(m) + " += " + w + " * " + ex(derivative(c, VarKind::Param, sp.grad_params[m]), zset, tvar) +
                    ";");
    }

    // Steps between checkpoints of the batched adjoint: E = ceil(sqrt(n)) at
    // run time, at most this many, so an instance takes at most
    // kBatchAdjMaxSteps = 64 * 64 steps and its checkpoints and one segment's
    // states and increments fit fixed per-thread arrays.
    static constexpr int kBatchAdjE = 64;

    std::string adjoint(const std::string& name) {
        mode = Mode::Forward;
        lane(0);
        const int KT = (int)(sp.payoffs.size() + sp.grad_params.size() + sp.grad_x0.size());
        Out o;
        o.l("extern \"C\" __global__ void __launch_bounds__(" + S(sp.block) + ") " + name + "(const sde_args a) {");
        o.ind++;
        o.l("const int lane = threadIdx.x & 31;");
        o.l("(void)lane;");
        o.l("const int rep = blockIdx.y;");
        o.l("const sde_u64 base = (sde_u64)blockIdx.x * blockDim.x;");
        o.l("const int n_steps = a.T - 1;");
        for (int k = 0; k < (int)u.params.size(); ++k)
            o.l("const " + R + " PR" + S(k) + " = (" + R + ")__ldg(&a.params[" + S(k) + "]);");
        if (xorm()) o.l("const sde_u32* mask_rep = a.masks ? a.masks + (sde_u64)rep * a.mask_stride : nullptr;");
        o.l("double fs[" + S(KT) + "] = {}, fq[" + S(KT) + "] = {};");
        adjoint_path(o, "fs");
        o.l("for (int k = 0; k < " + S(KT) + "; ++k) fq[k] = fs[k] * fs[k];");
        o.l("sde_block_reduce_store<" + S(KT) + ">(fs, fq, a.partials + (((sde_u64)rep * gridDim.x + blockIdx.x) * " +
            S(KT) + "u) * 4u);");
        o.ind--;
        o.l("}");
        return o.s.str();
    }

    // Device function of an adjoint template for the batched kernel: the
    // thread's PPT paths one after another (each path's forward pass and
    // reverse sweep), adding payoffs and gradients to fs / fq.  Uniform
    // steps of the instance; checkpoints every ceil(sqrt(steps)) steps in
    // per-thread arrays; increments drawn again in the reverse sweep.
    std::string batch_adjoint_template(const std::string& name, int K, int ppt_lanes) {
        mode = Mode::Batch;
        lane(0);
        const int KT = (int)(sp.payoffs.size() + sp.grad_params.size() + sp.grad_x0.size());
        Out o;
        o.l("static __device__ __forceinline__ void " + name +
            "(const sde_batch_inst& in, sde_u64 first0, const sde_batch_args& a, double (&fs)[" + S(K) +
            "], double (&fq)[" + S(K) + "]) {");
        o.ind++;
        shared_prologue(o);
        o.l("int E = 1;");
        o.l("while (E * E < n_steps) ++E;");
        o.l("for (int lj = 0; lj < " + S(ppt_lanes) + "; ++lj) {");
        o.ind++;
        o.l("const sde_u64 first = first0 + (sde_u64)lj * blockDim.x;");
        o.l("double pv[" + S(KT) + "] = {};");
        adjoint_path(o, "pv");
        o.l("for (int k = 0; k < " + S(KT) + "; ++k) { fs[k] += pv[k]; fq[k] += pv[k] * pv[k]; }");
        o.ind--;
        o.l("}");
        o.ind--;
        o.l("}");
        mode = Mode::Forward;
        return o.s.str();
    }

    // The step's time values in the reverse sweep.
    void adj_step_times(Out& o, bool rk) const {
        if (mode == Mode::Forward) {
            o.l("const " + R + " tc = " + T("times") + ";");
            o.l("const " + R + " dt = " + T("dts") + ";");
            if (rk) {
                o.l("const " + R + " tn = " + T("times", "t + 1") + ";");
                o.l("const " + R + " sdt = " + T("sqrt_dts") + ";");
            }
        } else {
            o.l("const " + R + " tc = (" + R + ")t * bdt;");
            o.l("const " + R + " dt = bdt;");
            if (rk) {
                o.l("const " + R + " tn = (" + R + ")(t + 1) * bdt;");
                o.l("const " + R + " sdt = bsdt;");
            }
        }
        o.l("(void)tc; (void)dt;");
        if (rk) o.l("(void)tn; (void)sdt;");
    }

    // One path's forward pass with checkpoints and reverse sweep; writes the
    // path's payoffs and gradients into out[] (zeros for an inactive lane).
    //
    // Pathwise adjoint of the step recursion, increments held fixed
    // (common random numbers; jump counts are piecewise constant in the
    // parameters).
    //
    // Euler-Maruyama: X' = X + sum_j c_j(t, X, theta) inc_j, so
    //   lambda_t = lambda_{t+1} + sum_p lambda_{t+1,p} sum_j dc_pj/dX inc_j,
    //   g_theta += sum_p lambda_{t+1,p} sum_j dc_pj/dtheta inc_j.
    //
    // Runge-Kutta (src/sim/runge_kutta.rs:17-97), sign sk = +-1 from the
    // step's uniform 0 held fixed:
    //   a_pj = c_pj(Z, t)          k1_p = sum_j a_pj inc_j
    //   pe_p = sum_{j in dW} a_pj sk sqrt(dt)
    //   B_p  = X_p + k1_p + pe_p   (the probe)
    //   k2_p = sum_j c_pj(B, t + dt) inc_j
    //   X'_p = X_p + (k1_p + k2_p) / 2
    // Z is the state the stage-1 coefficients see: X itself in textbook
    // semantics; in the reference's semantics the name->value cache, which
    // a step leaves at its probe B and the next step's stage 1 reads without
    // a refresh (src/func.rs:32-42: eval at an unchanged time keeps the
    // cache).  The cache is then part of the state: C' = B, C_0 = X_0,
    // checkpointed beside X, with its own adjoint LC.  Reverse:
    //   lB  = LC (reference semantics, else 0) + sum_pj (LA_p / 2) inc_j dc_pj/dB
    //   lk1 = LA / 2 + lB,  lpe = lB
    //   lZ  = sum_pj (lk1_p inc_j + [dW] lpe_p sk sqrt(dt)) dc_pj/dZ
    //   LA <- LA + lB (+ lZ in textbook semantics),  LC <- lZ.
    void adjoint_path(Out& o, const std::string& out) {
        const bool batch = mode == Mode::Batch;
        const bool rk = sp.scheme == SCHEME_RK;
        const bool refc = rk && sp.semantics == SEM_REFERENCE;
        const int PS = refc ? 2 * P : P;          // checkpointed values per path
        const int NS = rk ? NI + 1 : NI;          // stored values per step (+ RK's sign)
        const std::string E = batch ? "E" : S(sp.ckpt_every);
        const int EMAX = batch ? kBatchAdjE : sp.ckpt_every;
        const int K = (int)sp.payoffs.size();
        const int GP = (int)sp.grad_params.size(), GX = (int)sp.grad_x0.size();
        const std::string Zs = refc ? "Z" : "Y";  // stage-1 evaluation point in the reverse sweep
        o.l("{");
        o.ind++;
        lane_prologue(o);
        if (uses_chacha()) o.l("sde_u64 cblk = ~0ull; sde_u32 CB[16];");
        // checkpoints: [rep][n_ckpt][PS][path] in device memory for the plan
        // kernel; a per-thread array for the batched template
        std::function<std::string(const std::string&, int)> ck_at;
        if (batch) {
            o.l(R + " CKL[" + S(kBatchAdjE * PS) + "];");
            ck_at = [&](const std::string& seg, int v) { return "CKL[(" + seg + ") * " + S(PS) + " + " + S(v) + "]"; };
        } else {
            o.l(R + "* CK = (" + R + "*)a.ckpt;");
            o.l("const sde_u64 ckrow = (sde_u64)rep * a.n_ckpt;");
            ck_at = [&](const std::string& seg, int v) {
                return "CK[((ckrow + " + seg + ") * " + S(PS) + " + " + S(v) + ") * a.n_paths + i]";
            };
            // the forward pass's increments (and RK's sign),
            // [rep][t][slot][path], when the run holds a buffer for them: the
            // reverse sweep then reads them instead of drawing them again
            o.l(R + "* INC = (" + R + "*)a.inc;");
        }
        auto inc_at = [&](int k) {
            return "INC[(((sde_u64)rep * n_steps + t) * " + S(NS) + "ull + " + S(k) + "ull) * a.n_paths + i]";
        };
        // forward pass with checkpoints.  The plan kernel on the ChaCha8
        // streams runs it in groups of whole blocks (8 u64) with every block
        // word a compile-time index, as the forward kernels do (GBM adjoint
        // 2.055 -> 1.949 ms, Heston 4.171 -> 4.006 ms); the segment
        // recompute below reads the blocks by step (uniforms_ra).  The
        // batched template keeps the per-step form: the larger code slowed
        // the batch, which carries every template (157.9 -> 164.9 ms)
        const bool grouped = sp.rng == RNG_PSEUDO && NI > 0 && !batch;
        const int U = grouped ? group() : 1;
        std::vector<bool> done(std::max(1, (U * NI) / 8), false);
        auto fwd_step = [&](int g) {
            o.l("if (t % " + E + " == 0 && active) {");
            for (int p = 0; p < P; ++p) o.l("  " + ck_at("t / " + E, p) + " = X" + S(p) + ";");
            if (refc)
                for (int p = 0; p < P; ++p) o.l("  " + ck_at("t / " + E, P + p) + " = C" + S(p) + ";");
            o.l("}");
            step_header(o);
            if (grouped) uniforms(o, g, done);
            else uniforms_ra(o);
            wiener(o);
            if (rk) step(o);
            else step_reference(o);
            if (NS > 0 && !batch) {
                o.l("if (INC && active) {");
                for (int k = 0; k < NI; ++k) o.l("  " + inc_at(k) + " = " + inc_store_name(k) + ";");
                if (rk) o.l("  " + inc_at(NI) + " = sk;");
                o.l("}");
            }
        };
        if (grouped) {
            o.l("for (int t0 = 0; t0 < n_steps; t0 += " + S(U) + ") {");
            o.ind++;
            o.l("const sde_u64 blk0 = ((sde_u64)t0 * " + S(NI) + "ull) / 8ull;");
            for (int b = 0; b < (U * NI) / 8; ++b) o.l("sde_u32 " + V("B", b) + "[16];");
            for (int g = 0; g < U; ++g) {
                o.l("{ const int t = t0 + " + S(g) + ";");
                o.l("if (t < n_steps) {");
                o.ind++;
                fwd_step(g);
                o.ind--;
                o.l("} }");
            }
            o.ind--;
            o.l("}");
        } else {
            o.l("for (int t = 0; t < n_steps; ++t) {");
            o.ind++;
            fwd_step(0);
            o.ind--;
            o.l("}");
        }
        // payoffs and the terminal adjoint of payoff 0
        o.l("const " + R + " tT = " + (batch ? "(" + R + ")n_steps * bdt" : "(" + R + ")__ldg(&a.times[a.T - 1])") + ";");
        for (int k = 0; k < K; ++k)
            o.l(out + "[" + S(k) + "] = active ? (double)(" + ex(sp.payoffs[k], "X", "tT") + ") : 0.0;");
        for (int p = 0; p < P; ++p)
            o.l(R + " LA" + S(p) + " = " + ex(derivative(sp.payoffs[0], VarKind::Process, p), "X", "tT") + ";");
        if (refc)
            for (int p = 0; p < P; ++p) o.l(R + " LC" + S(p) + " = " + L(0.0) + ";");
        for (int m = 0; m < GP; ++m)
            o.l(R + " GP" + S(m) + " = " + ex(derivative(sp.payoffs[0], VarKind::Param, sp.grad_params[m]), "X", "tT") + ";");
        // reverse sweep over segments, recomputing each from its checkpoint
        o.l(R + " LX[" + S(EMAX * std::max(1, P)) + "];");
        if (refc) o.l(R + " LZ[" + S(EMAX * std::max(1, P)) + "];");
        o.l(R + " LI[" + S(EMAX * std::max(1, NI)) + "];");
        if (rk) o.l(R + " LS[" + S(EMAX) + "];");
        o.l("const int nseg = (n_steps + " + E + " - 1) / " + E + ";");
        o.l("for (int seg = nseg - 1; seg >= 0; --seg) {");
        o.ind++;
        o.l("const int s0 = seg * " + E + ";");
        o.l("const int s1 = min(s0 + " + E + ", n_steps);");
        for (int p = 0; p < P; ++p) o.l("X" + S(p) + " = active ? " + ck_at("seg", p) + " : X" + S(p) + ";");
        if (refc)
            for (int p = 0; p < P; ++p) o.l("C" + S(p) + " = active ? " + ck_at("seg", P + p) + " : C" + S(p) + ";");
        o.l("for (int t = s0; t < s1; ++t) {");
        o.ind++;
        o.l("const int s = t - s0;");
        for (int p = 0; p < P; ++p) o.l("LX[s * " + S(P) + " + " + S(p) + "] = X" + S(p) + ";");
        if (refc)
            for (int p = 0; p < P; ++p) o.l("LZ[s * " + S(P) + " + " + S(p) + "] = C" + S(p) + ";");
        step_header(o);
        // the step's increments: stored by the forward pass, or drawn again
        // (jump counts read the cache: the state itself but in reference RK)
        if (!refc)
            for (int p : u.levy) o.l("C" + S(p) + " = X" + S(p) + ";");
        if (NS > 0) {
            o.l(R + " IV[" + S(NS) + "];");
            if (!batch) {
                o.l("if (INC) {");
                // (issuing a whole segment's loads ahead into LI was measured:
                // slower, 2.23 against 2.08 ms for the GBM adjoint)
                for (int k = 0; k < NS; ++k) o.l("  IV[" + S(k) + "] = active ? " + inc_at(k) + " : " + L(0.0) + ";");
                o.l("} else {");
            } else {
                o.l("{");
            }
            o.ind++;
            uniforms_ra(o);
            wiener(o);
            poisson(o, "C", "tc");
            for (int k = 0; k < NI; ++k) o.l("IV[" + S(k) + "] = " + inc_store_name(k) + ";");
            if (rk) o.l("IV[" + S(NI) + "] = " + sk_expr() + ";");
            o.ind--;
            o.l("}");
            for (int k = 0; k < NI; ++k) o.l("const " + R + " " + inc_store_name(k) + " = IV[" + S(k) + "];");
            if (rk) o.l("const " + R + " sk = IV[" + S(NI) + "];");
        }
        for (int k = 0; k < NI; ++k) o.l("LI[s * " + S(NI) + " + " + S(k) + "] = " + inc_store_name(k) + ";");
        if (rk) {
            o.l("LS[s] = sk;");
            // stage 1 at the cache (reference) or the state (textbook), the
            // probe, stage 2 at the probe: the forward step, term by term
            const std::string zc = refc ? "C" : "X";
            for (int p : u.levy) {
                const auto& terms = u.procs[p].terms;
                o.l(R + " k1_" + S(p) + " = " + L(0.0) + ", pe" + S(p) + " = " + L(0.0) + ";");
                for (size_t j = 0; j < terms.size(); ++j) {
                    const std::string a = "a" + S(p) + "_" + S((int)j);
                    o.l("{ const " + R + " " + a + " = " + ex(terms[j].coef, zc, "tc") + ";");
                    o.l("  k1_" + S(p) + " = k1_" + S(p) + " + " + a + " * " + inc(terms[j]) + ";");
                    if (terms[j].kind == IncKind::Dw) o.l("  pe" + S(p) + " = pe" + S(p) + " + " + a + " * sk * sdt;");
                    o.l("}");
                }
            }
            for (int p : u.levy) o.l("const " + R + " B" + S(p) + " = X" + S(p) + " + k1_" + S(p) + " + pe" + S(p) + ";");
            for (int p : u.levy) {
                const auto& terms = u.procs[p].terms;
                o.l(R + " k2_" + S(p) + " = " + L(0.0) + ";");
                for (size_t j = 0; j < terms.size(); ++j)
                    o.l("k2_" + S(p) + " = k2_" + S(p) + " + " + ex(terms[j].coef, "B", "tn") + " * " + inc(terms[j]) + ";");
            }
            for (int p : u.levy) o.l("X" + S(p) + " = X" + S(p) + " + " + L(0.5) + " * (k1_" + S(p) + " + k2_" + S(p) + ");");
            if (refc)
                for (int p : u.levy) o.l("C" + S(p) + " = B" + S(p) + ";");
        } else {
            for (int p : u.levy) {
                o.l(R + " N" + S(p) + " = X" + S(p) + ";");
                for (const auto& tm : u.procs[p].terms)
                    o.l("N" + S(p) + " = N" + S(p) + " + " + ex(tm.coef, "C", "tc") + " * " + inc(tm) + ";");
            }
            for (int p : u.levy) o.l("X" + S(p) + " = N" + S(p) + ";");
        }
        o.ind--;
        o.l("}");
        o.l("for (int t = s1 - 1; t >= s0; --t) {");
        o.ind++;
        o.l("const int s = t - s0;");
        adj_step_times(o, rk);
        for (int p = 0; p < P; ++p) o.l("const " + R + " Y" + S(p) + " = LX[s * " + S(P) + " + " + S(p) + "];");
        adj_load_incs(o, rk);
        if (!rk) {
            for (int q = 0; q < P; ++q) o.l(R + " LN" + S(q) + " = " + L(0.0) + ";");
            for (int p : u.levy) {
                const auto& terms = u.procs[p].terms;
                for (size_t j = 0; j < terms.size(); ++j) {
                    const std::string li = "li" + S(p) + "_" + S((int)j);
                    o.l("{ const " + R + " " + li + " = LA" + S(p) + " * " + inc(terms[j]) + ";");
                    adj_coef(o, terms[j].coef, li, "Y", "tc", "LN");
                    o.l("}");
                }
            }
            for (int q = 0; q < P; ++q) o.l("LA" + S(q) + " += LN" + S(q) + ";");
        } else {
            if (refc)
                for (int p = 0; p < P; ++p) o.l("const " + R + " Z" + S(p) + " = LZ[s * " + S(P) + " + " + S(p) + "];");
            // the probe again, from the stage-1 coefficients
            for (int p = 0; p < P; ++p) {
                if (!u.procs[p].levy) {
                    o.l("const " + R + " B" + S(p) + " = Y" + S(p) + ";");
                    continue;
                }
                const auto& terms = u.procs[p].terms;
                o.l(R + " k1_" + S(p) + " = " + L(0.0) + ", pe" + S(p) + " = " + L(0.0) + ";");
                for (size_t j = 0; j < terms.size(); ++j) {
                    const std::string a = "a" + S(p) + "_" + S((int)j);
                    o.l("{ const " + R + " " + a + " = " + ex(terms[j].coef, Zs, "tc") + ";");
                    o.l("  k1_" + S(p) + " = k1_" + S(p) + " + " + a + " * " + inc(terms[j]) + ";");
                    if (terms[j].kind == IncKind::Dw) o.l("  pe" + S(p) + " = pe" + S(p) + " + " + a + " * sk * sdt;");
                    o.l("}");
                }
                o.l("const " + R + " B" + S(p) + " = Y" + S(p) + " + k1_" + S(p) + " + pe" + S(p) + ";");
            }
            // stage 2: k2_p = sum_j c_pj(B, tn) inc_j, weighted by LA_p / 2
            for (int q = 0; q < P; ++q) o.l(R + " lB" + S(q) + " = " + (refc ? "LC" + S(q) : L(0.0)) + ";");
            for (int p : u.levy) {
                const auto& terms = u.procs[p].terms;
                for (size_t j = 0; j < terms.size(); ++j) {
                    const std::string w = "w2_" + S(p) + "_" + S((int)j);
                    o.l("{ const " + R + " " + w + " = " + L(0.5) + " * LA" + S(p) + " * " + inc(terms[j]) + ";");
                    adj_coef(o, terms[j].coef, w, "B", "tn", "lB");
                    o.l("}");
                }
            }
            // stage 1: a_pj = c_pj(Z, tc) feeds k1 and the perturbation
            for (int q = 0; q < P; ++q) o.l(R + " lZ" + S(q) + " = " + L(0.0) + ";");
            for (int p : u.levy) {
                const auto& terms = u.procs[p].terms;
                o.l("const " + R + " lk1_" + S(p) + " = " + L(0.5) + " * LA" + S(p) + " + lB" + S(p) + ";");
                for (size_t j = 0; j < terms.size(); ++j) {
                    const std::string w = "w1_" + S(p) + "_" + S((int)j);
                    std::string wv = "lk1_" + S(p) + " * " + inc(terms[j]);
                    if (terms[j].kind == IncKind::Dw) wv += " + lB" + S(p) + " * sk * sdt";
                    o.l("{ const " + R + " " + w + " = " + wv + ";");
                    adj_coef(o, terms[j].coef, w, Zs, "tc", "lZ");
                    o.l("}");
                }
            }
            for (int q = 0; q < P; ++q)
                o.l("LA" + S(q) + " = LA" + S(q) + " + lB" + S(q) + (refc ? "" : " + lZ" + S(q)) + ";");
            if (refc)
                for (int q = 0; q < P; ++q) o.l("LC" + S(q) + " = lZ" + S(q) + ";");
        }
        o.ind--;
        o.l("}");
        o.ind--;
        o.l("}");
        for (int m = 0; m < GP; ++m) o.l(out + "[" + S(K + m) + "] = active ? (double)GP" + S(m) + " : 0.0;");
        // X0 feeds the state and, in reference RK, the cache C_0 = X_0
        for (int x = 0; x < GX; ++x) {
            const std::string q = S(sp.grad_x0[x]);
            o.l(out + "[" + S(K + GP + x) + "] = active ? (double)(LA" + q + (refc ? " + LC" + q : "") + ") : 0.0;");
        }
        o.ind--;
        o.l("}");
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
    if (s.icdf) r += "_acc";
    r += s.rng == RNG_PSEUDO ? "_pseudo" : (s.scramble == SCRAMBLE_XOR ? "_sobolxor" : "_sobolshift");
    if (s.ppt > 1) r += "_ppt" + std::to_string(s.ppt);
    if (s.ugrid) r += "_ug";
    return r;
}

MmaShape mma_shape(const Universe& u, const KernelSpec& s) {
    MmaShape m;
    if (s.precision != PREC_FP32 || s.scheme != SCHEME_EULER || s.adjoint || s.ppt != 1 || !u.alg.empty()) return m;
    std::vector<std::vector<double>> K;
    if (!diffusion_matrix(u, K)) return m;
    const int P = u.n_processes(), NI = u.n_stochastic();
    // two or four threads per path for wide universes whose drifts are
    // linear in their own process (each thread then needs only its part of
    // the state)
    bool two = s.tensor_cores == 1 && P >= 32 && NI >= 32;
    for (int p = 0; two && p < P; ++p) {
        double c = 0.0;
        two = linear_drift_of(u, p, c);
    }
    for (int k = 0; two && k < NI; ++k) two = u.token_kind[k] == IncKind::Dw;
    // (the kernel takes four too -- 512 threads, 64 registers, 32 warps per
    // SM -- but on the 64-dim basket that measured 31.1 ms against 27.8 ms
    // for two)
    m.split = two ? 2 : 1;
    const int nq = 16 * m.split;                            // each half's columns: multiples of 16
    m.npad = std::max(nq, (P + nq - 1) / nq * nq);          // M = 128 takes N = 16..256 in steps of 16
    m.kpad = std::max(nq, (NI + nq - 1) / nq * nq);         // K = 16 per FP16 MMA
    if (m.npad > 256) return m;
    m.ncols = 32;
    while (m.ncols < m.npad) m.ncols *= 2;
    const int operands = 2 * 128 * m.kpad * 2 + 2 * m.npad * m.kpad * 2;
    if (m.split > 1 && 128 * P * 4 > operands) {             // the payoff exchange reuses the operand area
        m.split = 1;
        return mma_shape(u, [&] { KernelSpec t = s; t.tensor_cores = 2; return t; }());
    }
    int need = operands + 64;                                // + four mbarriers and the TMEM address
    if (s.rng == RNG_SOBOL && s.scramble == SCRAMBLE_XOR && NI % 4 == 0) {
        // the LO words of a step are NI * 128 contiguous bytes of the table:
        // two step buffers, filled by bulk copies one step ahead
        m.lo_off = (need + 127) / 128 * 128;
        m.lo_step_bytes = NI * 128;
        need = m.lo_off + 2 * m.lo_step_bytes;
    }
    // at most 512 / ncols CTAs of an SM can hold tensor memory at once: ask
    // for enough shared memory (228 KB per SM) that no more are resident
    const int floor_bytes = 233472 / (512 / m.ncols + 1) + 1;
    m.smem_bytes = std::max(need, floor_bytes);
    if (m.smem_bytes > 227 * 1024) return m;
    // CTAs per SM that the shared memory allows (1 KB reserved and 1 KB of
    // static reduction scratch each), capped by the register budget of
    // __launch_bounds__: 128 registers a thread (one thread per path), 85
    // (two, 3 CTAs of 256) or 64 (four, 2 CTAs of 512)
    const int reg_cap = m.split == 1 ? 4 : m.split == 2 ? 3 : 2;
    m.min_blocks = std::max(1, std::min(reg_cap, 233472 / (m.smem_bytes + 2048)));
    m.eligible = true;
    return m;
}

std::string forward_kernel_name(const KernelSpec& s) { return "sde_step_" + tag(s) + (s.tensor_cores ? "_tc" : ""); }
std::string adjoint_kernel_name(const KernelSpec& s) { return "sde_adjoint_" + tag(s); }
std::string chunked_kernel_name(const KernelSpec& s) { return "sde_step_" + tag(s) + "_chunked"; }
bool has_chunked_kernel(const Universe& u, const KernelSpec& s) { return Gen::chunked_eligible(u, s); }
bool has_wide_kernel(const Universe& u, const KernelSpec& s) {
    return s.wide && s.precision == PREC_FP32 && s.rng == RNG_SOBOL && s.scramble == SCRAMBLE_XOR && !s.adjoint &&
           !s.tensor_cores && s.ppt == 1 && u.n_stochastic() > 0;
}
KernelSpec wide_spec(const KernelSpec& s) {
    KernelSpec w = s;
    w.ppt = 2;
    w.block = 128;
    w.wide = false;
    return w;
}
KernelSpec wide_ugrid_spec(const KernelSpec& s) {
    KernelSpec w = wide_spec(s);
    w.ugrid = true;
    return w;
}

std::string generate_source(const Universe& u, const KernelSpec& s) {
    Gen g(u, s);
    std::string src;
    if (s.tensor_cores) {
        const MmaShape m = mma_shape(u, s);
        std::vector<std::vector<double>> K;
        if (!m.eligible || !diffusion_matrix(u, K) || s.block != 128 * m.split)
            throw std::runtime_error("the universe is not eligible for the tensor-core lowering");
        g.mma = &m;
        src += g.forward_mma(forward_kernel_name(s), K);
        return src;
    }
    src += g.forward(forward_kernel_name(s));
    if (Gen::chunked_eligible(u, s)) {
        Gen gc(u, s);
        src += "\n" + gc.forward_chunked(chunked_kernel_name(s));
    }
    if (has_wide_kernel(u, s)) {
        const KernelSpec w = wide_spec(s), wu = wide_ugrid_spec(s);
        Gen gw(u, w), gu(u, wu);
        src += "\n" + gw.forward(forward_kernel_name(w));
        src += "\n" + gu.forward(forward_kernel_name(wu));
    }
    if (s.adjoint) {
        KernelSpec s1 = s;
        s1.ppt = 1;
        Gen ga(u, s1);
        src += "\n" + ga.adjoint(adjoint_kernel_name(s));
    }
    return src;
}

std::string batch_kernel_name(int block, int ppt) {
    return "sde_batch_b" + std::to_string(block) + "_p" + std::to_string(ppt);
}

std::string generate_batch_source(const std::vector<const Universe*>& us, const std::vector<KernelSpec>& specs,
                                  const std::vector<std::pair<int, int>>& variants, int K) {
    std::string src;
    std::vector<int> ppts;
    for (const auto& v : variants)
        if (std::find(ppts.begin(), ppts.end(), v.second) == ppts.end()) ppts.push_back(v.second);
    for (int ppt : ppts)
        for (size_t t = 0; t < us.size(); ++t) {
            KernelSpec s = specs[t];
            s.ppt = s.adjoint ? 1 : ppt;
            s.store_output = false;
            Gen g(*us[t], s);
            const std::string nm = "sde_tmpl" + std::to_string(t) + "_p" + std::to_string(ppt);
            src += (s.adjoint ? g.batch_adjoint_template(nm, K, ppt) : g.batch_template(nm, K)) + "\n";
        }
    for (const auto& v : variants) {
        const int block = v.first, ppt = v.second;
        Out o;
        o.l("extern \"C\" __global__ void __launch_bounds__(" + S(block) + ") " + batch_kernel_name(block, ppt) +
            "(const sde_batch_args a) {");
        o.ind++;
        o.l("__shared__ int s_item;");
        o.l("for (;;) {");
        o.ind++;
        o.l("if (threadIdx.x == 0) s_item = (int)atomicAdd(a.counter, 1u);");
        o.l("__syncthreads();");
        o.l("const int item = s_item;");
        o.l("if (item >= a.n_items) break;");
        o.l("const sde_batch_item it = a.items[item];");
        o.l("const sde_batch_inst in = a.inst[it.inst];");
        o.l("double fs[" + S(K) + "] = {}, fq[" + S(K) + "] = {};");
        o.l("switch (in.tmpl) {");
        for (size_t t = 0; t < us.size(); ++t)
            o.l("case " + S((int)t) + ": sde_tmpl" + S((int)t) + "_p" + S(ppt) + "(in, it.first_path, a, fs, fq); break;");
        o.l("default: break;");
        o.l("}");
        o.l("sde_block_reduce_store<" + S(K) + ">(fs, fq, a.item_partials + (sde_u64)item * " + S(K) + "u * 4u);");
        o.ind--;
        o.l("}");
        o.ind--;
        o.l("}");
        src += o.s.str() + "\n";
    }
    return src;
}

}  // namespace sde
