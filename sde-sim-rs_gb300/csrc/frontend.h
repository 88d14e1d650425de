// frontend.h -- equation and coefficient-expression front end.
//
// Accepts the sde-sim-rs equation grammar (src/proc/util.rs:52-166) and the
// fasteval 0.2.4 expression grammar its coefficients use (src/func.rs:18-30),
// and produces the setup-time IR that codegen lowers to device code.
#pragma once

#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace sde {

struct ParseError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

enum class Op {
    Const, Var, Neg, Not, Add, Sub, Mul, Div, Mod, Pow,
    Eq, Ne, Lt, Le, Gt, Ge, And, Or, Call
};

enum class Fn {
    Min, Max, Abs, Sign, Int, Ceil, Floor, Round, Log, E, Pi, Sin, Cos, Tan,
    Asin, Acos, Atan, Sinh, Cosh, Tanh, Asinh, Acosh, Atanh, Sqrt, Exp,
    // internal: used only by symbolic derivatives
    Step,     // 1 if x > 0 else 0
    Mul0,     // a * b, but 0 when b == 0 (chain rule: f'(g) may be infinite
              // exactly where g' vanishes, e.g. d sqrt(max(v,0)) at v <= 0)
    Sel,      // c > 0 ? a : b
};

enum class VarKind { Unresolved, Time, Process, Param };

struct Expr;
using ExprP = std::shared_ptr<const Expr>;

struct Expr {
    Op op = Op::Const;
    double value = 0.0;
    Fn fn = Fn::Min;
    std::string name;
    VarKind vk = VarKind::Unresolved;
    int idx = -1;
    std::vector<ExprP> args;
};

ExprP parse_expression(const std::string& text);   // throws ParseError

// Builders (with light constant folding, used by the derivative code)
ExprP mk_const(double v);
ExprP mk_var(VarKind k, int idx, const std::string& name);
ExprP mk_un(Op op, ExprP a);
ExprP mk_bin(Op op, ExprP a, ExprP b);
ExprP mk_call(Fn fn, std::vector<ExprP> args);
bool is_const(const ExprP& e, double v);

// Symbolic derivative d e / d var(kind, idx) (pathwise: comparisons, int,
// floor, ceil, round and sign have derivative 0; max/min select the branch).
ExprP derivative(const ExprP& e, VarKind kind, int idx);
bool depends_on(const ExprP& e, VarKind kind, int idx);

enum class IncKind { Dt = 0, Dw = 1, Dn = 2 };

struct Term {
    ExprP coef;
    IncKind kind = IncKind::Dt;
    int sidx = -1;          // stochastic index (dW/dN), order of first appearance
    ExprP lambda;           // dN intensity
};

struct Process {
    std::string name;
    bool levy = true;
    std::vector<Term> terms;
    ExprP alg;
};

struct Universe {
    std::vector<Process> procs;
    std::vector<std::string> tokens;     // stochastic registry, index -> token
    std::vector<IncKind> token_kind;
    std::vector<std::string> params;
    std::vector<int> levy, alg;          // process indices by kind, in order

    int n_processes() const { return (int)procs.size(); }
    int n_stochastic() const { return (int)tokens.size(); }
    int process_index(const std::string& name) const;  // registry: last wins
    // Resolve variable names of an expression against this universe.
    ExprP resolve(const ExprP& e) const;
};

// parse_equations (src/proc/util.rs:52-66) + ProcessUniverse::new
// (src/proc/mod.rs:70-89).  Names are resolved against processes, then "t",
// then the declared parameters.
Universe parse_universe(const std::vector<std::string>& equations,
                        const std::vector<std::string>& params);

}  // namespace sde
