// codegen.h -- lowering of a parsed process universe to sm_103a device code.
#pragma once

#include <string>
#include <vector>

#include "frontend.h"

namespace sde {

enum Scheme { SCHEME_EULER = 0, SCHEME_RK = 1 };
enum RngKind { RNG_PSEUDO = 0, RNG_SOBOL = 1 };
enum Scramble { SCRAMBLE_SHIFT = 0, SCRAMBLE_XOR = 1 };
enum Precision { PREC_FP64 = 0, PREC_FP32 = 1 };
enum Semantics { SEM_REFERENCE = 0, SEM_TEXTBOOK = 1 };

struct KernelSpec {
    int scheme = SCHEME_EULER;
    int rng = RNG_PSEUDO;
    int scramble = SCRAMBLE_SHIFT;
    int precision = PREC_FP64;
    int semantics = SEM_REFERENCE;
    bool store_output = true;           // filtration slices selected by out_tidx
    std::vector<ExprP> payoffs;         // resolved estimator expressions
    int block = 256;
    int ppt = 1;                        // paths per thread (independent chains)
    int icdf = 0;                       // 0: AS 26.2.23 (reference), 1: accurate
    int tensor_cores = 0;               // 1: correlated diffusions on tcgen05 when eligible
                                        // 2: the same with one thread per path always
    // adjoint: parameters and initial values to differentiate
    bool adjoint = false;
    std::vector<int> grad_params;       // parameter indices
    std::vector<int> grad_x0;           // process indices
    int ckpt_every = 19;                // steps between adjoint checkpoints
    bool wide = false;                  // also build the two-paths-per-thread kernel
                                        // (where has_wide_kernel allows it)
    bool ugrid = false;                 // FP32 dt and sqrt(dt) from the launch
                                        // arguments (a grid of equal steps)
};

// Tensor-core lowering of correlated diffusions: eligible when the plan is
// FP32 Euler, forward, one path per thread, without algebraic processes,
// and every dW coefficient is a constant times its own process.  Then the
// per-step increments are D = W K^T (paths x processes) on tcgen05.
struct MmaShape {
    bool eligible = false;
    int npad = 0;         // processes padded to a multiple of 16 (MMA N)
    int kpad = 0;         // Wiener indices padded to a multiple of 16 (MMA K)
    int ncols = 0;        // tensor-memory columns allocated (power of 2 >= 32)
    int smem_bytes = 0;   // dynamic shared memory of the kernel
    int min_blocks = 1;   // CTAs per SM the kernel is register-budgeted for
    int split = 1;        // threads per path (2: each steps half the processes)
    int lo_off = 0;       // XOR Sobol, NI % 4 == 0: shared-memory offset of the two
                          // step buffers of LO words (bulk-copied a step ahead); 0: none
    int lo_step_bytes = 0;  // one step's LO words (NI * 128 bytes)
};
MmaShape mma_shape(const Universe& u, const KernelSpec& s);

// Name of the forward kernel in the generated source.
std::string forward_kernel_name(const KernelSpec& s);
std::string adjoint_kernel_name(const KernelSpec& s);

// FP64 forward plans on pseudo / shifted-Sobol streams also get a chunked
// kernel for runs with few paths: a CTA of 8 warps per 32 paths draws a
// chunk of steps' increments in parallel, then warp 0 steps through it.
bool has_chunked_kernel(const Universe& u, const KernelSpec& s);
std::string chunked_kernel_name(const KernelSpec& s);

// FP32 forward plans on XOR-scrambled Sobol with spec.wide set also carry
// a kernel that steps two paths per thread in CTAs of 128 threads, for runs
// with many paths; wide_spec is its specification.
// It has a twin for grids whose FP32 steps are all equal, which takes dt and
// sqrt(dt) from the launch arguments instead of loading them each step.
bool has_wide_kernel(const Universe& u, const KernelSpec& s);
KernelSpec wide_spec(const KernelSpec& s);
KernelSpec wide_ugrid_spec(const KernelSpec& s);

// CUDA C source of the kernels for one universe (without the runtime
// header, which the JIT prepends).
std::string generate_source(const Universe& u, const KernelSpec& s);

// Expression emitter, exposed for tests of the lowering.
std::string emit_expression(const ExprP& e, bool fp32);

// Batched instances: one device function per (template, paths-per-thread)
// and one persistent work-queue kernel per (block, paths-per-thread)
// variant, all estimating K payoff columns.
std::string batch_kernel_name(int block, int ppt);
std::string generate_batch_source(const std::vector<const Universe*>& templates,
                                  const std::vector<KernelSpec>& specs,
                                  const std::vector<std::pair<int, int>>& variants, int K);

}  // namespace sde
