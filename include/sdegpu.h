/*
 * sdegpu.h -- C ABI of libsdegpu.so, the GB300 (sm_103a) engine for the
 * sde-sim-rs path-simulation hot path.
 *
 * The drop-in boundary is the reference's whole simulate call: parse the
 * equation strings once, then advance every scenario through every time
 * step on the GPU and return the filtration.  The per-step Rust functions
 * (euler_iteration, runge_kutta_iteration) are far too fine-grained to cross
 * an FFI or device boundary, so they have no entry point of their own; they
 * are lowered into the step kernel.
 *
 * Conventions
 *  - Every function returns an int status (SDE_OK = 0); on failure the
 *    message is kept per thread and read with sde_last_error().  No C++
 *    exception and no abort crosses the ABI.
 *  - Plain pointers and sizes only.  "host" buffers are caller-allocated
 *    host memory; device buffers are cudaMalloc'ed memory of the current
 *    device; stream arguments are cudaStream_t values (NULL = legacy default
 *    stream).
 *  - Objects (sde_plan, sde_result) are engine-owned and released with the
 *    matching *_destroy call.  A plan may be run from several threads; a
 *    result belongs to one thread at a time.
 */
#ifndef SDEGPU_H
#define SDEGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SDE_ABI_VERSION 1

typedef enum sde_status {
    SDE_OK = 0,
    SDE_ERR_PARSE = 1,        /* equation/expression grammar (reference: Err(String)) */
    SDE_ERR_INVALID = 2,      /* bad argument (sizes, unknown scheme, unsorted times) */
    SDE_ERR_COMPILE = 3,      /* NVRTC lowering failed                                */
    SDE_ERR_CUDA = 4,         /* CUDA runtime error                                   */
    SDE_ERR_OOM = 5,          /* device or host allocation failed                     */
    SDE_ERR_RNG_INDEX = 6,    /* reference panics "RNG Index .. out of bounds"        */
    SDE_ERR_UNSUPPORTED = 7,  /* combination not built (e.g. > 21201 Sobol dims)      */
    SDE_ERR_DEVICE = 8        /* a kernel reported a failure through its status word  */
} sde_status;

enum { SDE_SCHEME_EULER = 0, SDE_SCHEME_RK = 1 };
enum { SDE_RNG_PSEUDO = 0, SDE_RNG_SOBOL = 1 };
/* SHIFT: the reference's per-scenario random shift of Sobol point s+5.
 * XOR:   one random XOR mask per (replicate, dimension), points 0..N-1.      */
enum { SDE_SCRAMBLE_SHIFT = 0, SDE_SCRAMBLE_XOR = 1 };
enum { SDE_FP64 = 0, SDE_FP32 = 1 };
/* REFERENCE: coefficients see the reference's name->value cache exactly as
 *            src/func.rs:32-42 refreshes it (stale probe state in RK).
 * TEXTBOOK:  every evaluation sees the state it names.                       */
enum { SDE_SEM_REFERENCE = 0, SDE_SEM_TEXTBOOK = 1 };
/* FULL: all time points; CHECKPOINTS: the time indices given at run time;
 * TERMINAL: the last time point only; NONE: estimators only.                 */
enum { SDE_OUT_FULL = 0, SDE_OUT_CHECKPOINTS = 1, SDE_OUT_TERMINAL = 2, SDE_OUT_NONE = 3 };
/* layouts for sde_result_copy_values */
enum { SDE_LAYOUT_REFERENCE = 0,  /* [replicate][path][time][process]  */
       SDE_LAYOUT_DEVICE = 1 };   /* [replicate][time][process][path]  */

typedef struct sde_plan sde_plan;
typedef struct sde_result sde_result;

typedef struct sde_options {
    uint32_t struct_size;   /* sizeof(sde_options), set by sde_options_init */
    int32_t scheme;         /* SDE_SCHEME_*        default EULER           */
    int32_t rng;            /* SDE_RNG_*           default PSEUDO          */
    int32_t scramble;       /* SDE_SCRAMBLE_*      default SHIFT           */
    int32_t precision;      /* SDE_FP64 | SDE_FP32 default FP64            */
    int32_t semantics;      /* SDE_SEM_*           default REFERENCE       */
    int32_t output;         /* SDE_OUT_*           default FULL            */
    int32_t block_size;     /* threads per block, 0 = 256                  */
    int32_t ckpt_every;     /* adjoint plans: steps between checkpoints,
                               0 = 19                                      */
    int32_t paths_per_thread; /* independent paths a thread steps in
                               lockstep (1, 2 or 4); 0 = automatic: 1, or
                               for FP32 XOR-Sobol plans without a set
                               block_size, 2 in CTAs of 128 threads on runs
                               of about 0.6M paths and more (same results
                               bit for bit)                                */
    int32_t icdf;           /* SDE_ICDF_*          default AS26            */
    int32_t tensor_cores;   /* SDE_TC_*            default OFF             */
    int32_t adjoint_recompute; /* adjoint plans: 1 = draw the increments
                               again in the reverse sweep; 0 (default) =
                               keep the forward pass's increments in device
                               memory when they fit in a quarter of the
                               free memory (else draw them again)          */
    int32_t chunked;        /* SDE_CHUNKED_*       default AUTO            */
    int32_t reserved[2];
} sde_options;

/* FP64 forward plans on pseudo or shifted-Sobol streams with 1, 2, 4 or 8
 * stochastic indices also carry a chunked kernel for runs with few paths
 * (the reference's 10,000): a CTA of 8 warps owns 32 paths, draws a chunk
 * of steps' increments with all 8 warps, then steps the paths through it
 * with one.  Same arithmetic, same results bit for bit.  AUTO uses it when
 * the one-thread-per-path kernel would give fewer than 4 warps per SM.     */
enum { SDE_CHUNKED_AUTO = 0, SDE_CHUNKED_ON = 1, SDE_CHUNKED_OFF = 2 };

/* TC_ON: when the plan is FP32 Euler-Maruyama, forward, one path per
 * thread, without algebraic processes, and every dW coefficient is a
 * constant times its own process (correlated GBM baskets), the step's
 * Wiener terms run as one tcgen05 product per 128 paths (three FP16
 * products of hi / lo splits, FP32 accumulation, about FP32 accuracy) and
 * 128 paths make one CTA.  With at least 32 processes and 32 Wiener
 * indices, only dt and dW terms, and drifts that are constant * own
 * process, two threads share a path (each draws half its normals and
 * steps half its processes; 256 threads per CTA).  TC_ON_ROW keeps one
 * thread per path.  Other plans keep the CUDA-core kernel;
 * sde_plan_tensor_cores tells which was built.
 * No counterpart in the reference (its coefficient loop is
 * src/sim/euler.rs:17-33).                                                */
enum { SDE_TC_OFF = 0, SDE_TC_ON = 1, SDE_TC_ON_ROW = 2 };

/* AS26: the reference's Abramowitz-Stegun 26.2.23 normal (|err| ~ 4.5e-4).
 * ACCURATE: that value refined by Halley steps on Phi through erfc of the
 *           exact tail probability (FP64: two steps, FP32: one).          */
enum { SDE_ICDF_AS26 = 0, SDE_ICDF_ACCURATE = 1 };

typedef struct sde_run_args {
    uint32_t struct_size;       /* sizeof(sde_run_args), set by sde_run_args_init */
    const double* times;        /* host [n_times], strictly increasing            */
    int32_t n_times;
    const double* x0;           /* host [n_x0] time-0 row by process index;
                                   missing processes start at 0.0              */
    int32_t n_x0;
    const double* params;       /* host [n_params] values of the named params   */
    int32_t n_params;
    uint64_t n_paths;           /* paths per replicate                          */
    int32_t n_replicates;       /* >= 1                                         */
    uint64_t seed;              /* scenario s uses ChaCha8 seed_from_u64(seed+s);
                                   XOR replicate r uses masks from seed + r     */
    uint64_t path_offset;       /* scenario index of path 0 (default 0)         */
    const int32_t* checkpoints; /* host time indices for SDE_OUT_CHECKPOINTS    */
    int32_t n_checkpoints;
    void* stream;               /* cudaStream_t or NULL                         */
    void* device_out;           /* optional caller-owned device buffer for the
                                   filtration (device layout); NULL = engine    */
    uint64_t device_out_bytes;
} sde_run_args;

/* ---- version / errors ------------------------------------------------- */
int32_t sde_abi_version(void);
/* Copies the calling thread's last error message (NUL-terminated). */
int sde_last_error(char* buf, size_t buf_len);

void sde_options_init(sde_options* opts);
void sde_run_args_init(sde_run_args* args);

/* ---- plans -------------------------------------------------------------
 * Replaces sde_sim_rs::proc::util::parse_equations
 *   (src/proc/util.rs:52-55, -> ProcessUniverse src/proc/mod.rs:70-89)
 * and the per-call fasteval compilation of every coefficient
 *   (src/func.rs:18-30): the universe is lowered to one sm_103a kernel with
 * NVRTC.  param_names declares names that expressions may use besides the
 * processes and t (values are given per run).  payoffs are estimator
 * expressions over the terminal state (empty for none).                   */
int sde_plan_create(const char* const* equations, int32_t n_equations,
                    const char* const* param_names, int32_t n_params,
                    const char* const* payoffs, int32_t n_payoffs,
                    const sde_options* opts, sde_plan** out_plan);
/* Pathwise adjoint (no counterpart in the reference, which has no
 * derivatives): a plan whose runs also return d E[payoffs[0]] / d params
 * (grad_params, names of declared parameters) and / d X0 (grad_x0, process
 * names), by a reverse sweep of the step recursion -- Euler-Maruyama
 * (src/sim/euler.rs:5-37) or Runge-Kutta (src/sim/runge_kutta.rs:17-97,
 * its sign held fixed; in the reference's semantics the name->value cache
 * that the next stage 1 reads is differentiated as state) -- recomputed
 * from checkpoints every opts->ckpt_every steps.  No algebraic processes.
 * The run's estimates are [payoffs..., grad_params..., grad_x0...] per
 * replicate (per-path sums and sums of squares).                          */
int sde_plan_create_adjoint(const char* const* equations, int32_t n_equations,
                            const char* const* param_names, int32_t n_params,
                            const char* const* payoffs, int32_t n_payoffs,
                            const char* const* grad_params, int32_t n_grad_params,
                            const char* const* grad_x0, int32_t n_grad_x0,
                            const sde_options* opts, sde_plan** out_plan);
/* Number of estimator columns a run of this plan returns. */
int sde_plan_n_estimates(const sde_plan* plan, int32_t* n);
int sde_plan_destroy(sde_plan* plan);
int sde_plan_n_processes(const sde_plan* plan, int32_t* n);
int sde_plan_n_stochastic(const sde_plan* plan, int32_t* n);
/* ProcessUniverse.processes[i].name() (src/proc/mod.rs:46-59) */
int sde_plan_process_name(const sde_plan* plan, int32_t i, char* buf, size_t buf_len);
/* ProcessUniverse.process_registry lookup; *index = -1 if absent */
int sde_plan_process_index(const sde_plan* plan, const char* name, int32_t* index);
/* ProcessUniverse.stochastic_registry, index -> token (src/proc/util.rs:145-146) */
int sde_plan_stochastic_token(const sde_plan* plan, int32_t i, char* buf, size_t buf_len);
/* The generated CUDA C (for inspection); *needed gets the size incl. NUL. */
int sde_plan_source(const sde_plan* plan, char* buf, size_t buf_len, size_t* needed);
/* The NVRTC / ptxas log of the plan's compilation (registers, spills). */
int sde_plan_compile_log(const sde_plan* plan, char* buf, size_t buf_len, size_t* needed);
/* *on = 1 if the forward kernel was lowered to tcgen05 (SDE_TC_ON and an
 * eligible universe), else 0.  No counterpart in the reference. */
int sde_plan_tensor_cores(const sde_plan* plan, int32_t* on);

/* ---- runs --------------------------------------------------------------
 * Replaces the scenario loop of sde_sim_rs::sim::simulate
 *   (src/sim/mod.rs:41-88: per-scenario filtration, RNG, step loop).
 * Asynchronous on args->stream; results are read through sde_result_*.   */
int sde_run(sde_plan* plan, const sde_run_args* args, sde_result** out_result);

/* Reference-shaped one-shot entry: sde_sim_rs::sim::simulate
 *   (src/sim/mod.rs:20-27) and simulate_py (src/py_binding.rs:10-18).
 * scheme "euler" | "runge-kutta" (else SDE_ERR_INVALID; the reference
 * panics); rng_method "sobol" or anything else = pseudo (src/sim/mod.rs:65).
 * FP64, reference semantics, full filtration.  has_seed = 0 draws the seed
 * from the OS like src/sim/mod.rs:28-29.                                   */
int sde_simulate(const char* const* equations, int32_t n_equations,
                 const double* times, int32_t n_times,
                 const char* const* init_names, const double* init_values, int32_t n_init,
                 uint64_t n_scenarios, const char* scheme, const char* rng_method,
                 uint64_t seed, int32_t has_seed, sde_result** out_result);

/* ---- results ------------------------------------------------------------ */
int sde_result_destroy(sde_result* r);
/* Blocks until the run finished; reports a device status failure. */
int sde_result_wait(sde_result* r);
int sde_result_shape(const sde_result* r, uint64_t* n_paths, int32_t* n_out_times,
                     int32_t* n_processes, int32_t* n_replicates);
/* Time indices of the output slots [n_out_times]. */
int sde_result_time_indices(const sde_result* r, int32_t* host_out);
/* Device pointer of the filtration, layout [rep][time][process][path]. */
int sde_result_device_values(const sde_result* r, void** device_ptr, int32_t* elem_bytes);
/* Filtration copied to host as f64 in the given SDE_LAYOUT_*. */
int sde_result_copy_values(sde_result* r, double* host_out, int32_t layout);
/* Long / tidy rows in the reference's order (scenario, time, process),
 * the columns of ScenarioFiltration::to_lazyframe + concat
 *   (src/filtration.rs:81-116, src/sim/mod.rs:91).  Each host array has
 * n_replicates * n_paths * n_out_times * n_processes entries; any may be
 * NULL.  Built on the device, then copied.                                 */
int sde_result_copy_long(sde_result* r, int32_t* scenario, double* time,
                         int32_t* process, double* value);
/* The same rows in pinned host memory: *n_rows rows per column, read-only,
 * valid until sde_result_destroy.  Built on the device and copied once
 * (later calls return the same arrays); a caller that wraps them (numpy,
 * Arrow) copies nothing.  The values are the result's own; the scenario,
 * time and process columns depend only on the run's shape and are shared
 * by results of the same shape (the engine keeps the last 8 shapes, and a
 * result keeps its own alive), so a repeated call copies only values.    */
int sde_result_long_host(sde_result* r, const int32_t** scenario, const double** time,
                         const int32_t** process, const double** value, uint64_t* n_rows);
/* Per replicate and estimator: sum and sum of squares of the payoff over
 * paths, FP64 with compensated summation; arrays
 * [n_replicates][sde_plan_n_estimates].                                   */
int sde_result_estimates(sde_result* r, double* host_sum, double* host_sumsq);
/* The step kernel the run launched: *kernel one of SDE_KERNEL_*, its CTA
 * size and the paths one CTA steps (0 and 0 for a run without paths).  No
 * counterpart in the reference.                                           */
enum { SDE_KERNEL_NONE = 0, SDE_KERNEL_FORWARD = 1, SDE_KERNEL_CHUNKED = 2, SDE_KERNEL_WIDE = 3,
       SDE_KERNEL_TENSOR_CORES = 4, SDE_KERNEL_ADJOINT = 5 };
int sde_result_launch_info(const sde_result* r, int32_t* kernel, int32_t* block, int32_t* paths_per_block);

/* ---- estimates with no device allocation --------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory (their device memory comes from an arena or budget they do not
 * control, or an allocation's implicit synchronisation is not acceptable
 * where they call): runs a forward, pseudo-random plan and returns its
 * estimator sums with every piece of scratch in one 4 MiB static device
 * array of the library (held by each GPU that loads it until exit).  Host
 * inputs; host outputs host_sum / host_sumsq [n_replicates][n_payoffs];
 * synchronous on stream.  A run needing more than 4 MiB of scratch (about
 * 5e5 blocks x payoffs x replicates) fails with SDE_ERR_INVALID.  The
 * first call on a device loads the plan's kernels and resolves the array's
 * address.  Every call copies from pageable host memory and synchronizes
 * the stream, so none may be made on a stream under capture.  Every call
 * shares the array: calls that overlap on the GPU (other streams, other
 * threads) race.  A call that fails after queueing work waits for that work
 * before it returns.                                                       */
int sde_run_estimates_static(sde_plan* plan, const double* times, int32_t n_times,
                             const double* x0, int32_t n_x0, const double* params, int32_t n_params,
                             uint64_t n_paths, int32_t n_replicates, uint64_t seed, void* stream,
                             double* host_sum, double* host_sumsq);

/* ---- batched instances ---------------------------------------------------
 * No counterpart in the reference (one universe per simulate call): many
 * independent instances of a few templates (plans from sde_plan_create or
 * sde_plan_create_adjoint, pseudo-random, same precision), each with its
 * own uniform step count, horizon, path count, seed, initial values and
 * parameters, run by one persistent work-queue kernel captured in a CUDA
 * graph.  Paths per thread and block shape come from a timing autotuner at
 * prepare time.  An adjoint template's instances also return the gradients
 * of its payoff 0, as its plan's runs do; they take at most 4096 steps
 * (checkpoints every ceil(sqrt(steps)) steps in per-thread arrays; more is
 * SDE_ERR_UNSUPPORTED).                                                   */
typedef struct sde_batch sde_batch;
typedef struct sde_batch_job sde_batch_job;

typedef struct sde_batch_instances {
    uint32_t struct_size;       /* sizeof(sde_batch_instances)                 */
    int32_t n_instances;
    const int32_t* template_id; /* host [n]: index into the batch's templates  */
    const int32_t* n_steps;     /* host [n]: uniform steps on [0, t_end]       */
    const double* t_end;        /* host [n]                                    */
    const uint64_t* n_paths;    /* host [n]                                    */
    const uint64_t* seed;       /* host [n]: path s uses seed_from_u64(seed+s) */
    const double* x0;           /* host [n][x0_stride] by process index        */
    int32_t x0_stride;
    const double* params;       /* host [n][param_stride] by parameter index   */
    int32_t param_stride;
} sde_batch_instances;

int sde_batch_create(const sde_plan* const* templates, int32_t n_templates, sde_batch** out_batch);
int sde_batch_destroy(sde_batch* batch);
/* Uploads the instances, builds the work queue (longest instances first),
 * picks (block, paths per thread) by timing each candidate when autotune is
 * positive (0: the first candidate; -1 - v: candidate v, of the shapes
 * (128, 1), (256, 1), (128, 2), (256, 2), (128, 4)), and captures the
 * launch in a CUDA graph.                                                 */
int sde_batch_prepare(sde_batch* batch, const sde_batch_instances* inst, int32_t autotune,
                      void* stream, sde_batch_job** out_job);
/* Replays the graph: one persistent launch over every instance. */
int sde_batch_job_run(sde_batch_job* job, void* stream);
/* Waits; per instance and payoff: sum and sum of squares over its paths,
 * arrays [n_instances][n_payoffs] (n_payoffs = the largest template's
 * estimate count: payoffs, plus gradients for an adjoint template).      */
int sde_batch_job_results(sde_batch_job* job, double* host_sum, double* host_sumsq);
int sde_batch_job_info(const sde_batch_job* job, int32_t* block, int32_t* paths_per_thread,
                       int32_t* n_items, uint64_t* path_steps, int32_t* n_payoffs);
int sde_batch_job_destroy(sde_batch_job* job);

/* ---- known-answer kernels (device versions of the RNG building blocks) --
 * rand_chacha ChaCha8Rng::seed_from_u64(seed), u64 values [first, first+n)
 *   (src/rng/pseudo.rs:14-31).                                             */
int sde_kat_chacha8_u64(uint64_t seed, uint64_t first, uint64_t n, uint64_t* host_out);
/* Joe-Kuo D6 Sobol points [first, first+n) x dims as uint32
 *   (sobol crate via src/rng/sobol.rs:15-25).                              */
int sde_kat_sobol_points(int32_t dims, uint64_t first, uint64_t n, uint32_t* host_out);
/* fast_inverse_normal_cdf over host p[n] in FP64 (src/proc/increment.rs:161-179). */
int sde_kat_icdf(const double* host_p, uint64_t n, double* host_out);
/* Host-side Joe-Kuo direction numbers [dims][32] (no GPU needed). */
int sde_sobol_directions(int32_t dims, uint32_t* host_out);

/* ---- test hook -----------------------------------------------------------
 * No counterpart in the reference.  Sets, for runs launched afterwards from
 * any thread, how many SM clocks the tensor-core step with several threads
 * per path waits for its A operand before it gives up (0 restores the
 * default of about 1 s; a short budget polls without suspending).  A run
 * that gave up stops stepping, waits with the full budget for its copies
 * and product in flight, frees its tensor memory and reports SDE_ERR_DEVICE
 * from sde_result_wait; the plan stays usable.  For tests of that path.  */
int sde_debug_tc_wait_cycles(uint64_t cycles);

/* ---- measurement helper ------------------------------------------------
 * Times a kernel that keeps the SFU (MUFU) pipe busy and reports its
 * throughput in operations per second; the roofline denominator of the
 * terminal-only (SFU-bound) kernels.                                       */
int sde_probe_sfu_peak(double* ops_per_second);
/* Times a kernel in which every thread expands its own ChaCha8 key and
 * generates consecutive 16-word blocks, and reports blocks per second; the
 * roofline denominator of the pseudo-random kernels, whose bound is the
 * reference's generator.                                                  */
int sde_probe_chacha8_rate(double* blocks_per_second);

#ifdef __cplusplus
}
#endif
#endif
