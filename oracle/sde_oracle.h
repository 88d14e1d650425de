/*
 * sde_oracle.h -- CPU restatement of the sde-sim-rs path-simulation algorithm.
 *
 * TEST INFRASTRUCTURE ONLY.  The GPU engine's parity tests compare with this
 * library; only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference
 * arm may load it.  The product (libsdegpu.so) never links or calls it.
 *
 * It restates, in plain C, the reference crate's hot path:
 *   src/sim/mod.rs:20-92         simulate (scenario loop, RNG choice)
 *   src/sim/euler.rs:5-37        euler_iteration
 *   src/sim/runge_kutta.rs:5-107 runge_kutta_iteration (stale-cache semantics)
 *   src/proc/increment.rs:26-200 dt / dW / dN incrementors and inverse CDFs
 *   src/rng/pseudo.rs:14-59      ChaCha8 per scenario, n_inc draws per step
 *   src/rng/sobol.rs:15-78       Sobol point s+5 plus a per-scenario random shift
 *   src/filtration.rs:22-116     [time][process] buffer and its name->value cache
 *   src/proc/util.rs:52-166      equation grammar
 *   src/func.rs:18-42            coefficient evaluation through the cache
 * and, for the third-party crates that are not vendored in the reference
 * (rand 0.9.2 / rand_core / rand_chacha 0.9, sobol 1.0.2, fasteval 0.2.4),
 * their published algorithms: PCG32-based seed_from_u64, ChaCha with 8
 * rounds, (u64 >> 11) * 2^-53 doubles, Joe-Kuo D6 Gray-code Sobol points
 * (uint32 * 2^-32), and the fasteval expression grammar.
 *
 * Pins: the ChaCha core at 20 rounds against the `cryptography` package and
 * at 8 rounds against the published ChaCha8 zero-key test vector; Sobol
 * points against scipy.stats.qmc.Sobol(bits=32).  The PCG32 seeding and the
 * fasteval evaluation order are restated, not pinned (the crates' sources and
 * a Rust toolchain are not available).
 */
#ifndef SDE_ORACLE_H
#define SDE_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_universe orc_universe;

enum { ORC_EULER = 0, ORC_RK = 1 };
enum { ORC_PSEUDO = 0, ORC_SOBOL = 1 };
enum { ORC_SCRAMBLE_SHIFT = 0, ORC_SCRAMBLE_XOR = 1 };
enum { ORC_SEM_REFERENCE = 0, ORC_SEM_TEXTBOOK = 1 };

typedef struct orc_cfg {
    int scheme;     /* ORC_EULER | ORC_RK                                  */
    int rng;        /* ORC_PSEUDO | ORC_SOBOL                              */
    int scramble;   /* ORC_SCRAMBLE_SHIFT (reference) | ORC_SCRAMBLE_XOR   */
    int semantics;  /* ORC_SEM_REFERENCE | ORC_SEM_TEXTBOOK                */
    uint64_t seed;  /* scenario s uses ChaCha8 stream seed_from_u64(seed+s);
                       in XOR mode replicate r uses masks from seed + r     */
    uint64_t n_paths_per_replicate; /* N: XOR replicates restart points at 0 */
    const uint32_t* sobol_v;        /* [dims][32] direction numbers          */
    int sobol_dims;
    int icdf;       /* 0: AS 26.2.23 (reference); 1: the accurate option      */
} orc_cfg;

/* One Poisson draw (fast_inverse_poisson_cdf, src/proc/increment.rs:182-200):
 * step t, stochastic index idx, uniform u, lambda * dt, count k. */
typedef struct orc_jump {
    int32_t t, idx;
    double u, lam;
    uint64_t k;
} orc_jump;

/* ---- universe (equation parsing, src/proc/util.rs:52-166) ------------- */
int  orc_parse(const char* const* eqs, int n_eq,
               const char* const* param_names, const double* param_vals,
               int n_params, orc_universe** out, char* err, size_t errlen);
void orc_free(orc_universe* u);
int  orc_n_processes(const orc_universe* u);
int  orc_n_stochastic(const orc_universe* u);
int  orc_process_name(const orc_universe* u, int i, char* buf, size_t n);
int  orc_process_is_levy(const orc_universe* u, int i);
int  orc_stochastic_token(const orc_universe* u, int i, char* buf, size_t n);
int  orc_process_index(const orc_universe* u, const char* name); /* registry */

/* ---- simulation (src/sim/mod.rs:20-92) --------------------------------
 * Paths [path_begin, path_end) of the global scenario range.  x0 is the
 * time-0 row indexed by process (missing initial values are 0.0).
 * out_full: [path][T][P] (reference row order) or NULL.
 * out_terminal: [path][P] or NULL.  Returns 0 or an error code. */
int orc_simulate(const orc_universe* u, const double* times, int n_times,
                 const double* x0, uint64_t path_begin, uint64_t path_end,
                 const orc_cfg* cfg, double* out_full, double* out_terminal,
                 int n_threads, char* err, size_t errlen);

/* Estimator: sum and sum of squares of payoff(X_T) over paths, Neumaier
 * compensated, computed per path inside the same threaded scenario loop. */
int orc_estimate(const orc_universe* u, const double* times, int n_times,
                 const double* x0, uint64_t path_begin, uint64_t path_end,
                 const orc_cfg* cfg, const char* payoff, int n_threads,
                 double* sum, double* sumsq, char* err, size_t errlen);

/* payoff(expr) over rows of terminal values [n][P] at time t. */
int orc_eval_payoff(const orc_universe* u, const char* expr, double t,
                    const double* rows, int64_t n, double* out,
                    char* err, size_t errlen);

/* ---- RNG primitives ---------------------------------------------------- */
void     orc_chacha_block(const uint32_t key[8], uint64_t counter,
                          uint64_t stream, int rounds, uint32_t out[16]);
void     orc_seed_from_u64(uint64_t state, uint32_t key[8]);
/* u64 values first..first+n-1 of ChaCha8Rng::seed_from_u64(seed). */
void     orc_chacha8_u64(uint64_t seed, uint64_t first, uint64_t n, uint64_t* out);
double   orc_u64_to_f64(uint64_t x);
uint32_t orc_xor_mask(uint64_t seed, int replicate, int dim);

/* ---- Sobol (sobol crate / Joe-Kuo D6) ---------------------------------- */
/* poly[d], vinit[d][18] as in the Joe-Kuo table -> V[d][32]. */
int  orc_sobol_directions(const int64_t* poly, const int64_t* vinit, int dims,
                          uint32_t* V);
void orc_sobol_points(const uint32_t* V, int dims, uint64_t first, uint64_t n,
                      uint32_t* out /* [n][dims] */);

/* ---- inverse CDFs (src/proc/increment.rs:161-200) ---------------------- */
double   orc_icdf_as26(double p);
double   orc_icdf_accurate(double p);
uint64_t orc_poisson(double u, double lambda);

/* Every Poisson draw of scenario `scenario` in draw order (at most max_out). */
int orc_jump_trace(const orc_universe* u, const double* times, int n_times, const double* x0,
                   uint64_t scenario, const orc_cfg* cfg, orc_jump* out, int max_out, int* n_out,
                   char* err, size_t errlen);

#ifdef __cplusplus
}
#endif
#endif
