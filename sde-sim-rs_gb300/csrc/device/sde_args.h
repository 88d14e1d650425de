/*
 * sde_args.h -- launch arguments shared by the host library and the device
 * kernels (both the nvcc-built ones and the NVRTC-lowered step kernels).
 * Plain C layout; passed to kernels by value.
 */
#ifndef SDE_ARGS_H
#define SDE_ARGS_H

typedef unsigned long long sde_u64;
typedef unsigned int sde_u32;

/* Forward pass over n_rep replicates x n_paths paths. */
typedef struct sde_args {
    const double* times;      /* [T]   time grid (src/filtration.rs:14)            */
    const double* dts;        /* [T-1] times[t+1]-times[t] (increment.rs:37-43)      */
    const double* sqrt_dts;   /* [T-1] sqrt(dts) (increment.rs:74-80)                */
    const float* times_f;     /* float copies for the FP32 stepping kernels          */
    const float* dts_f;
    const float* sqrt_dts_f;
    const double* x0;         /* [P]   time-0 row                                    */
    const double* params;     /* [n_params] named parameters                         */
    const int* out_tidx;      /* [T]   output slot of time index t, or -1            */
    const sde_u32* sobol_v;   /* [dims][32] Joe-Kuo direction numbers                */
    const sde_u32* sobol_vt;  /* [32][dims] the same, transposed                     */
    const sde_u32* sobol_lo;  /* [dims/4][32][4]: xor of direction numbers 0..4 by
                                 5 bits, four dimensions per low index      */
    const sde_u32* masks;     /* [n_rep][dims] XOR scramble masks                    */
    void* out;                /* [rep][n_out][P][n_paths] filtration slices          */
    double* partials;         /* [rep][gridDim.x][K][4] estimator partial sums       */
    float* ckpt;              /* adjoint checkpoints [rep][n_ckpt][P][n_paths]       */
    double* grad_partials;    /* [rep][gridDim.x][G][2] adjoint gradient partials   */
    void* inc;                /* adjoint: the forward pass's increments
                                 [rep][T-1][n_inc][n_paths], or NULL (recompute)    */
    int* status;              /* device status word (0 = ok)                         */
    sde_u64 n_paths;          /* paths per replicate                                 */
    sde_u64 path_base;        /* scenario index of path 0 of replicate 0             */
    sde_u64 seed;             /* ChaCha8 stream seed (scenario s -> seed + s)        */
    int T;                    /* time points                                         */
    int n_out;                /* output slots                                        */
    int sobol_dims;           /* dimensions held by the tables                       */
    int n_rep;                /* replicates                                          */
    int ckpt_every;           /* adjoint: steps between checkpoints                  */
    int n_ckpt;               /* adjoint: checkpoints per path                       */
    int mask_stride;          /* words per replicate row of masks (multiple of 32)  */
    float udt_f, usdt_f;      /* the FP32 step and its square root when every
                                 step of the grid has them (uniform-grid kernels) */
    int pad1;
    sde_u64 tc_wait_cycles;   /* tensor-core step, several threads per path: SM
                                 clocks the A-ready wait lasts before it gives up
                                 (0: about 1 s, the other waits' budget)         */
} sde_args;

/* ---- batched instances: many independent SDE instances in one persistent
 *      launch.  Instance i runs n_steps uniform steps of size dt on its own
 *      template (lowered universe), parameters and initial values. */
typedef struct sde_batch_inst {
    double dt, sdt;           /* step and its square root                       */
    sde_u64 n_paths;          /* paths of this instance                         */
    sde_u64 seed;             /* path s uses ChaCha8 seed_from_u64(seed + s)     */
    float dt_f, sdt_f;
    int tmpl;                 /* template (universe) index                      */
    int n_steps;
    int x0_off;               /* offset of the instance's x0 row                */
    int par_off;              /* offset of the instance's parameter row         */
} sde_batch_inst;

typedef struct sde_batch_item {
    sde_u64 first_path;       /* first path of the chunk                        */
    int inst;                 /* instance                                       */
    int pad;
} sde_batch_item;

typedef struct sde_batch_args {
    const sde_batch_inst* inst;
    const sde_batch_item* items;  /* chunks, longest instances first            */
    const double* x0;
    const double* params;
    unsigned int* counter;        /* work-queue head, zeroed before each launch */
    double* item_partials;        /* [n_items][K][4]                            */
    int n_items;
    int pad0;
} sde_batch_args;

#endif
