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
    const sde_u32* sobol_lo;  /* [dims][32] xor of direction numbers 0..4 by 5 bits  */
    const sde_u32* masks;     /* [n_rep][dims] XOR scramble masks                    */
    void* out;                /* [rep][n_out][P][n_paths] filtration slices          */
    double* partials;         /* [rep][gridDim.x][K][4] estimator partial sums       */
    float* ckpt;              /* adjoint checkpoints [rep][n_ckpt][P][n_paths]       */
    double* grad_partials;    /* [rep][gridDim.x][G][2] adjoint gradient partials   */
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
    int pad1;
} sde_args;

#endif
