// kernels.h -- host launchers of the nvcc-built (non-lowered) kernels.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

#include "device/sde_args.h"

namespace sde {

// XOR scramble masks [n_rep][stride]: replicate r, dimension d -> high word
// of u64 number d of ChaCha8Rng::seed_from_u64(seed + r).
cudaError_t launch_make_xor_masks(sde_u32* masks, int n_rep, int stride, sde_u64 seed, cudaStream_t s);

// Estimator partials [n_rep][n_blocks][K][4] -> [n_rep][K][2] {sum, sumsq},
// compensated, deterministic.
cudaError_t launch_reduce_partials(const double* partials, int n_blocks, int K, int n_rep,
                                   double* out, cudaStream_t s);

// Item partials [n_items][K][4] -> per instance [n][K][2]; instance i owns
// items ranges[2i] .. ranges[2i+1]-1.
cudaError_t launch_reduce_ranges(const double* item_partials, const int* ranges, int n, int K,
                                 double* out, cudaStream_t s);

// Filtration [rep][slot][p][path] (f32 or f64) -> long rows ordered
// (scenario, time, process) as in src/filtration.rs:81-116.
cudaError_t launch_long_export(const void* vals, int elem_bytes, sde_u64 n_paths, int n_out, int P,
                               int n_rep, const double* slot_times, sde_u64 scen_base,
                               int32_t* scen, double* time, int32_t* proc, double* value,
                               cudaStream_t s);

cudaError_t launch_kat_chacha8(sde_u64 seed, sde_u64 first, sde_u64 n, sde_u64* out, cudaStream_t s);
cudaError_t launch_kat_sobol(const sde_u32* V, int dims, sde_u64 first, sde_u64 n, sde_u32* out,
                             cudaStream_t s);
cudaError_t launch_kat_icdf(const double* p, sde_u64 n, double* out, cudaStream_t s);

// SFU (MUFU) throughput probe: ops/s over a timed launch.
cudaError_t run_sfu_probe(double* ops_per_second);
// ChaCha8 block-rate probe: blocks/s over a timed launch.
cudaError_t run_chacha_probe(double* blocks_per_second);

}  // namespace sde
