// kernels.cu -- nvcc-built kernels of the engine: scramble masks, the
// estimator finalisation, the long-format filtration export, the
// known-answer kernels of the RNG building blocks and the SFU probe.
// The step kernels themselves are lowered per plan (codegen.cpp) and
// compiled with NVRTC.
#include "kernels.h"
#include "device/sde_rt.cuh"

namespace sde {

__global__ void k_make_xor_masks(sde_u32* __restrict__ masks, int n_rep, int stride, sde_u64 seed) {
    // one thread per (replicate, ChaCha block of 8 u64)
    const int blocks_per_rep = (stride + 7) / 8;
    const sde_u64 gid = (sde_u64)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= (sde_u64)n_rep * blocks_per_rep) return;
    const int r = (int)(gid / blocks_per_rep);
    const int b = (int)(gid % blocks_per_rep);
    sde_u32 key[8], w[16];
    sde_seed_from_u64(seed + (sde_u64)r, key);
    sde_chacha8_block(key, (sde_u64)b, w);
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const int d = b * 8 + j;
        if (d < stride) masks[(sde_u64)r * stride + d] = w[2 * j + 1];
    }
}

cudaError_t launch_make_xor_masks(sde_u32* masks, int n_rep, int stride, sde_u64 seed, cudaStream_t s) {
    const sde_u64 n = (sde_u64)n_rep * ((stride + 7) / 8);
    if (n == 0) return cudaSuccess;
    k_make_xor_masks<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(masks, n_rep, stride, seed);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------

__device__ __forceinline__ void merge_pair(double& s, double& c, double s2, double c2) {
    sde_neumaier(s, c, s2);
    c += c2;
}

__global__ void k_reduce_partials(const double* __restrict__ partials, int n_blocks, int K,
                                  double* __restrict__ out) {
    const int k = blockIdx.x, rep = blockIdx.y;
    double s = 0.0, sc = 0.0, q = 0.0, qc = 0.0;
    for (int b = threadIdx.x; b < n_blocks; b += blockDim.x) {
        const double* p = partials + (((sde_u64)rep * n_blocks + b) * K + k) * 4;
        merge_pair(s, sc, p[0], p[1]);
        merge_pair(q, qc, p[2], p[3]);
    }
    __shared__ double sm[256][4];
    sm[threadIdx.x][0] = s; sm[threadIdx.x][1] = sc;
    sm[threadIdx.x][2] = q; sm[threadIdx.x][3] = qc;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) {
            merge_pair(sm[threadIdx.x][0], sm[threadIdx.x][1], sm[threadIdx.x + h][0], sm[threadIdx.x + h][1]);
            merge_pair(sm[threadIdx.x][2], sm[threadIdx.x][3], sm[threadIdx.x + h][2], sm[threadIdx.x + h][3]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[((sde_u64)rep * K + k) * 2 + 0] = sm[0][0] + sm[0][1];
        out[((sde_u64)rep * K + k) * 2 + 1] = sm[0][2] + sm[0][3];
    }
}

cudaError_t launch_reduce_partials(const double* partials, int n_blocks, int K, int n_rep,
                                   double* out, cudaStream_t s) {
    if (K == 0 || n_rep == 0) return cudaSuccess;
    k_reduce_partials<<<dim3(K, n_rep), 256, 0, s>>>(partials, n_blocks, K, out);
    return cudaGetLastError();
}

__global__ void k_reduce_ranges(const double* __restrict__ partials, const int* __restrict__ ranges,
                                int K, double* __restrict__ out) {
    const int inst = blockIdx.x, k = blockIdx.y;
    const int b0 = ranges[2 * inst], b1 = ranges[2 * inst + 1];
    double s = 0.0, sc = 0.0, q = 0.0, qc = 0.0;
    for (int b = b0 + threadIdx.x; b < b1; b += blockDim.x) {
        const double* p = partials + ((sde_u64)b * K + k) * 4;
        merge_pair(s, sc, p[0], p[1]);
        merge_pair(q, qc, p[2], p[3]);
    }
    __shared__ double sm[128][4];
    sm[threadIdx.x][0] = s; sm[threadIdx.x][1] = sc;
    sm[threadIdx.x][2] = q; sm[threadIdx.x][3] = qc;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) {
            merge_pair(sm[threadIdx.x][0], sm[threadIdx.x][1], sm[threadIdx.x + h][0], sm[threadIdx.x + h][1]);
            merge_pair(sm[threadIdx.x][2], sm[threadIdx.x][3], sm[threadIdx.x + h][2], sm[threadIdx.x + h][3]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[((sde_u64)inst * K + k) * 2 + 0] = sm[0][0] + sm[0][1];
        out[((sde_u64)inst * K + k) * 2 + 1] = sm[0][2] + sm[0][3];
    }
}

cudaError_t launch_reduce_ranges(const double* item_partials, const int* ranges, int n, int K,
                                 double* out, cudaStream_t s) {
    if (n == 0 || K == 0) return cudaSuccess;
    k_reduce_ranges<<<dim3(n, K), 128, 0, s>>>(item_partials, ranges, K, out);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Long-format export: the filtration viewed as [rep][J][path] with
// J = slot*P + p is transposed to [rep][path][J] through a 32x32 shared
// tile, so both the reads (along paths) and the writes (along J) coalesce.

template <class T>
__global__ void k_long_export(const T* __restrict__ vals, sde_u64 n_paths, int J, int P,
                              const double* __restrict__ slot_times, sde_u64 scen_base,
                              int32_t* __restrict__ scen, double* __restrict__ time,
                              int32_t* __restrict__ proc, double* __restrict__ value) {
    __shared__ double tile[32][33];
    const int rep = blockIdx.z;
    const sde_u64 path0 = (sde_u64)blockIdx.x * 32;
    const int j0 = blockIdx.y * 32;
    const T* src = vals + (sde_u64)rep * J * n_paths;
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int j = j0 + r;
        const sde_u64 path = path0 + threadIdx.x;
        if (j < J && path < n_paths) tile[r][threadIdx.x] = (double)src[(sde_u64)j * n_paths + path];
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const sde_u64 path = path0 + r;
        const int j = j0 + threadIdx.x;
        if (j < J && path < n_paths) {
            const sde_u64 row = ((sde_u64)rep * n_paths + path) * J + j;
            if (value) value[row] = tile[threadIdx.x][r];
            if (scen) scen[row] = (int32_t)(scen_base + (sde_u64)rep * n_paths + path);
            if (time) time[row] = slot_times[j / P];
            if (proc) proc[row] = j % P;
        }
    }
}

cudaError_t launch_long_export(const void* vals, int elem_bytes, sde_u64 n_paths, int n_out, int P,
                               int n_rep, const double* slot_times, sde_u64 scen_base,
                               int32_t* scen, double* time, int32_t* proc, double* value,
                               cudaStream_t s) {
    const int J = n_out * P;
    if (J == 0 || n_paths == 0 || n_rep == 0) return cudaSuccess;
    dim3 grid((unsigned)((n_paths + 31) / 32), (unsigned)((J + 31) / 32), (unsigned)n_rep);
    dim3 block(32, 8);
    if (elem_bytes == 8)
        k_long_export<double><<<grid, block, 0, s>>>((const double*)vals, n_paths, J, P, slot_times,
                                                      scen_base, scen, time, proc, value);
    else
        k_long_export<float><<<grid, block, 0, s>>>((const float*)vals, n_paths, J, P, slot_times,
                                                     scen_base, scen, time, proc, value);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Known-answer kernels

__global__ void k_kat_chacha8(sde_u64 seed, sde_u64 first, sde_u64 n, sde_u64* __restrict__ out) {
    const sde_u64 i = (sde_u64)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const sde_u64 pos = first + i;
    sde_u32 key[8], w[16];
    sde_seed_from_u64(seed, key);
    sde_chacha8_block(key, pos / 8, w);
    const int j = (int)(pos % 8);
    out[i] = sde_pair(w[2 * j], w[2 * j + 1]);
}

cudaError_t launch_kat_chacha8(sde_u64 seed, sde_u64 first, sde_u64 n, sde_u64* out, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_kat_chacha8<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(seed, first, n, out);
    return cudaGetLastError();
}

__global__ void k_kat_sobol(const sde_u32* __restrict__ V, int dims, sde_u64 first, sde_u64 n,
                            sde_u32* __restrict__ out) {
    const sde_u64 i = (sde_u64)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * (sde_u64)dims) return;
    const sde_u64 pt = i / dims;
    const int d = (int)(i % dims);
    out[i] = sde_sobol_direct(V, d, sde_gray((sde_u32)(first + pt)));
}

cudaError_t launch_kat_sobol(const sde_u32* V, int dims, sde_u64 first, sde_u64 n, sde_u32* out,
                             cudaStream_t s) {
    const sde_u64 tot = n * (sde_u64)dims;
    if (tot == 0) return cudaSuccess;
    k_kat_sobol<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(V, dims, first, n, out);
    return cudaGetLastError();
}

__global__ void k_kat_icdf(const double* __restrict__ p, sde_u64 n, double* __restrict__ out) {
    const sde_u64 i = (sde_u64)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = sde_icdf_as26(p[i]);
}

cudaError_t launch_kat_icdf(const double* p, sde_u64 n, double* out, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_kat_icdf<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(p, n, out);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// SFU probe: 8 independent MUFU chains per thread (ex2.approx, lg2.approx,
// rsqrt.approx alternate), ITER iterations; every MUFU result feeds the next.

__device__ __forceinline__ float mufu_lg2(float x) {
    float y;
    asm volatile("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float mufu_rsq(float x) {
    float y;
    asm volatile("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ float mufu_rcp(float x) {
    float y;
    asm volatile("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// The op mix of the step kernels' normals: lg2, rsqrt and rcp in equal
// parts (ex2, which some parts issue at a higher rate, is left out).
template <int ITER>
__global__ void k_sfu_probe(float seed, float* __restrict__ sink) {
    float a0 = seed + threadIdx.x * 1e-7f, a1 = a0 + 0.1f, a2 = a0 + 0.2f, a3 = a0 + 0.3f;
    float a4 = a0 + 0.4f, a5 = a0 + 0.5f, a6 = a0 + 0.6f, a7 = a0 + 0.7f;
#pragma unroll 4
    for (int i = 0; i < ITER; ++i) {
        a0 = mufu_lg2(a0 + 1.5f); a1 = mufu_rsq(a1 + 1.5f); a2 = mufu_rcp(a2 + 1.5f);
        a3 = mufu_lg2(a3 + 1.5f); a4 = mufu_rsq(a4 + 1.5f); a5 = mufu_rcp(a5 + 1.5f);
        a6 = mufu_lg2(a6 + 1.5f); a7 = mufu_rsq(a7 + 1.5f);
    }
    const float r = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    if (r == 12345.678f) sink[threadIdx.x] = r;
}

// ChaCha8 block rate: each thread expands its own key (as a scenario does)
// and generates ITER consecutive blocks, folding their words into one so
// that none is dead; the roofline denominator of the pseudo-random kernels,
// whose bound is the reference's generator.  (sink: 1024 words; only a
// thread whose fold hits the magic value writes, at threadIdx.x < 256.)
template <int ITER>
__global__ void k_chacha_probe(sde_u64 seed, sde_u32* __restrict__ sink) {
    sde_u32 key[8];
    sde_seed_from_u64(seed + (sde_u64)blockIdx.x * blockDim.x + threadIdx.x, key);
    sde_u32 acc = 0u;
#pragma unroll 1
    for (int i = 0; i < ITER; ++i) {
        sde_u32 o[16];
        sde_chacha8_block(key, (sde_u64)i, o);
#pragma unroll
        for (int w = 0; w < 16; ++w) acc ^= o[w];
    }
    if (acc == 0x9e3779b9u) sink[threadIdx.x] = acc;
}

cudaError_t run_chacha_probe(double* blocks_per_second) {
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    sde_u32* sink = nullptr;
    e = cudaMalloc(&sink, 1024 * sizeof(sde_u32));
    if (e != cudaSuccess) return e;
    constexpr int ITER = 256;
    const int threads = 256, blocks = sms * 8;
    cudaEvent_t t0, t1;
    cudaEventCreate(&t0);
    cudaEventCreate(&t1);
    k_chacha_probe<ITER><<<blocks, threads>>>(1ull, sink);  // warm-up
    cudaEventRecord(t0);
    const int reps = 5;
    for (int r = 0; r < reps; ++r) k_chacha_probe<ITER><<<blocks, threads>>>(7ull + (sde_u64)r * 1000003ull, sink);
    cudaEventRecord(t1);
    e = cudaEventSynchronize(t1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, t0, t1);
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    cudaFree(sink);
    if (e != cudaSuccess) return e;
    *blocks_per_second = (double)reps * blocks * threads * ITER / (ms * 1e-3);
    return cudaGetLastError();
}

cudaError_t run_sfu_probe(double* ops_per_second) {
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    float* sink = nullptr;
    e = cudaMalloc(&sink, 1024 * sizeof(float));
    if (e != cudaSuccess) return e;
    constexpr int ITER = 4096;
    const int threads = 512, blocks = sms * 8;
    cudaEvent_t t0, t1;
    cudaEventCreate(&t0);
    cudaEventCreate(&t1);
    k_sfu_probe<ITER><<<blocks, threads>>>(0.5f, sink);  // warm-up
    cudaEventRecord(t0);
    const int reps = 5;
    for (int r = 0; r < reps; ++r) k_sfu_probe<ITER><<<blocks, threads>>>(0.5f + r, sink);
    cudaEventRecord(t1);
    e = cudaEventSynchronize(t1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, t0, t1);
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    cudaFree(sink);
    if (e != cudaSuccess) return e;
    const double ops = (double)reps * blocks * threads * ITER * 8.0;
    *ops_per_second = ops / (ms * 1e-3);
    return cudaGetLastError();
}

}  // namespace sde
