// noalloc.cu -- payoff estimates through a forward plan with no device
// allocation.
//
// Some callers cannot call cudaMalloc: an application that hands out device
// memory only through its own arena or budget, a latency-critical loop that
// cannot afford the implicit synchronisation of an allocation, a process
// whose device memory another runtime has already reserved.  For them this
// entry point runs the plan's step kernel and the estimator reduction with
// all of their scratch (staged time grid, initial values, parameters, block
// partial sums, estimates) in one file-scope device array of fixed size.
// The caller passes host inputs and host outputs.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>

#include "../../include/sdegpu.h"
#include "codegen.h"
#include "device/sde_args.h"
#include "engine_internal.h"
#include "kernels.h"

namespace sde {

// 4 MiB, held by every GPU that loads this library until the process exits.
constexpr size_t kStaticScratchBytes = 4u << 20;
static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

// dts, sqrt(dts) and the FP32 copies from the staged time grid, computed the
// way the host staging of sde_run computes them (IEEE subtraction, correctly
// rounded sqrt, round-to-nearest float conversion); no output slots.
__global__ void k_stage_time_grid(const double* __restrict__ times, int T, double* __restrict__ dts,
                                  double* __restrict__ sdts, float* __restrict__ tf, float* __restrict__ dtf,
                                  float* __restrict__ sdtf, int* __restrict__ tidx) {
    for (int t = threadIdx.x; t < T; t += blockDim.x) {
        tf[t] = (float)times[t];
        tidx[t] = -1;
        if (t + 1 < T) {
            const double d = times[t + 1] - times[t];
            const double r = sqrt(d);
            dts[t] = d;
            sdts[t] = r;
            dtf[t] = (float)d;
            sdtf[t] = (float)r;
        }
    }
}

// Device address of the scratch array, resolved once per device with that
// device current.  Host code may not use the symbol itself as an address.
static cudaError_t scratch_address(int dev, unsigned char** out) {
    static std::mutex mu;
    static std::map<int, unsigned char*> addr;
    std::lock_guard<std::mutex> g(mu);
    auto it = addr.find(dev);
    if (it != addr.end()) {
        *out = it->second;
        return cudaSuccess;
    }
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess) return e;
    addr[dev] = (unsigned char*)p;
    *out = (unsigned char*)p;
    return cudaSuccess;
}

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

static int fail_with(int code, const std::string& msg) {
    set_last_error(msg);
    return code;
}

static int cuda_fail(cudaError_t e, const char* what) {
    return fail_with(e == cudaErrorMemoryAllocation ? SDE_ERR_OOM : SDE_ERR_CUDA,
                     std::string(what) + ": " + cudaGetErrorString(e));
}

}  // namespace sde

using namespace sde;

extern "C" int sde_run_estimates_static(sde_plan* plan, const double* times, int32_t n_times, const double* x0,
                                        int32_t n_x0, const double* params, int32_t n_params, uint64_t n_paths,
                                        int32_t n_replicates, uint64_t seed, void* stream, double* host_sum,
                                        double* host_sumsq) {
    if (!plan || !times || !host_sum || !host_sumsq) return fail_with(SDE_ERR_INVALID, "NULL argument");
    if ((n_x0 > 0 && !x0) || (n_params > 0 && !params)) return fail_with(SDE_ERR_INVALID, "NULL argument");
    const int T = n_times;
    if (T < 1) return fail_with(SDE_ERR_INVALID, "need at least one time point");
    for (int t = 1; t < T; ++t)
        if (!(times[t] > times[t - 1])) return fail_with(SDE_ERR_INVALID, "time_steps must be strictly increasing");
    if (n_replicates < 1 || n_replicates > 65535) return fail_with(SDE_ERR_INVALID, "n_replicates must be in 1..65535");
    PlanView v;
    const int rc = plan_view(plan, &v);  // first call on a device: loads the plan's kernels
    if (rc != SDE_OK) return rc;
    if (v.adjoint) return fail_with(SDE_ERR_UNSUPPORTED, "the static-scratch entry runs forward plans");
    if (v.tensor_cores)
        return fail_with(SDE_ERR_UNSUPPORTED, "the static-scratch entry runs CUDA-core plans (tensor_cores off)");
    if (v.rng != RNG_PSEUDO)
        return fail_with(SDE_ERR_UNSUPPORTED, "the static-scratch entry runs pseudo-random plans (Sobol tables are "
                                              "engine-allocated)");
    if (v.n_payoffs < 1) return fail_with(SDE_ERR_INVALID, "the plan has no payoff to estimate");
    if (n_params != v.n_params) return fail_with(SDE_ERR_INVALID, "parameter count does not match the plan");
    if (n_x0 < 0 || n_x0 > v.n_processes) return fail_with(SDE_ERR_INVALID, "more initial values than processes");
    if (v.scheme == SCHEME_RK && v.n_stochastic == 0 && T > 1)
        return fail_with(SDE_ERR_RNG_INDEX, "RNG Index 0 out of bounds (max 0)");
    const int P = v.n_processes, K = v.n_payoffs, Tm1 = T > 1 ? T - 1 : 1;
    const uint64_t per_block = (uint64_t)v.block * (uint64_t)v.ppt;
    const uint64_t gx = n_paths / per_block + (n_paths % per_block != 0);
    if (gx > 0x7fffffffull) return fail_with(SDE_ERR_INVALID, "too many paths for one launch");
    // scratch layout, every piece 256-byte aligned
    size_t off = 0;
    const size_t o_times = off; off = align256(off + (size_t)T * 8);
    const size_t o_dts = off; off = align256(off + (size_t)Tm1 * 8);
    const size_t o_sdts = off; off = align256(off + (size_t)Tm1 * 8);
    const size_t o_x0 = off; off = align256(off + (size_t)(P > 0 ? P : 1) * 8);
    const size_t o_par = off; off = align256(off + (size_t)(n_params > 0 ? n_params : 1) * 8);
    const size_t o_tf = off; off = align256(off + (size_t)T * 4);
    const size_t o_dtf = off; off = align256(off + (size_t)Tm1 * 4);
    const size_t o_sdtf = off; off = align256(off + (size_t)Tm1 * 4);
    const size_t o_tidx = off; off = align256(off + (size_t)T * 4);
    const size_t o_part = off; off = align256(off + (size_t)n_replicates * gx * K * 4 * 8);
    const size_t o_est = off; off = align256(off + (size_t)n_replicates * K * 2 * 8);
    if (off > kStaticScratchBytes) {
        char msg[256];
        std::snprintf(msg, sizeof msg, "this run needs %zu bytes of scratch; the static scratch holds %zu bytes",
                      off, kStaticScratchBytes);
        return fail_with(SDE_ERR_INVALID, msg);
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    unsigned char* base = nullptr;
    e = scratch_address(dev, &base);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress");
    if (n_paths == 0) {
        for (int i = 0; i < n_replicates * K; ++i) host_sum[i] = host_sumsq[i] = 0.0;
        return SDE_OK;
    }
    cudaStream_t s = (cudaStream_t)stream;
    // From the first copy on, a failure first waits for what this call has
    // already queued on s, so no work of a failed call is left writing the
    // shared array when the caller's next call starts.
    auto async_fail = [s](cudaError_t err, const char* what) {
        (void)cudaStreamSynchronize(s);
        return cuda_fail(err, what);
    };
    double* d_times = (double*)(base + o_times);
    double* d_x0 = (double*)(base + o_x0);
    double* d_par = (double*)(base + o_par);
    double* d_est = (double*)(base + o_est);
    if ((e = cudaMemcpyAsync(d_times, times, (size_t)T * 8, cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return async_fail(e, "stage times");
    if ((e = cudaMemsetAsync(d_x0, 0, (size_t)(P > 0 ? P : 1) * 8, s)) != cudaSuccess) return async_fail(e, "stage x0");
    if (n_x0 > 0 && (e = cudaMemcpyAsync(d_x0, x0, (size_t)n_x0 * 8, cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return async_fail(e, "stage x0");
    if (n_params > 0 &&
        (e = cudaMemcpyAsync(d_par, params, (size_t)n_params * 8, cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return async_fail(e, "stage params");
    k_stage_time_grid<<<1, 256, 0, s>>>(d_times, T, (double*)(base + o_dts), (double*)(base + o_sdts),
                                        (float*)(base + o_tf), (float*)(base + o_dtf), (float*)(base + o_sdtf),
                                        (int*)(base + o_tidx));
    if ((e = cudaGetLastError()) != cudaSuccess) return async_fail(e, "stage time grid");
    sde_args A;
    std::memset(&A, 0, sizeof A);
    A.times = d_times;
    A.dts = (const double*)(base + o_dts);
    A.sqrt_dts = (const double*)(base + o_sdts);
    A.times_f = (const float*)(base + o_tf);
    A.dts_f = (const float*)(base + o_dtf);
    A.sqrt_dts_f = (const float*)(base + o_sdtf);
    A.x0 = d_x0;
    A.params = d_par;
    A.out_tidx = (const int*)(base + o_tidx);
    A.partials = (double*)(base + o_part);
    A.n_paths = n_paths;
    A.seed = seed;
    A.T = T;
    A.n_rep = n_replicates;
    void* kargs[] = {&A};
    if ((e = cudaLaunchKernel((const void*)v.kernel, dim3((unsigned)gx, (unsigned)n_replicates), dim3(v.block), kargs,
                              0, s)) != cudaSuccess)
        return async_fail(e, "step kernel launch");
    if ((e = launch_reduce_partials(A.partials, (int)gx, K, n_replicates, d_est, s)) != cudaSuccess)
        return async_fail(e, "estimator reduction");
    // [rep][K][2] -> the caller's [rep][K] sums and sums of squares
    if ((e = cudaMemcpy2DAsync(host_sum, 8, d_est, 16, 8, (size_t)n_replicates * K, cudaMemcpyDeviceToHost, s)) !=
        cudaSuccess)
        return async_fail(e, "estimates D2H");
    if ((e = cudaMemcpy2DAsync(host_sumsq, 8, d_est + 1, 16, 8, (size_t)n_replicates * K, cudaMemcpyDeviceToHost,
                               s)) != cudaSuccess)
        return async_fail(e, "estimates D2H");
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail(e, "kernel execution");
    return SDE_OK;
}
