// engine.cpp -- plans, runs and results behind the C ABI (include/sdegpu.h).
//
// A plan is the reference's parse_equations (src/proc/util.rs:52-66) plus a
// one-time lowering of every coefficient to device code: the generated CUDA
// C is compiled by NVRTC for sm_103a and loaded per device with
// cudaLibraryLoadData.  A run replaces the scenario loop of sim::simulate
// (src/sim/mod.rs:41-88) with one kernel launch over (paths x replicates).
#include <cuda_runtime.h>
#include <nvrtc.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <functional>
#include <list>
#include <map>
#include <memory>
#include <mutex>
#include <random>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/sdegpu.h"
#include "_gen/embedded.h"
#include "_gen/joe_kuo_d6.h"
#include "codegen.h"
#include "frontend.h"
#include "engine_internal.h"
#include "kernels.h"

namespace sde {

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------

static thread_local std::string g_last_error;
// Budget of the tensor-core step's A-ready wait in SM clocks for runs
// launched from now on (0: the default of about 1 s); set only by
// sde_debug_tc_wait_cycles, a test hook.
static std::atomic<unsigned long long> g_tc_wait_cycles{0ull};

struct Error {
    int code;
    std::string msg;
};

[[noreturn]] static void fail(int code, const std::string& msg) { throw Error{code, msg}; }

static void cuda_check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) {
        if (e == cudaErrorMemoryAllocation) fail(SDE_ERR_OOM, std::string(what) + ": " + cudaGetErrorString(e));
        fail(SDE_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    }
}

template <class F>
static int guarded(F&& f) {
    try {
        f();
        return SDE_OK;
    } catch (const Error& e) {
        g_last_error = e.msg;
        return e.code;
    } catch (const ParseError& e) {
        g_last_error = e.what();
        return SDE_ERR_PARSE;
    } catch (const std::bad_alloc&) {
        g_last_error = "host allocation failed";
        return SDE_ERR_OOM;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        return SDE_ERR_INVALID;
    }
}

// ---------------------------------------------------------------------------
// memory pools: device buffers and pinned host buffers are cached by size so
// repeated runs do not pay cudaMalloc / cudaHostAlloc.
// ---------------------------------------------------------------------------

static size_t round_size(size_t n) {
    if (n <= 256) return 256;
    if (n <= (1u << 20)) {
        size_t r = 256;
        while (r < n) r <<= 1;
        return r;
    }
    const size_t g = 1u << 20;
    return (n + g - 1) / g * g;
}

struct Pool {
    bool pinned;
    std::mutex mu;
    std::map<std::pair<int, size_t>, std::vector<void*>> free_;
    std::unordered_map<void*, std::pair<int, size_t>> live_;

    explicit Pool(bool p) : pinned(p) {}

    void* get(size_t n) {
        int dev = 0;
        if (!pinned) cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
        const size_t sz = round_size(n);
        {
            std::lock_guard<std::mutex> g(mu);
            auto it = free_.find({dev, sz});
            if (it != free_.end() && !it->second.empty()) {
                void* p = it->second.back();
                it->second.pop_back();
                live_[p] = {dev, sz};
                return p;
            }
        }
        void* p = nullptr;
        cudaError_t e = pinned ? cudaHostAlloc(&p, sz, cudaHostAllocDefault) : cudaMalloc(&p, sz);
        if (e != cudaSuccess) {
            cudaGetLastError();
            trim(dev);
            e = pinned ? cudaHostAlloc(&p, sz, cudaHostAllocDefault) : cudaMalloc(&p, sz);
            if (e != cudaSuccess) {
                cudaGetLastError();
                fail(SDE_ERR_OOM, std::string(pinned ? "cudaHostAlloc" : "cudaMalloc") + " of " +
                                      std::to_string(sz) + " bytes failed");
            }
        }
        std::lock_guard<std::mutex> g(mu);
        live_[p] = {dev, sz};
        return p;
    }
    void put(void* p) {
        if (!p) return;
        std::lock_guard<std::mutex> g(mu);
        auto it = live_.find(p);
        if (it == live_.end()) return;
        free_[it->second].push_back(p);
        live_.erase(it);
    }
    void trim(int dev) {
        std::lock_guard<std::mutex> g(mu);
        for (auto& kv : free_) {
            if (!pinned && kv.first.first != dev) continue;
            for (void* p : kv.second) pinned ? cudaFreeHost(p) : cudaFree(p);
            kv.second.clear();
        }
    }
};

static Pool& dpool() { static Pool* p = new Pool(false); return *p; }
static Pool& hpool() { static Pool* p = new Pool(true); return *p; }

struct DBuf {
    void* p = nullptr;
    DBuf() = default;
    explicit DBuf(size_t n) : p(n ? dpool().get(n) : nullptr) {}
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    DBuf(DBuf&& o) noexcept : p(o.p) { o.p = nullptr; }
    DBuf& operator=(DBuf&& o) noexcept { std::swap(p, o.p); return *this; }
    ~DBuf() { dpool().put(p); }
    template <class T> T* as() const { return (T*)p; }
};

struct HBuf {
    void* p = nullptr;
    HBuf() = default;
    explicit HBuf(size_t n) : p(n ? hpool().get(n) : nullptr) {}
    HBuf(const HBuf&) = delete;
    HBuf& operator=(const HBuf&) = delete;
    HBuf(HBuf&& o) noexcept : p(o.p) { o.p = nullptr; }
    HBuf& operator=(HBuf&& o) noexcept { std::swap(p, o.p); return *this; }
    ~HBuf() { hpool().put(p); }
    template <class T> T* as() const { return (T*)p; }
};

// ---------------------------------------------------------------------------
// Joe-Kuo D6 direction numbers.  Scaled form of the Bratley-Fox recurrence:
//   v_k = v_{k-s} ^ (v_{k-s} >> s) ^ xor_{i<s} a_i v_{k-i},  v_k = m_k 2^(32-k)
// ---------------------------------------------------------------------------

static const int kSobolMaxDims = kJkDims;

static void sobol_directions_host(int dims, uint32_t* V) {
    for (int d = 0; d < dims; ++d) {
        uint32_t* v = V + (size_t)d * 32;
        if (d == 0) {
            for (int k = 0; k < 32; ++k) v[k] = 0x80000000u >> k;
            continue;
        }
        const uint32_t poly = kJkPoly[d];
        int s = 31;
        while (!((poly >> s) & 1u)) --s;
        for (int k = 0; k < s && k < 32; ++k) v[k] = kJkVinit[(size_t)d * 18 + k] << (31 - k);
        for (int k = s; k < 32; ++k) {
            uint32_t x = v[k - s] ^ (v[k - s] >> s);
            for (int i = 1; i < s; ++i)
                if ((poly >> (s - i)) & 1u) x ^= v[k - i];
            v[k] = x;
        }
    }
}

struct SobolTables {
    DBuf V, VT, LO;
    int dims = 0;
};

static std::mutex g_tab_mu;
static std::map<int, std::unique_ptr<SobolTables>> g_tables;  // by device

static SobolTables& sobol_tables(cudaStream_t stream) {
    int dev = 0;
    cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    std::lock_guard<std::mutex> g(g_tab_mu);
    auto& t = g_tables[dev];
    if (t) return *t;
    const int dims = kSobolMaxDims;
    // LO: [dims/4][32 low indices][4 dimensions] -- a lane's words of four
    // consecutive dimensions are one aligned 16-byte load, and a warp's 32
    // lanes read 512 contiguous bytes; padded to a multiple of 4 dimensions
    const int dims4 = (dims + 3) / 4 * 4;
    std::vector<uint32_t> V((size_t)dims * 32), VT((size_t)dims * 32), LO((size_t)dims4 * 32, 0u);
    sobol_directions_host(dims, V.data());
    for (int d = 0; d < dims; ++d)
        for (int b = 0; b < 32; ++b) VT[(size_t)b * dims + d] = V[(size_t)d * 32 + b];
    for (int d = 0; d < dims; ++d)
        for (int l = 0; l < 32; ++l) {
            uint32_t x = 0;
            for (int b = 0; b < 5; ++b)
                if ((l >> b) & 1) x ^= V[(size_t)d * 32 + b];
            LO[(size_t)(d >> 2) * 128 + (size_t)l * 4 + (d & 3)] = x;
        }
    auto nt = std::make_unique<SobolTables>();
    const size_t bytes = (size_t)dims * 32 * 4;
    nt->V = DBuf(bytes);
    nt->VT = DBuf(bytes);
    nt->LO = DBuf((size_t)dims4 * 32 * 4);
    cuda_check(cudaMemcpyAsync(nt->V.p, V.data(), bytes, cudaMemcpyHostToDevice, stream), "upload Sobol V");
    cuda_check(cudaMemcpyAsync(nt->VT.p, VT.data(), bytes, cudaMemcpyHostToDevice, stream), "upload Sobol VT");
    cuda_check(cudaMemcpyAsync(nt->LO.p, LO.data(), LO.size() * 4, cudaMemcpyHostToDevice, stream), "upload Sobol LO");
    cuda_check(cudaStreamSynchronize(stream), "Sobol tables");
    nt->dims = dims;
    t = std::move(nt);
    return *t;
}

// ---------------------------------------------------------------------------
// JIT: NVRTC -> cubin (cached by source), cudaLibrary per device
// ---------------------------------------------------------------------------

struct Cubin {
    std::vector<char> image;
    std::string log;
};

static std::mutex g_jit_mu;
static std::unordered_map<std::string, std::shared_ptr<Cubin>> g_cubins;

static std::shared_ptr<Cubin> compile_cubin(const std::string& gen_src, bool fp32) {
    std::string src = std::string(kEmbArgs) + "\n" + kEmbLog + "\n" + kEmbChacha + "\n" + kEmbShift + "\n" + kEmbRt +
                      "\n" + gen_src;
    const std::string key = std::string(fp32 ? "f32|" : "f64|") + src;
    {
        std::lock_guard<std::mutex> g(g_jit_mu);
        auto it = g_cubins.find(key);
        if (it != g_cubins.end()) return it->second;
    }
    nvrtcProgram prog;
    if (nvrtcCreateProgram(&prog, src.c_str(), "sde_plan.cu", 0, nullptr, nullptr) != NVRTC_SUCCESS)
        fail(SDE_ERR_COMPILE, "nvrtcCreateProgram failed");
    // 177: runtime helpers a given plan does not call
    std::vector<const char*> opts = {"--gpu-architecture=sm_103a", "--std=c++17", "-default-device",
                                     "--ptxas-options=-v", "--diag-suppress=177"};
    if (fp32) {
        opts.push_back("-ftz=true");
        opts.push_back("-prec-div=false");
        opts.push_back("-prec-sqrt=false");
        opts.push_back("-fmad=true");
    } else {
        // the reference never contracts a*b+c; keep every product rounded
        opts.push_back("-fmad=false");
    }
    nvrtcResult r = nvrtcCompileProgram(prog, (int)opts.size(), opts.data());
    auto c = std::make_shared<Cubin>();
    size_t ls = 0;
    nvrtcGetProgramLogSize(prog, &ls);
    c->log.resize(ls);
    if (ls) nvrtcGetProgramLog(prog, &c->log[0]);
    if (r != NVRTC_SUCCESS) {
        nvrtcDestroyProgram(&prog);
        fail(SDE_ERR_COMPILE, std::string("NVRTC: ") + nvrtcGetErrorString(r) + "\n" + c->log);
    }
    size_t cs = 0;
    nvrtcGetCUBINSize(prog, &cs);
    c->image.resize(cs);
    nvrtcGetCUBIN(prog, c->image.data());
    nvrtcDestroyProgram(&prog);
    std::lock_guard<std::mutex> g(g_jit_mu);
    g_cubins[key] = c;
    return c;
}

struct Loaded {
    cudaLibrary_t lib = nullptr;
    cudaKernel_t fwd = nullptr;
    cudaKernel_t adj = nullptr;
    cudaKernel_t chk = nullptr;  // chunked forward kernel for small runs
    cudaKernel_t wide = nullptr; // two paths per thread, for large runs
    cudaKernel_t wide_ug = nullptr;  // the same on a grid of equal steps
};

// ---------------------------------------------------------------------------
// plans and results
// ---------------------------------------------------------------------------

}  // namespace sde

struct sde_plan {
    sde::Universe u;
    sde::KernelSpec spec;
    int output = SDE_OUT_FULL;
    bool auto_block = true;  // block size chosen per run from the path count
    int mma_smem = 0;        // dynamic shared memory of a tensor-core forward kernel
    bool adjoint_recompute = false;  // adjoint: never keep the forward increments
    int chunked = SDE_CHUNKED_AUTO;  // small runs: the chunked kernel (when built)
    std::string chk_name;            // empty: the plan has no chunked kernel
    std::string wide_name;           // empty: the plan has no two-paths-per-thread kernel
    std::string wide_ug_name;        // its uniform-grid twin
    std::string source;
    std::string fwd_name, adj_name;
    std::shared_ptr<sde::Cubin> cubin;
    std::mutex mu;
    std::map<int, sde::Loaded> loaded;  // by device
};

namespace sde {
// The scenario, time and process columns of long rows depend only on the
// run's shape (replicates, paths, output slots and their times, processes,
// first scenario), not on its values.  Results of the same shape share one
// pinned copy of them, so a repeated drop-in call copies only its values.
struct LongIndex {
    uint64_t n_rep = 0, n_paths = 0, scen_base = 0;
    int n_out = 0, P = 0;
    std::vector<double> slot_times;
    HBuf block;  // [scenario i32][time f64][process i32], 8-byte aligned columns
    size_t o_time = 0, o_proc = 0, bytes = 0;
};
}  // namespace sde

struct sde_result {
    std::shared_ptr<sde_plan> plan_keep;  // keeps the plan alive for one-shot runs
    sde_plan* plan = nullptr;
    uint64_t n_paths = 0;
    int n_rep = 1, n_out = 0, P = 0, K = 0, elem = 8;
    uint64_t scen_base = 0;
    std::vector<int32_t> slot_tidx;
    std::vector<double> slot_times;
    sde::DBuf out;                 // engine-owned filtration
    void* out_ptr = nullptr;       // filtration (engine- or caller-owned)
    sde::DBuf args_dev;            // staged time grid etc.
    sde::DBuf partials, est_dev, masks, ckpt, inc;
    sde::HBuf est_host;
    sde::HBuf stage;               // pinned inputs, alive until the run is done
    sde::HBuf long_host;           // pinned long-format values (sde_result_long_host)
    std::shared_ptr<const sde::LongIndex> long_index;  // the shape's pinned index columns
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    sde::DBuf status;              // kernel status word (tensor-core waits)
    sde::HBuf status_host;
    bool waited = false;
    int kernel = SDE_KERNEL_NONE, block = 0, per_block = 0;  // what the run launched
};

namespace sde {

static Loaded& ensure_loaded(sde_plan* p) {
    int dev = 0;
    cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    std::lock_guard<std::mutex> g(p->mu);
    Loaded& L = p->loaded[dev];
    if (!L.lib) {
        cuda_check(cudaLibraryLoadData(&L.lib, p->cubin->image.data(), nullptr, nullptr, 0, nullptr,
                                       nullptr, 0),
                   "cudaLibraryLoadData");
        cuda_check(cudaLibraryGetKernel(&L.fwd, L.lib, p->fwd_name.c_str()), "cudaLibraryGetKernel");
        if (p->mma_smem > 0)
            cuda_check(cudaKernelSetAttributeForDevice(L.fwd, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                       p->mma_smem, dev),
                       "tensor-core kernel shared memory");
        if (p->spec.adjoint)
            cuda_check(cudaLibraryGetKernel(&L.adj, L.lib, p->adj_name.c_str()), "cudaLibraryGetKernel");
        if (!p->chk_name.empty())
            cuda_check(cudaLibraryGetKernel(&L.chk, L.lib, p->chk_name.c_str()), "cudaLibraryGetKernel");
        if (!p->wide_name.empty()) {
            cuda_check(cudaLibraryGetKernel(&L.wide, L.lib, p->wide_name.c_str()), "cudaLibraryGetKernel");
            cuda_check(cudaLibraryGetKernel(&L.wide_ug, L.lib, p->wide_ug_name.c_str()), "cudaLibraryGetKernel");
        }
    }
    return L;
}

static int n_estimates(const sde_plan* p) {
    return (int)(p->spec.payoffs.size() + p->spec.grad_params.size() + p->spec.grad_x0.size());
}

static KernelSpec spec_from(const sde_options* o) {
    KernelSpec s;
    s.scheme = o->scheme;
    s.rng = o->rng;
    s.scramble = o->scramble;
    s.precision = o->precision;
    s.semantics = o->semantics;
    s.store_output = o->output != SDE_OUT_NONE;
    s.block = o->block_size > 0 ? o->block_size : 256;
    if (s.scheme != SCHEME_EULER && s.scheme != SCHEME_RK) fail(SDE_ERR_INVALID, "unknown scheme");
    if (s.rng != RNG_PSEUDO && s.rng != RNG_SOBOL) fail(SDE_ERR_INVALID, "unknown rng");
    if (s.scramble != SCRAMBLE_SHIFT && s.scramble != SCRAMBLE_XOR) fail(SDE_ERR_INVALID, "unknown scramble");
    if (s.precision != PREC_FP64 && s.precision != PREC_FP32) fail(SDE_ERR_INVALID, "unknown precision");
    if (s.semantics != SEM_REFERENCE && s.semantics != SEM_TEXTBOOK) fail(SDE_ERR_INVALID, "unknown semantics");
    if (o->output < SDE_OUT_FULL || o->output > SDE_OUT_NONE) fail(SDE_ERR_INVALID, "unknown output mode");
    if (s.block % 32 != 0 || s.block > 1024) fail(SDE_ERR_INVALID, "block_size must be a multiple of 32 up to 1024");
    s.ckpt_every = o->ckpt_every > 0 ? o->ckpt_every : 19;
    s.ppt = o->paths_per_thread > 0 ? o->paths_per_thread : 1;
    // automatic: FP32 XOR-Sobol plans pick one or two paths per thread per run
    s.wide = o->paths_per_thread == 0 && o->block_size <= 0;
    s.icdf = o->icdf;
    if (s.icdf != SDE_ICDF_AS26 && s.icdf != SDE_ICDF_ACCURATE) fail(SDE_ERR_INVALID, "unknown icdf");
    s.tensor_cores = o->tensor_cores;
    if (s.tensor_cores != SDE_TC_OFF && s.tensor_cores != SDE_TC_ON && s.tensor_cores != SDE_TC_ON_ROW)
        fail(SDE_ERR_INVALID, "unknown tensor_cores");
    if (s.ppt != 1 && s.ppt != 2 && s.ppt != 4) fail(SDE_ERR_INVALID, "paths_per_thread must be 1, 2 or 4");
    if (s.ckpt_every > 256) fail(SDE_ERR_INVALID, "ckpt_every must be at most 256");
    return s;
}

static sde_plan* plan_create(const std::vector<std::string>& eqs, const std::vector<std::string>& params,
                             const std::vector<std::string>& payoffs, const sde_options& o,
                             const std::vector<std::string>* grad_params = nullptr,
                             const std::vector<std::string>* grad_x0 = nullptr) {
    auto p = std::make_unique<sde_plan>();
    p->u = parse_universe(eqs, params);
    p->spec = spec_from(&o);
    p->output = o.output;
    p->auto_block = o.block_size <= 0;
    if (o.adjoint_recompute != 0 && o.adjoint_recompute != 1) fail(SDE_ERR_INVALID, "adjoint_recompute must be 0 or 1");
    p->adjoint_recompute = o.adjoint_recompute == 1;
    if (o.chunked != SDE_CHUNKED_AUTO && o.chunked != SDE_CHUNKED_ON && o.chunked != SDE_CHUNKED_OFF)
        fail(SDE_ERR_INVALID, "unknown chunked");
    p->chunked = o.chunked;
    for (const auto& s : payoffs) p->spec.payoffs.push_back(p->u.resolve(parse_expression(s)));
    if (grad_params || grad_x0) {
        if (p->spec.payoffs.empty()) fail(SDE_ERR_INVALID, "an adjoint plan needs a payoff");
        if (!p->u.alg.empty()) fail(SDE_ERR_UNSUPPORTED, "the adjoint does not take algebraic processes");
        p->spec.adjoint = true;
        for (const auto& g : *grad_params) {
            int k = -1;
            for (int i = 0; i < (int)p->u.params.size(); ++i)
                if (p->u.params[i] == g) k = i;
            if (k < 0) fail(SDE_ERR_INVALID, "gradient parameter '" + g + "' is not a declared parameter");
            p->spec.grad_params.push_back(k);
        }
        for (const auto& g : *grad_x0) {
            int k = p->u.process_index(g);
            if (k < 0) fail(SDE_ERR_INVALID, "gradient initial value '" + g + "' is not a process");
            p->spec.grad_x0.push_back(k);
        }
    }
    if (n_estimates(p.get()) > 32) fail(SDE_ERR_INVALID, "at most 32 payoffs and gradients");
    if (p->spec.tensor_cores) {
        // tcgen05 lowering where the universe allows it; the CUDA-core
        // kernel otherwise
        const MmaShape m = mma_shape(p->u, p->spec);
        if (m.eligible) {
            p->spec.block = 128 * m.split;  // one MMA row per path, one or two threads per path
            p->auto_block = false;
            p->mma_smem = m.smem_bytes;
        } else {
            p->spec.tensor_cores = 0;
        }
    }
    p->fwd_name = forward_kernel_name(p->spec);
    p->adj_name = adjoint_kernel_name(p->spec);
    if (has_chunked_kernel(p->u, p->spec) && p->chunked != SDE_CHUNKED_OFF) p->chk_name = chunked_kernel_name(p->spec);
    if (has_wide_kernel(p->u, p->spec)) {
        p->wide_name = forward_kernel_name(wide_spec(p->spec));
        p->wide_ug_name = forward_kernel_name(wide_ugrid_spec(p->spec));
    }
    p->source = generate_source(p->u, p->spec);
    p->cubin = compile_cubin(p->source, p->spec.precision == PREC_FP32);
    return p.release();
}

static sde_result* run(sde_plan* p, const sde_run_args& a) {
    const Universe& u = p->u;
    const int P = u.n_processes(), NI = u.n_stochastic(), T = a.n_times;
    if (T < 1 || !a.times) fail(SDE_ERR_INVALID, "need at least one time point");
    for (int t = 1; t < T; ++t)
        if (!(a.times[t] > a.times[t - 1])) fail(SDE_ERR_INVALID, "time_steps must be strictly increasing");
    if (a.n_replicates < 1) fail(SDE_ERR_INVALID, "n_replicates must be >= 1");
    if (a.n_replicates > 65535) fail(SDE_ERR_INVALID, "at most 65535 replicates");
    if (a.n_params != (int)u.params.size()) fail(SDE_ERR_INVALID, "parameter count does not match the plan");
    if (a.n_x0 > P) fail(SDE_ERR_INVALID, "more initial values than processes");
    if (p->spec.scheme == SCHEME_RK && NI == 0 && T > 1)
        fail(SDE_ERR_RNG_INDEX, "RNG Index 0 out of bounds (max 0)");
    const uint64_t N = a.n_paths;
    const uint64_t total = N * (uint64_t)a.n_replicates;
    const bool sobol = p->spec.rng == RNG_SOBOL;
    const bool xorm = sobol && p->spec.scramble == SCRAMBLE_XOR;
    const uint64_t dims_needed = (uint64_t)(T - 1) * NI;
    if (sobol && dims_needed > (uint64_t)kSobolMaxDims)
        fail(SDE_ERR_UNSUPPORTED, "Sobol sequence needs " + std::to_string(dims_needed) +
                                      " dimensions; the Joe-Kuo table has " + std::to_string(kSobolMaxDims));
    if (sobol && !xorm && a.path_offset + total + 5 > (1ull << 32))
        fail(SDE_ERR_UNSUPPORTED, "Sobol point index beyond 2^32");
    if (xorm && N > (1ull << 32)) fail(SDE_ERR_UNSUPPORTED, "more than 2^32 Sobol points per replicate");
    // the adjoint kernel steps one path per thread
    const int ppt_eff = p->spec.adjoint ? 1 : p->spec.ppt;
    int block = p->spec.block;
    int dev = 0, sms = 148;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint64_t warps = (N + 32ull * ppt_eff - 1) / (32ull * ppt_eff) * (uint64_t)a.n_replicates;
    if (p->auto_block) {
        // few paths (the reference's 10,000): spread the warps over every SM
        // rather than filling a few with 8-warp blocks
        const uint64_t wpb = std::min<uint64_t>(8, std::max<uint64_t>(1, (warps + sms - 1) / std::max(1, sms)));
        block = (int)(32 * wpb);
    }
    // the chunked kernel (8 warps per 32 paths) when one thread per path
    // would give fewer than 4 warps per SM
    const bool use_chk = !p->chk_name.empty() && !p->spec.adjoint &&
                         (p->chunked == SDE_CHUNKED_ON || warps < 4ull * (uint64_t)std::max(1, sms));
    if (use_chk) block = 256;
    // a tensor-core CTA steps 128 paths (one MMA tile) with 128 or 256 threads
    const bool tc_plan = p->spec.tensor_cores && !p->spec.adjoint;
    // two paths per thread in CTAs of 128 from 64 such warps per SM (about
    // 0.6M paths on GB300): 3% faster on Heston at 2^20 x 4 and 2^18 x 16
    // paths; runs of up to 2^18 paths are 10-15% faster with one
    const bool use_wide = !p->wide_name.empty() && !use_chk && !tc_plan &&
                          (N + 63) / 64 * (uint64_t)a.n_replicates >= 64ull * (uint64_t)std::max(1, sms);
    if (use_wide) block = 128;
    const uint64_t per_block = tc_plan ? 128ull : use_chk ? 32ull : use_wide ? 256ull : (uint64_t)block * ppt_eff;
    const uint64_t gx = (N + per_block - 1) / per_block;
    if (gx > 0x7fffffffull) fail(SDE_ERR_INVALID, "too many paths for one launch");

    // output slots
    std::vector<int32_t> slots;
    switch (p->output) {
    case SDE_OUT_FULL:
        for (int t = 0; t < T; ++t) slots.push_back(t);
        break;
    case SDE_OUT_CHECKPOINTS:
        for (int k = 0; k < a.n_checkpoints; ++k) {
            int t = a.checkpoints[k];
            if (t < 0 || t >= T) fail(SDE_ERR_INVALID, "checkpoint index out of range");
            if (!slots.empty() && t <= slots.back()) fail(SDE_ERR_INVALID, "checkpoints must be increasing");
            slots.push_back(t);
        }
        break;
    case SDE_OUT_TERMINAL:
        slots.push_back(T - 1);
        break;
    default:
        break;
    }
    if (p->spec.adjoint) slots.clear();  // adjoint runs return estimators only

    auto r = std::make_unique<sde_result>();
    r->plan = p;
    r->n_paths = N;
    r->n_rep = a.n_replicates;
    r->n_out = (int)slots.size();
    r->P = P;
    r->K = n_estimates(p);
    r->elem = p->spec.precision == PREC_FP32 ? 4 : 8;
    r->scen_base = a.path_offset;
    r->slot_tidx = slots;
    for (int t : slots) r->slot_times.push_back(a.times[t]);
    r->stream = (cudaStream_t)a.stream;

    Loaded& L = ensure_loaded(p);

    // stage the small inputs in one pinned block and copy them in one go
    const int Tm1 = std::max(1, T - 1);
    const size_t nd = (size_t)T + 2 * Tm1 + std::max(1, P) + std::max<size_t>(1, u.params.size());
    const size_t nf = (size_t)T + 2 * Tm1;
    const size_t bytes = nd * 8 + nf * 4 + (size_t)T * 4 + 64;
    r->stage = HBuf(bytes);
    char* h = r->stage.as<char>();
    double* hd = (double*)h;
    double* h_times = hd;
    double* h_dts = h_times + T;
    double* h_sdts = h_dts + Tm1;
    double* h_x0 = h_sdts + Tm1;
    double* h_par = h_x0 + std::max(1, P);
    float* hf = (float*)(hd + nd);
    float* h_times_f = hf;
    float* h_dts_f = hf + T;
    float* h_sdts_f = h_dts_f + Tm1;
    int32_t* h_tidx = (int32_t*)(hf + nf);
    for (int t = 0; t < T; ++t) {
        h_times[t] = a.times[t];
        h_times_f[t] = (float)a.times[t];
        h_tidx[t] = -1;
    }
    bool ugrid = T > 1;  // every FP32 step and its square root equal
    for (int t = 0; t + 1 < T; ++t) {
        h_dts[t] = a.times[t + 1] - a.times[t];
        h_sdts[t] = std::sqrt(a.times[t + 1] - a.times[t]);
        h_dts_f[t] = (float)h_dts[t];
        h_sdts_f[t] = (float)h_sdts[t];
        ugrid = ugrid && h_dts_f[t] == h_dts_f[0] && h_sdts_f[t] == h_sdts_f[0];
    }
    for (int q = 0; q < std::max(1, P); ++q) h_x0[q] = (a.x0 && q < a.n_x0) ? a.x0[q] : 0.0;
    for (size_t k = 0; k < u.params.size(); ++k) h_par[k] = a.params[k];
    for (size_t s = 0; s < slots.size(); ++s) h_tidx[slots[s]] = (int32_t)s;
    r->args_dev = DBuf(bytes);
    cuda_check(cudaMemcpyAsync(r->args_dev.p, h, bytes, cudaMemcpyHostToDevice, r->stream), "stage inputs");
    char* d = r->args_dev.as<char>();
    auto dptr = [&](const void* hp) { return d + ((const char*)hp - h); };

    sde_args A;
    std::memset(&A, 0, sizeof A);
    A.times = (const double*)dptr(h_times);
    A.dts = (const double*)dptr(h_dts);
    A.sqrt_dts = (const double*)dptr(h_sdts);
    A.times_f = (const float*)dptr(h_times_f);
    A.dts_f = (const float*)dptr(h_dts_f);
    A.sqrt_dts_f = (const float*)dptr(h_sdts_f);
    A.x0 = (const double*)dptr(h_x0);
    A.params = (const double*)dptr(h_par);
    A.out_tidx = (const int*)dptr(h_tidx);
    A.n_paths = N;
    A.path_base = a.path_offset;
    A.seed = a.seed;
    A.T = T;
    A.n_out = r->n_out;
    A.n_rep = a.n_replicates;
    if (ugrid) {
        A.udt_f = h_dts_f[0];
        A.usdt_f = h_sdts_f[0];
    }

    if (sobol) {
        SobolTables& st = sobol_tables(r->stream);
        A.sobol_v = st.V.as<sde_u32>();
        A.sobol_vt = st.VT.as<sde_u32>();
        A.sobol_lo = st.LO.as<sde_u32>();
        A.sobol_dims = st.dims;
        if (xorm) {
            const int stride = (int)((dims_needed + 31) / 32 * 32);
            r->masks = DBuf((size_t)stride * a.n_replicates * 4 + 4);
            cuda_check(launch_make_xor_masks(r->masks.as<sde_u32>(), a.n_replicates, stride, a.seed, r->stream),
                       "XOR masks");
            A.masks = r->masks.as<sde_u32>();
            A.mask_stride = stride;
        }
    }

    // filtration buffer
    const size_t out_bytes = (size_t)r->n_out * P * N * a.n_replicates * r->elem;
    if (r->n_out > 0 && P > 0 && N > 0) {
        if (a.device_out) {
            if (a.device_out_bytes < out_bytes)
                fail(SDE_ERR_INVALID, "device_out is smaller than the filtration (" + std::to_string(out_bytes) + " bytes)");
            r->out_ptr = a.device_out;
        } else {
            r->out = DBuf(out_bytes);
            r->out_ptr = r->out.p;
        }
    }
    A.out = r->out_ptr;

    if (r->K > 0) {
        r->partials = DBuf((size_t)a.n_replicates * gx * r->K * 4 * 8 + 8);
        r->est_dev = DBuf((size_t)a.n_replicates * r->K * 2 * 8);
        r->est_host = HBuf((size_t)a.n_replicates * r->K * 2 * 8);
        A.partials = r->partials.as<double>();
    }

    if (p->spec.adjoint) {
        // checkpoints [rep][n_ckpt][PS][path]: the state at every
        // ckpt_every-th step; Runge-Kutta in the reference's semantics also
        // carries the name->value cache that the next step's stage 1 reads
        // (PS = 2P), the other schemes the P processes
        const bool rk = p->spec.scheme == SCHEME_RK;
        const int PS = (rk && p->spec.semantics == SEM_REFERENCE ? 2 : 1) * std::max(1, P);
        const int E = p->spec.ckpt_every;
        A.ckpt_every = E;
        A.n_ckpt = std::max(1, (T - 1 + E - 1) / E);
        r->ckpt = DBuf((size_t)A.n_ckpt * PS * N * a.n_replicates * r->elem + 8);
        A.ckpt = r->ckpt.as<float>();
        // the forward pass's increments (and Runge-Kutta's sign)
        // [rep][T-1][NI (+1)][path], kept for the reverse sweep when they fit
        // in a quarter of the free memory (the sweep otherwise draws them
        // again: ChaCha blocks and normals)
        const size_t inc_bytes = (size_t)(T - 1) * (NI + (rk && NI > 0 ? 1 : 0)) * N * a.n_replicates * r->elem;
        size_t free_b = 0, total_b = 0;
        if (!p->adjoint_recompute && inc_bytes > 0 && cudaMemGetInfo(&free_b, &total_b) == cudaSuccess &&
            inc_bytes <= free_b / 4) {
            r->inc = DBuf(inc_bytes);
            A.inc = r->inc.p;
        }
    }

    const bool tc = tc_plan;
    if (tc && N > 0) {
        r->status = DBuf(16);
        r->status_host = HBuf(16);
        *r->status_host.as<int>() = 0;
        cuda_check(cudaMemsetAsync(r->status.p, 0, 16, r->stream), "status word");
        A.status = r->status.as<int>();
        A.tc_wait_cycles = g_tc_wait_cycles.load(std::memory_order_relaxed);
    }

    if (N > 0 && T >= 1) {
        r->kernel = p->spec.adjoint ? SDE_KERNEL_ADJOINT : use_chk ? SDE_KERNEL_CHUNKED : use_wide ? SDE_KERNEL_WIDE
                    : tc ? SDE_KERNEL_TENSOR_CORES : SDE_KERNEL_FORWARD;
        r->block = block;
        r->per_block = (int)per_block;
        void* kargs[] = {&A};
        cuda_check(cudaLaunchKernel((const void*)(p->spec.adjoint ? L.adj : use_chk ? L.chk
                                                  : use_wide ? (ugrid ? L.wide_ug : L.wide) : L.fwd),
                                    dim3((unsigned)gx, (unsigned)a.n_replicates), dim3(block), kargs,
                                    tc ? (size_t)p->mma_smem : 0, r->stream),
                   "step kernel launch");
        if (tc)
            cuda_check(cudaMemcpyAsync(r->status_host.p, r->status.p, 4, cudaMemcpyDeviceToHost, r->stream),
                       "status D2H");
        if (r->K > 0) {
            cuda_check(launch_reduce_partials(r->partials.as<double>(), (int)gx, r->K, a.n_replicates,
                                              r->est_dev.as<double>(), r->stream),
                       "estimator reduction");
            cuda_check(cudaMemcpyAsync(r->est_host.p, r->est_dev.p, (size_t)a.n_replicates * r->K * 2 * 8,
                                       cudaMemcpyDeviceToHost, r->stream),
                       "estimates D2H");
        }
    } else if (r->K > 0) {
        std::memset(r->est_host.p, 0, (size_t)a.n_replicates * r->K * 2 * 8);
    }
    cuda_check(cudaEventCreateWithFlags(&r->done, cudaEventDisableTiming), "cudaEventCreate");
    cuda_check(cudaEventRecord(r->done, r->stream), "cudaEventRecord");
    return r.release();
}

static void wait(sde_result* r) {
    if (!r->waited) {
        cuda_check(cudaEventSynchronize(r->done), "kernel execution");
        r->waited = true;
    }
    if (r->status_host.p && *r->status_host.as<int>() != 0)
        fail(SDE_ERR_DEVICE, "a tensor-core wait in the step kernel timed out; the run's values are not valid");
}

}  // namespace sde

// ===========================================================================
// C ABI
// ===========================================================================

using namespace sde;

extern "C" {

int32_t sde_abi_version(void) { return SDE_ABI_VERSION; }

int sde_debug_tc_wait_cycles(uint64_t cycles) {
    g_tc_wait_cycles.store(cycles, std::memory_order_relaxed);
    return SDE_OK;
}

int sde_last_error(char* buf, size_t n) {
    if (!buf || n == 0) return SDE_ERR_INVALID;
    std::snprintf(buf, n, "%s", g_last_error.c_str());
    return SDE_OK;
}

void sde_options_init(sde_options* o) {
    if (!o) return;
    std::memset(o, 0, sizeof *o);
    o->struct_size = sizeof *o;
    o->scheme = SDE_SCHEME_EULER;
    o->rng = SDE_RNG_PSEUDO;
    o->scramble = SDE_SCRAMBLE_SHIFT;
    o->precision = SDE_FP64;
    o->semantics = SDE_SEM_REFERENCE;
    o->output = SDE_OUT_FULL;
}

void sde_run_args_init(sde_run_args* a) {
    if (!a) return;
    std::memset(a, 0, sizeof *a);
    a->struct_size = sizeof *a;
    a->n_replicates = 1;
}

static std::mutex g_sim_mu;
static std::list<std::pair<std::string, std::shared_ptr<sde_plan>>> g_sim_plans;  // most recent first

static std::vector<std::string> strs(const char* const* s, int n) {
    std::vector<std::string> v;
    for (int i = 0; i < n; ++i) {
        if (!s || !s[i]) fail(SDE_ERR_INVALID, "NULL string");
        v.emplace_back(s[i]);
    }
    return v;
}

int sde_plan_create(const char* const* equations, int32_t n_equations, const char* const* param_names,
                    int32_t n_params, const char* const* payoffs, int32_t n_payoffs,
                    const sde_options* opts, sde_plan** out_plan) {
    return guarded([&] {
        if (!out_plan) fail(SDE_ERR_INVALID, "out_plan is NULL");
        *out_plan = nullptr;
        if (n_equations < 0 || n_params < 0 || n_payoffs < 0) fail(SDE_ERR_INVALID, "negative count");
        sde_options o;
        sde_options_init(&o);
        if (opts) {
            if (opts->struct_size != sizeof(sde_options)) fail(SDE_ERR_INVALID, "sde_options.struct_size mismatch");
            o = *opts;
        }
        *out_plan = plan_create(strs(equations, n_equations), strs(param_names, n_params),
                                strs(payoffs, n_payoffs), o);
    });
}

int sde_plan_create_adjoint(const char* const* equations, int32_t n_equations, const char* const* param_names,
                            int32_t n_params, const char* const* payoffs, int32_t n_payoffs,
                            const char* const* grad_params, int32_t n_grad_params, const char* const* grad_x0,
                            int32_t n_grad_x0, const sde_options* opts, sde_plan** out_plan) {
    return guarded([&] {
        if (!out_plan) fail(SDE_ERR_INVALID, "out_plan is NULL");
        *out_plan = nullptr;
        if (n_equations < 0 || n_params < 0 || n_payoffs < 0 || n_grad_params < 0 || n_grad_x0 < 0)
            fail(SDE_ERR_INVALID, "negative count");
        sde_options o;
        sde_options_init(&o);
        if (opts) {
            if (opts->struct_size != sizeof(sde_options)) fail(SDE_ERR_INVALID, "sde_options.struct_size mismatch");
            o = *opts;
        }
        auto gp = strs(grad_params, n_grad_params);
        auto gx = strs(grad_x0, n_grad_x0);
        *out_plan = plan_create(strs(equations, n_equations), strs(param_names, n_params),
                                strs(payoffs, n_payoffs), o, &gp, &gx);
    });
}

int sde_plan_n_estimates(const sde_plan* p, int32_t* n) {
    return guarded([&] {
        if (!p || !n) fail(SDE_ERR_INVALID, "NULL argument");
        *n = n_estimates(p);
    });
}

int sde_plan_destroy(sde_plan* p) {
    return guarded([&] {
        if (!p) return;
        for (auto& kv : p->loaded)
            if (kv.second.lib) {
                int cur = 0;
                cudaGetDevice(&cur);
                cudaSetDevice(kv.first);
                cudaLibraryUnload(kv.second.lib);
                cudaSetDevice(cur);
            }
        delete p;
    });
}

int sde_plan_n_processes(const sde_plan* p, int32_t* n) {
    return guarded([&] {
        if (!p || !n) fail(SDE_ERR_INVALID, "NULL argument");
        *n = p->u.n_processes();
    });
}

int sde_plan_n_stochastic(const sde_plan* p, int32_t* n) {
    return guarded([&] {
        if (!p || !n) fail(SDE_ERR_INVALID, "NULL argument");
        *n = p->u.n_stochastic();
    });
}

int sde_plan_process_name(const sde_plan* p, int32_t i, char* buf, size_t n) {
    return guarded([&] {
        if (!p || !buf) fail(SDE_ERR_INVALID, "NULL argument");
        if (i < 0 || i >= p->u.n_processes()) fail(SDE_ERR_INVALID, "process index out of range");
        std::snprintf(buf, n, "%s", p->u.procs[i].name.c_str());
    });
}

int sde_plan_process_index(const sde_plan* p, const char* name, int32_t* index) {
    return guarded([&] {
        if (!p || !name || !index) fail(SDE_ERR_INVALID, "NULL argument");
        *index = p->u.process_index(name);
    });
}

int sde_plan_stochastic_token(const sde_plan* p, int32_t i, char* buf, size_t n) {
    return guarded([&] {
        if (!p || !buf) fail(SDE_ERR_INVALID, "NULL argument");
        if (i < 0 || i >= p->u.n_stochastic()) fail(SDE_ERR_INVALID, "stochastic index out of range");
        std::snprintf(buf, n, "%s", p->u.tokens[i].c_str());
    });
}

int sde_plan_source(const sde_plan* p, char* buf, size_t n, size_t* needed) {
    return guarded([&] {
        if (!p) fail(SDE_ERR_INVALID, "NULL plan");
        if (needed) *needed = p->source.size() + 1;
        if (buf && n) std::snprintf(buf, n, "%s", p->source.c_str());
    });
}

int sde_plan_compile_log(const sde_plan* p, char* buf, size_t n, size_t* needed) {
    return guarded([&] {
        if (!p) fail(SDE_ERR_INVALID, "NULL plan");
        const std::string& s = p->cubin->log;
        if (needed) *needed = s.size() + 1;
        if (buf && n) std::snprintf(buf, n, "%s", s.c_str());
    });
}

int sde_plan_tensor_cores(const sde_plan* p, int32_t* on) {
    return guarded([&] {
        if (!p || !on) fail(SDE_ERR_INVALID, "NULL argument");
        *on = p->spec.tensor_cores && !p->spec.adjoint ? 1 : 0;
    });
}

int sde_run(sde_plan* p, const sde_run_args* a, sde_result** out) {
    return guarded([&] {
        if (!p || !a || !out) fail(SDE_ERR_INVALID, "NULL argument");
        if (a->struct_size != sizeof(sde_run_args)) fail(SDE_ERR_INVALID, "sde_run_args.struct_size mismatch");
        *out = nullptr;
        *out = run(p, *a);
    });
}

int sde_simulate(const char* const* equations, int32_t n_equations, const double* times, int32_t n_times,
                 const char* const* init_names, const double* init_values, int32_t n_init,
                 uint64_t n_scenarios, const char* scheme, const char* rng_method, uint64_t seed,
                 int32_t has_seed, sde_result** out) {
    return guarded([&] {
        if (!out || !scheme || !rng_method) fail(SDE_ERR_INVALID, "NULL argument");
        *out = nullptr;
        sde_options o;
        sde_options_init(&o);
        if (std::strcmp(scheme, "euler") == 0) o.scheme = SDE_SCHEME_EULER;
        else if (std::strcmp(scheme, "runge-kutta") == 0) o.scheme = SDE_SCHEME_RK;
        else fail(SDE_ERR_INVALID, std::string("unknown scheme '") + scheme + "'");
        o.rng = std::strcmp(rng_method, "sobol") == 0 ? SDE_RNG_SOBOL : SDE_RNG_PSEUDO;
        // the one-shot entry keeps recently lowered universes: repeated calls
        // with the same equations skip parsing, lowering and module loading
        const auto eqs = strs(equations, n_equations);
        std::string key = std::to_string(o.scheme) + "|" + std::to_string(o.rng);
        for (const auto& e : eqs) key += "\x1f" + e;
        std::shared_ptr<sde_plan> plan;
        {
            std::lock_guard<std::mutex> g(g_sim_mu);
            for (auto it = g_sim_plans.begin(); it != g_sim_plans.end(); ++it)
                if (it->first == key) {
                    plan = it->second;
                    g_sim_plans.splice(g_sim_plans.begin(), g_sim_plans, it);
                    break;
                }
        }
        if (!plan) {
            plan.reset(plan_create(eqs, {}, {}, o));
            std::lock_guard<std::mutex> g(g_sim_mu);
            g_sim_plans.emplace_front(key, plan);
            if (g_sim_plans.size() > 16) g_sim_plans.pop_back();
        }
        std::vector<double> x0(std::max(1, plan->u.n_processes()), 0.0);
        for (int k = 0; k < n_init; ++k) {
            int idx = plan->u.process_index(init_names[k]);
            if (idx >= 0) x0[idx] = init_values[k];
        }
        if (!has_seed) {
            std::random_device rd;
            seed = ((uint64_t)rd() << 32) ^ rd();
        }
        sde_run_args a;
        sde_run_args_init(&a);
        a.times = times;
        a.n_times = n_times;
        a.x0 = x0.data();
        a.n_x0 = plan->u.n_processes();
        a.n_paths = n_scenarios;
        a.seed = seed;
        sde_result* r = run(plan.get(), a);
        r->plan_keep = plan;
        *out = r;
    });
}

int sde_result_destroy(sde_result* r) {
    return guarded([&] {
        if (!r) return;
        if (r->done) {
            cudaEventSynchronize(r->done);
            cudaEventDestroy(r->done);
        }
        delete r;
    });
}

int sde_result_wait(sde_result* r) {
    return guarded([&] {
        if (!r) fail(SDE_ERR_INVALID, "NULL result");
        wait(r);
    });
}

int sde_result_shape(const sde_result* r, uint64_t* n_paths, int32_t* n_out, int32_t* n_proc, int32_t* n_rep) {
    return guarded([&] {
        if (!r) fail(SDE_ERR_INVALID, "NULL result");
        if (n_paths) *n_paths = r->n_paths;
        if (n_out) *n_out = r->n_out;
        if (n_proc) *n_proc = r->P;
        if (n_rep) *n_rep = r->n_rep;
    });
}

int sde_result_time_indices(const sde_result* r, int32_t* out) {
    return guarded([&] {
        if (!r || !out) fail(SDE_ERR_INVALID, "NULL argument");
        std::copy(r->slot_tidx.begin(), r->slot_tidx.end(), out);
    });
}

int sde_result_device_values(const sde_result* r, void** dptr, int32_t* elem) {
    return guarded([&] {
        if (!r || !dptr) fail(SDE_ERR_INVALID, "NULL argument");
        *dptr = r->out_ptr;
        if (elem) *elem = r->elem;
    });
}

int sde_result_copy_values(sde_result* r, double* host, int32_t layout) {
    return guarded([&] {
        if (!r || !host) fail(SDE_ERR_INVALID, "NULL argument");
        const size_t n = (size_t)r->n_rep * r->n_paths * r->n_out * r->P;
        if (n == 0) return;
        if (!r->out_ptr) fail(SDE_ERR_INVALID, "the plan stores no filtration");
        if (layout == SDE_LAYOUT_DEVICE) {
            wait(r);
            if (r->elem == 8) {
                cuda_check(cudaMemcpy(host, r->out_ptr, n * 8, cudaMemcpyDeviceToHost), "D2H");
            } else {
                std::vector<float> tmp(n);
                cuda_check(cudaMemcpy(tmp.data(), r->out_ptr, n * 4, cudaMemcpyDeviceToHost), "D2H");
                for (size_t i = 0; i < n; ++i) host[i] = tmp[i];
            }
            return;
        }
        if (layout != SDE_LAYOUT_REFERENCE) fail(SDE_ERR_INVALID, "unknown layout");
        DBuf val(n * 8);
        cuda_check(launch_long_export(r->out_ptr, r->elem, r->n_paths, r->n_out, r->P, r->n_rep, nullptr,
                                      0, nullptr, nullptr, nullptr, val.as<double>(), r->stream),
                   "export");
        cuda_check(cudaMemcpyAsync(host, val.p, n * 8, cudaMemcpyDeviceToHost, r->stream), "D2H");
        cuda_check(cudaStreamSynchronize(r->stream), "D2H");
        r->waited = true;
    });
}

int sde_result_copy_long(sde_result* r, int32_t* scen, double* time, int32_t* proc, double* value) {
    return guarded([&] {
        if (!r) fail(SDE_ERR_INVALID, "NULL result");
        const size_t n = (size_t)r->n_rep * r->n_paths * r->n_out * r->P;
        if (n == 0) return;
        if (!r->out_ptr) fail(SDE_ERR_INVALID, "the plan stores no filtration");
        DBuf st(std::max<size_t>(1, r->slot_times.size()) * 8);
        cuda_check(cudaMemcpyAsync(st.p, r->slot_times.data(), r->slot_times.size() * 8, cudaMemcpyHostToDevice,
                                   r->stream),
                   "slot times");
        DBuf ds(scen ? n * 4 : 0), dt(time ? n * 8 : 0), dp(proc ? n * 4 : 0), dv(value ? n * 8 : 0);
        cuda_check(launch_long_export(r->out_ptr, r->elem, r->n_paths, r->n_out, r->P, r->n_rep,
                                      st.as<double>(), r->scen_base, ds.as<int32_t>(), dt.as<double>(),
                                      dp.as<int32_t>(), dv.as<double>(), r->stream),
                   "long export");
        if (scen) cuda_check(cudaMemcpyAsync(scen, ds.p, n * 4, cudaMemcpyDeviceToHost, r->stream), "D2H");
        if (time) cuda_check(cudaMemcpyAsync(time, dt.p, n * 8, cudaMemcpyDeviceToHost, r->stream), "D2H");
        if (proc) cuda_check(cudaMemcpyAsync(proc, dp.p, n * 4, cudaMemcpyDeviceToHost, r->stream), "D2H");
        if (value) cuda_check(cudaMemcpyAsync(value, dv.p, n * 8, cudaMemcpyDeviceToHost, r->stream), "D2H");
        cuda_check(cudaStreamSynchronize(r->stream), "D2H");
        r->waited = true;
    });
}

namespace sde {
static std::mutex g_lix_mu;
static std::list<std::shared_ptr<LongIndex>> g_lix;  // most recent first
static const size_t kLixMaxEntries = 8, kLixMaxBytes = (size_t)1 << 30;

// The shape's index columns: from the cache, or exported on the result's
// stream and copied into a new pinned block (then cached, least recently
// used entries leaving beyond 8 shapes or 1 GiB; results keep theirs alive).
static std::shared_ptr<const LongIndex> long_index(sde_result* r, size_t n) {
    {
        std::lock_guard<std::mutex> g(g_lix_mu);
        for (auto it = g_lix.begin(); it != g_lix.end(); ++it) {
            const LongIndex& e = **it;
            if (e.n_rep == (uint64_t)r->n_rep && e.n_paths == r->n_paths && e.n_out == r->n_out && e.P == r->P &&
                e.scen_base == r->scen_base && e.slot_times == r->slot_times) {
                auto hit = *it;
                g_lix.erase(it);
                g_lix.push_front(hit);
                return hit;
            }
        }
    }
    auto e = std::make_shared<LongIndex>();
    e->n_rep = r->n_rep;
    e->n_paths = r->n_paths;
    e->scen_base = r->scen_base;
    e->n_out = r->n_out;
    e->P = r->P;
    e->slot_times = r->slot_times;
    e->o_time = (n * 4 + 7) / 8 * 8;
    e->o_proc = e->o_time + n * 8;
    e->bytes = e->o_proc + n * 4;
    e->block = HBuf(e->bytes);
    DBuf st(std::max<size_t>(1, r->slot_times.size()) * 8);
    cuda_check(cudaMemcpyAsync(st.p, r->slot_times.data(), r->slot_times.size() * 8, cudaMemcpyHostToDevice, r->stream),
               "slot times");
    DBuf d(e->bytes);
    char* dd = d.as<char>();
    cuda_check(launch_long_export(r->out_ptr, r->elem, r->n_paths, r->n_out, r->P, r->n_rep, st.as<double>(),
                                  r->scen_base, (int32_t*)dd, (double*)(dd + e->o_time), (int32_t*)(dd + e->o_proc),
                                  nullptr, r->stream),
               "long export (index columns)");
    cuda_check(cudaMemcpyAsync(e->block.p, dd, e->bytes, cudaMemcpyDeviceToHost, r->stream), "D2H");
    cuda_check(cudaStreamSynchronize(r->stream), "D2H");
    std::lock_guard<std::mutex> g(g_lix_mu);
    g_lix.push_front(e);
    size_t total = 0, kept = 0;
    for (auto it = g_lix.begin(); it != g_lix.end();) {
        total += (*it)->bytes;
        if (++kept > kLixMaxEntries || (kept > 1 && total > kLixMaxBytes)) {
            it = g_lix.erase(it);
        } else {
            ++it;
        }
    }
    return e;
}
}  // namespace sde

int sde_result_long_host(sde_result* r, const int32_t** scen, const double** time, const int32_t** proc,
                         const double** value, uint64_t* n_rows) {
    return guarded([&] {
        if (!r || !scen || !time || !proc || !value || !n_rows) fail(SDE_ERR_INVALID, "NULL argument");
        const size_t n = (size_t)r->n_rep * r->n_paths * r->n_out * r->P;
        *n_rows = n;
        if (n == 0) {
            *scen = nullptr; *time = nullptr; *proc = nullptr; *value = nullptr;
            return;
        }
        if (!r->out_ptr) fail(SDE_ERR_INVALID, "the plan stores no filtration");
        if (!r->long_host.p) {
            // the values: exported on the device and copied once into a
            // pinned block the result owns; the index columns are the shape's
            r->long_index = long_index(r, n);
            r->long_host = HBuf(n * 8);
            DBuf dv(n * 8);
            cuda_check(launch_long_export(r->out_ptr, r->elem, r->n_paths, r->n_out, r->P, r->n_rep, nullptr, 0,
                                          nullptr, nullptr, nullptr, dv.as<double>(), r->stream),
                       "long export");
            cuda_check(cudaMemcpyAsync(r->long_host.p, dv.p, n * 8, cudaMemcpyDeviceToHost, r->stream), "D2H");
            cuda_check(cudaStreamSynchronize(r->stream), "D2H");
            r->waited = true;
        }
        const char* h = r->long_index->block.as<char>();
        *scen = (const int32_t*)h;
        *time = (const double*)(h + r->long_index->o_time);
        *proc = (const int32_t*)(h + r->long_index->o_proc);
        *value = r->long_host.as<const double>();
    });
}

int sde_result_launch_info(const sde_result* r, int32_t* kernel, int32_t* block, int32_t* per_block) {
    return guarded([&] {
        if (!r) fail(SDE_ERR_INVALID, "NULL result");
        if (kernel) *kernel = r->kernel;
        if (block) *block = r->block;
        if (per_block) *per_block = r->per_block;
    });
}

int sde_result_estimates(sde_result* r, double* sum, double* sumsq) {
    return guarded([&] {
        if (!r) fail(SDE_ERR_INVALID, "NULL result");
        wait(r);
        const double* e = r->est_host.as<double>();
        for (int i = 0; i < r->n_rep * r->K; ++i) {
            if (sum) sum[i] = e[2 * i];
            if (sumsq) sumsq[i] = e[2 * i + 1];
        }
    });
}

int sde_kat_chacha8_u64(uint64_t seed, uint64_t first, uint64_t n, uint64_t* host_out) {
    return guarded([&] {
        if (!host_out && n) fail(SDE_ERR_INVALID, "NULL output");
        DBuf d(n * 8);
        cuda_check(launch_kat_chacha8(seed, first, n, d.as<sde_u64>(), nullptr), "chacha8 kernel");
        cuda_check(cudaMemcpy(host_out, d.p, n * 8, cudaMemcpyDeviceToHost), "D2H");
    });
}

int sde_kat_sobol_points(int32_t dims, uint64_t first, uint64_t n, uint32_t* host_out) {
    return guarded([&] {
        if (dims < 1 || dims > kSobolMaxDims) fail(SDE_ERR_INVALID, "dims out of range");
        if (first + n > (1ull << 32)) fail(SDE_ERR_UNSUPPORTED, "Sobol index beyond 2^32");
        SobolTables& st = sobol_tables(nullptr);
        DBuf d(n * dims * 4);
        cuda_check(launch_kat_sobol(st.V.as<sde_u32>(), dims, first, n, d.as<sde_u32>(), nullptr), "sobol kernel");
        cuda_check(cudaMemcpy(host_out, d.p, n * dims * 4, cudaMemcpyDeviceToHost), "D2H");
    });
}

int sde_kat_icdf(const double* host_p, uint64_t n, double* host_out) {
    return guarded([&] {
        DBuf dp(n * 8), dq(n * 8);
        cuda_check(cudaMemcpy(dp.p, host_p, n * 8, cudaMemcpyHostToDevice), "H2D");
        cuda_check(launch_kat_icdf(dp.as<double>(), n, dq.as<double>(), nullptr), "icdf kernel");
        cuda_check(cudaMemcpy(host_out, dq.p, n * 8, cudaMemcpyDeviceToHost), "D2H");
    });
}

int sde_sobol_directions(int32_t dims, uint32_t* host_out) {
    return guarded([&] {
        if (dims < 1 || dims > kSobolMaxDims) fail(SDE_ERR_INVALID, "dims out of range");
        if (!host_out) fail(SDE_ERR_INVALID, "NULL output");
        sobol_directions_host(dims, host_out);
    });
}

int sde_probe_sfu_peak(double* ops) {
    return guarded([&] {
        if (!ops) fail(SDE_ERR_INVALID, "NULL output");
        cuda_check(run_sfu_probe(ops), "SFU probe");
    });
}

int sde_probe_chacha8_rate(double* blocks) {
    return guarded([&] {
        if (!blocks) fail(SDE_ERR_INVALID, "NULL output");
        cuda_check(run_chacha_probe(blocks), "ChaCha8 probe");
    });
}

}  // extern "C"

namespace sde {

int plan_view(sde_plan* p, PlanView* v) {
    return guarded([&] {
        if (!p || !v) fail(SDE_ERR_INVALID, "NULL argument");
        Loaded& L = ensure_loaded(p);
        v->kernel = (void*)L.fwd;
        v->n_processes = p->u.n_processes();
        v->n_stochastic = p->u.n_stochastic();
        v->n_payoffs = (int)p->spec.payoffs.size();
        v->n_params = (int)p->u.params.size();
        v->block = p->spec.block;
        v->ppt = p->spec.ppt;
        v->rng = p->spec.rng;
        v->scheme = p->spec.scheme;
        v->adjoint = p->spec.adjoint ? 1 : 0;
        v->tensor_cores = p->spec.tensor_cores ? 1 : 0;
    });
}

void set_last_error(const std::string& msg) { g_last_error = msg; }

}  // namespace sde

// ===========================================================================
// Batched instances: one persistent work-queue kernel over many instances
// ===========================================================================

namespace sde {

// The batched adjoint template checkpoints every ceil(sqrt(steps)) steps in
// per-thread arrays of 64 checkpoints and 64 steps.
constexpr int kBatchAdjointMaxSteps = 64 * 64;

// candidate (block, paths per thread) shapes the autotuner times
static const std::vector<std::pair<int, int>> kBatchVariants = {
    {128, 1}, {256, 1}, {128, 2}, {256, 2}, {128, 4}};

}  // namespace sde

struct sde_batch {
    std::vector<sde::Universe> u;
    std::vector<sde::KernelSpec> specs;
    int K = 0;
    bool fp32 = true;
    std::string source;
    std::shared_ptr<sde::Cubin> cubin;
    struct Dev {
        cudaLibrary_t lib = nullptr;
        std::vector<cudaKernel_t> kernels;  // per variant
        std::vector<int> grid;              // persistent grid per variant
    };
    std::mutex mu;
    std::map<int, Dev> dev;
};

struct sde_batch_job {
    sde_batch* b = nullptr;
    int n_inst = 0, n_items = 0, variant = 0;
    uint64_t path_steps = 0;
    sde::DBuf inst, items, x0, params, counter, item_partials, ranges, est;
    sde::HBuf est_host;
    sde_batch_args args{};
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t done = nullptr;
};

namespace sde {

static sde_batch::Dev& batch_loaded(sde_batch* b) {
    int dev = 0, sms = 0;
    cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    std::lock_guard<std::mutex> g(b->mu);
    auto& D = b->dev[dev];
    if (D.lib) return D;
    cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count");
    cuda_check(cudaLibraryLoadData(&D.lib, b->cubin->image.data(), nullptr, nullptr, 0, nullptr, nullptr, 0),
               "cudaLibraryLoadData");
    for (const auto& v : kBatchVariants) {
        cudaKernel_t k;
        cuda_check(cudaLibraryGetKernel(&k, D.lib, batch_kernel_name(v.first, v.second).c_str()),
                   "cudaLibraryGetKernel");
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void*)k, v.first, 0) != cudaSuccess ||
            per_sm < 1) {
            cudaGetLastError();
            per_sm = 2048 / v.first;
        }
        D.kernels.push_back(k);
        D.grid.push_back(per_sm * sms);
    }
    return D;
}

// Work items for one (block, ppt) shape: chunks of block*ppt paths, the
// instances with the most steps first so the queue drains evenly.
static void build_items(sde_batch_job* j, const sde_batch_instances& in, int variant, cudaStream_t s) {
    const int chunk = kBatchVariants[variant].first * kBatchVariants[variant].second;
    std::vector<int> order(in.n_instances);
    for (int i = 0; i < in.n_instances; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return in.n_steps[a] > in.n_steps[b]; });
    std::vector<sde_batch_item> items;
    std::vector<int> ranges(2 * (size_t)in.n_instances);
    for (int i : order) {
        ranges[2 * i] = (int)items.size();
        for (uint64_t f = 0; f < in.n_paths[i]; f += chunk) items.push_back({f, i, 0});
        ranges[2 * i + 1] = (int)items.size();
    }
    j->n_items = (int)items.size();
    j->variant = variant;
    j->items = DBuf(std::max<size_t>(1, items.size()) * sizeof(sde_batch_item));
    j->ranges = DBuf(ranges.size() * sizeof(int) + 8);
    j->item_partials = DBuf(std::max<size_t>(1, items.size()) * j->b->K * 4 * 8);
    if (!items.empty())
        cuda_check(cudaMemcpyAsync(j->items.p, items.data(), items.size() * sizeof(sde_batch_item),
                                   cudaMemcpyHostToDevice, s), "items H2D");
    cuda_check(cudaMemcpyAsync(j->ranges.p, ranges.data(), ranges.size() * sizeof(int), cudaMemcpyHostToDevice, s),
               "ranges H2D");
    cuda_check(cudaStreamSynchronize(s), "items");
    j->args.items = j->items.as<sde_batch_item>();
    j->args.item_partials = j->item_partials.as<double>();
    j->args.n_items = j->n_items;
}

static void batch_enqueue(sde_batch_job* j, cudaStream_t s) {
    auto& D = batch_loaded(j->b);
    cuda_check(cudaMemsetAsync(j->counter.p, 0, sizeof(unsigned), s), "queue reset");
    void* kargs[] = {&j->args};
    const auto& v = kBatchVariants[j->variant];
    cuda_check(cudaLaunchKernel((const void*)D.kernels[j->variant], dim3((unsigned)D.grid[j->variant]),
                                dim3(v.first), kargs, 0, s),
               "batch kernel launch");
    cuda_check(launch_reduce_ranges(j->item_partials.as<double>(), j->ranges.as<int>(), j->n_inst, j->b->K,
                                    j->est.as<double>(), s),
               "batch reduction");
    cuda_check(cudaMemcpyAsync(j->est_host.p, j->est.p, (size_t)j->n_inst * j->b->K * 16, cudaMemcpyDeviceToHost, s),
               "batch results D2H");
}

static float time_variant(sde_batch_job* j, cudaStream_t s) {
    cudaEvent_t e0, e1;
    cuda_check(cudaEventCreate(&e0), "event");
    cuda_check(cudaEventCreate(&e1), "event");
    batch_enqueue(j, s);  // warm
    float best = 1e30f;
    for (int r = 0; r < 2; ++r) {
        cuda_check(cudaEventRecord(e0, s), "event");
        batch_enqueue(j, s);
        cuda_check(cudaEventRecord(e1, s), "event");
        cuda_check(cudaEventSynchronize(e1), "autotune run");
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        best = std::min(best, ms);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return best;
}

}  // namespace sde

extern "C" {

int sde_batch_create(const sde_plan* const* templates, int32_t n_templates, sde_batch** out) {
    return guarded([&] {
        if (!out || !templates || n_templates < 1) fail(SDE_ERR_INVALID, "need at least one template");
        *out = nullptr;
        auto b = std::make_unique<sde_batch>();
        std::vector<const Universe*> us;
        for (int t = 0; t < n_templates; ++t) {
            const sde_plan* p = templates[t];
            if (!p) fail(SDE_ERR_INVALID, "NULL template");
            if (p->spec.rng != RNG_PSEUDO) fail(SDE_ERR_UNSUPPORTED, "batched templates use the pseudo-random streams");
            if (t > 0 && p->spec.precision != templates[0]->spec.precision)
                fail(SDE_ERR_INVALID, "batched templates must share one precision");
            if (p->spec.scheme == SCHEME_RK && p->u.n_stochastic() == 0)
                fail(SDE_ERR_RNG_INDEX, "RNG Index 0 out of bounds (max 0)");
            b->u.push_back(p->u);
            b->specs.push_back(p->spec);
            // an adjoint template's estimates: its payoffs, then the
            // gradients of payoff 0 (as its plan's runs return them)
            b->K = std::max(b->K, (int)(p->spec.payoffs.size() + p->spec.grad_params.size() + p->spec.grad_x0.size()));
        }
        if (b->K < 1) fail(SDE_ERR_INVALID, "batched templates need at least one payoff");
        for (auto& u : b->u) us.push_back(&u);
        b->fp32 = templates[0]->spec.precision == PREC_FP32;
        b->source = generate_batch_source(us, b->specs, kBatchVariants, b->K);
        b->cubin = compile_cubin(b->source, b->fp32);
        *out = b.release();
    });
}

int sde_batch_destroy(sde_batch* b) {
    return guarded([&] {
        if (!b) return;
        for (auto& kv : b->dev)
            if (kv.second.lib) cudaLibraryUnload(kv.second.lib);
        delete b;
    });
}

int sde_batch_prepare(sde_batch* b, const sde_batch_instances* in, int32_t autotune, void* stream,
                      sde_batch_job** out) {
    return guarded([&] {
        if (!b || !in || !out) fail(SDE_ERR_INVALID, "NULL argument");
        if (in->struct_size != sizeof(sde_batch_instances)) fail(SDE_ERR_INVALID, "sde_batch_instances.struct_size mismatch");
        *out = nullptr;
        cudaStream_t s = (cudaStream_t)stream;
        const int n = in->n_instances;
        if (n < 1) fail(SDE_ERR_INVALID, "no instances");
        auto j = std::make_unique<sde_batch_job>();
        j->b = b;
        j->n_inst = n;
        std::vector<sde_batch_inst> hi(n);
        int maxP = 1, maxK = 1;
        for (auto& u : b->u) {
            maxP = std::max(maxP, u.n_processes());
            maxK = std::max(maxK, (int)u.params.size());
        }
        if (in->x0_stride < maxP && in->x0) fail(SDE_ERR_INVALID, "x0_stride is smaller than a template's process count");
        for (int i = 0; i < n; ++i) {
            const int t = in->template_id[i];
            if (t < 0 || t >= (int)b->u.size()) fail(SDE_ERR_INVALID, "template_id out of range");
            if (in->n_steps[i] < 1) fail(SDE_ERR_INVALID, "n_steps must be >= 1");
            if (b->specs[t].adjoint && in->n_steps[i] > kBatchAdjointMaxSteps)
                fail(SDE_ERR_UNSUPPORTED, "a batched adjoint instance takes at most " +
                                              std::to_string(kBatchAdjointMaxSteps) + " steps");
            if (!(in->t_end[i] > 0)) fail(SDE_ERR_INVALID, "t_end must be positive");
            if ((int)b->u[t].params.size() > in->param_stride)
                fail(SDE_ERR_INVALID, "param_stride is smaller than a template's parameter count");
            const double dt = in->t_end[i] / in->n_steps[i];
            hi[i].dt = dt;
            hi[i].sdt = std::sqrt(dt);
            hi[i].dt_f = (float)dt;
            hi[i].sdt_f = (float)std::sqrt(dt);
            hi[i].n_paths = in->n_paths[i];
            hi[i].seed = in->seed[i];
            hi[i].tmpl = t;
            hi[i].n_steps = in->n_steps[i];
            hi[i].x0_off = i * in->x0_stride;
            hi[i].par_off = i * in->param_stride;
            j->path_steps += in->n_paths[i] * (uint64_t)in->n_steps[i];
        }
        const size_t nx = (size_t)n * std::max(1, in->x0_stride), np = (size_t)n * std::max(1, in->param_stride);
        j->inst = DBuf(n * sizeof(sde_batch_inst));
        j->x0 = DBuf(nx * 8);
        j->params = DBuf(np * 8);
        j->counter = DBuf(16);
        j->est = DBuf((size_t)n * b->K * 16);
        j->est_host = HBuf((size_t)n * b->K * 16);
        std::vector<double> zx(nx, 0.0), zp(np, 0.0);
        if (in->x0) std::copy(in->x0, in->x0 + (size_t)n * in->x0_stride, zx.begin());
        if (in->params) std::copy(in->params, in->params + (size_t)n * in->param_stride, zp.begin());
        cuda_check(cudaMemcpyAsync(j->inst.p, hi.data(), n * sizeof(sde_batch_inst), cudaMemcpyHostToDevice, s), "H2D");
        cuda_check(cudaMemcpyAsync(j->x0.p, zx.data(), nx * 8, cudaMemcpyHostToDevice, s), "H2D");
        cuda_check(cudaMemcpyAsync(j->params.p, zp.data(), np * 8, cudaMemcpyHostToDevice, s), "H2D");
        j->args.inst = j->inst.as<sde_batch_inst>();
        j->args.x0 = j->x0.as<double>();
        j->args.params = j->params.as<double>();
        j->args.counter = j->counter.as<unsigned>();
        batch_loaded(b);
        int best = 0;
        if (autotune < 0) {
            // a fixed candidate, -1 - autotune (tests of each shape)
            best = -1 - autotune;
            if (best >= (int)kBatchVariants.size()) fail(SDE_ERR_INVALID, "no such candidate shape");
        } else if (autotune) {
            float best_ms = 1e30f;
            for (int v = 0; v < (int)kBatchVariants.size(); ++v) {
                build_items(j.get(), *in, v, s);
                const float ms = time_variant(j.get(), s);
                if (ms < best_ms) { best_ms = ms; best = v; }
            }
        }
        build_items(j.get(), *in, best, s);
        // capture reset + persistent kernel + reduction + D2H in one graph
        cudaStream_t cap = nullptr;
        cuda_check(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking), "capture stream");
        cuda_check(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal), "begin capture");
        try {
            batch_enqueue(j.get(), cap);
        } catch (...) {
            cudaGraph_t g;
            cudaStreamEndCapture(cap, &g);
            cudaStreamDestroy(cap);
            throw;
        }
        cuda_check(cudaStreamEndCapture(cap, &j->graph), "end capture");
        cudaStreamDestroy(cap);
        cuda_check(cudaGraphInstantiate(&j->exec, j->graph, 0), "graph instantiate");
        cuda_check(cudaEventCreateWithFlags(&j->done, cudaEventDisableTiming), "event");
        *out = j.release();
    });
}

int sde_batch_job_run(sde_batch_job* j, void* stream) {
    return guarded([&] {
        if (!j) fail(SDE_ERR_INVALID, "NULL job");
        cudaStream_t s = (cudaStream_t)stream;
        cuda_check(cudaGraphLaunch(j->exec, s), "graph launch");
        cuda_check(cudaEventRecord(j->done, s), "event");
    });
}

int sde_batch_job_results(sde_batch_job* j, double* sum, double* sumsq) {
    return guarded([&] {
        if (!j) fail(SDE_ERR_INVALID, "NULL job");
        cuda_check(cudaEventSynchronize(j->done), "batch execution");
        const double* e = j->est_host.as<double>();
        for (int i = 0; i < j->n_inst * j->b->K; ++i) {
            if (sum) sum[i] = e[2 * i];
            if (sumsq) sumsq[i] = e[2 * i + 1];
        }
    });
}

int sde_batch_job_info(const sde_batch_job* j, int32_t* block, int32_t* ppt, int32_t* n_items, uint64_t* path_steps,
                       int32_t* n_payoffs) {
    return guarded([&] {
        if (!j) fail(SDE_ERR_INVALID, "NULL job");
        if (block) *block = kBatchVariants[j->variant].first;
        if (ppt) *ppt = kBatchVariants[j->variant].second;
        if (n_items) *n_items = j->n_items;
        if (path_steps) *path_steps = j->path_steps;
        if (n_payoffs) *n_payoffs = j->b->K;
    });
}

int sde_batch_job_destroy(sde_batch_job* j) {
    return guarded([&] {
        if (!j) return;
        if (j->done) {
            cudaEventSynchronize(j->done);
            cudaEventDestroy(j->done);
        }
        if (j->exec) cudaGraphExecDestroy(j->exec);
        if (j->graph) cudaGraphDestroy(j->graph);
        delete j;
    });
}

}  // extern "C"
