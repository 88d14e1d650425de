// engine_internal.h -- what other translation units of the library may see
// of a plan (engine.cpp owns the plan type).
#pragma once

#include <string>

struct sde_plan;

namespace sde {

struct PlanView {
    void* kernel;      // forward step kernel (cudaKernel_t) on the current device
    int n_processes;
    int n_stochastic;
    int n_payoffs;     // estimator columns of a forward run
    int n_params;
    int block;         // threads per block the kernel was lowered for
    int ppt;           // paths per thread
    int rng;           // RNG_PSEUDO / RNG_SOBOL
    int scheme;        // SCHEME_EULER / SCHEME_RK
    int adjoint;       // 1 for adjoint plans
    int tensor_cores;  // 1 if the forward kernel runs on tcgen05 (dynamic shared memory)
};

// Fills v for plan p, loading its module on the current device if needed.
// Returns an SDE_* status; on failure the message is the thread's last error.
int plan_view(sde_plan* p, PlanView* v);
void set_last_error(const std::string& msg);

}  // namespace sde
