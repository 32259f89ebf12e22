// Library-internal interface between the C-ABI translation units.
#pragma once
#include <cuda_runtime.h>

#include "fv_types.h"
#include "gbfv.h"

namespace gbfv {

// A validated descriptor: parsed names, variant, grid geometry.
struct GbfvPlan {
    int eq, fl, rc, in, periodic, var, nvar, elem;
    double gamma, cfl;
    double cell_lengths[3];
    Grid G;
};

}  // namespace gbfv

int gbfv_internal_fail(int code, const char* msg);
int gbfv_internal_plan(const gbfv_desc* d, gbfv::GbfvPlan* p);
int gbfv_internal_begin(gbfv::StepState* st, double end_time, long long step_limit, cudaStream_t q);
// Enqueues one time step on caller buffers: U state, V second state, L stage-0
// flux difference (each nvar * total values), st step state.
int gbfv_internal_prim_to_cons(const gbfv::GbfvPlan& p, const double* prim, double* cons);
int gbfv_internal_load_state(const gbfv::GbfvPlan& p, const double* host, void* dev, cudaStream_t q);
int gbfv_internal_step(const gbfv::GbfvPlan& p, void* U, void* V, void* L, gbfv::StepState* st,
                       const gbfv::StepParams& P, cudaStream_t q);

// Autotuner support (gbfv_tune.cu): GBFV_AUTOTUNE=0 in the environment
// disables tuning; the cache maps a scheme / grid key to the chosen candidate
// for the life of the process (thread safe).
int gbfv_autotune_enabled();
bool gbfv_tune_cache_get(const char* key, int* cand);
void gbfv_tune_cache_put(const char* key, int cand);
