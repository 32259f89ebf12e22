// Table of kernel launchers, filled by the per-variant translation units
// (fv_variant.cu compiled once per arithmetic variant and equation).
#pragma once
#include <cuda_runtime.h>

#include "fv_types.h"

namespace gbfv {

// Arithmetic variants of the step.
enum Variant { VAR_F64 = 0, VAR_F64_EXACT = 1, VAR_F32 = 2, VAR_F64_DF = 3, NUM_VARIANTS = 4 };
enum Equation { EQ_BURGERS = 0, EQ_EULER1 = 1, EQ_EULER2 = 2, EQ_EULER3 = 3, NUM_EQ = 4 };
enum Flux { FL_HLL = 0, FL_HLL3 = 1, FL_GODUNOV = 2, FL_CENTRAL = 3, FL_RUSANOV = 4, FL_ROE = 5, NUM_FLUX = 6 };
constexpr int NUM_RECON = 8;

// The fluxes each equation offers (alsfvm/include/alsfvm/numflux/
// numerical_flux_list.hpp:41-113): Euler hll, hll3, central; Burgers
// godunov, central, rusanov, roe.
inline bool flux_applies(int eq, int fl) {
    if (eq == EQ_BURGERS) return fl == FL_GODUNOV || fl == FL_CENTRAL || fl == FL_RUSANOV || fl == FL_ROE;
    return fl == FL_HLL || fl == FL_HLL3 || fl == FL_CENTRAL;
}

typedef int (*StageLauncher)(const StageArgs& a, cudaStream_t s);
typedef int (*ApplyLauncher)(const StageArgs& a, cudaStream_t s);

typedef int (*ReconLauncher)(const ReconArgs& a, cudaStream_t s);

typedef int (*CheckLauncher)(const CheckArgs& a, cudaStream_t s);

// Persistent ensemble stage launch: grid = ctas (0: one wave of resident CTAs).
typedef int (*BatchLauncher)(const BatchArgs& a, int ctas, cudaStream_t s);

struct Registry {
    // [variant][equation][flux][recon][dim-1]
    StageLauncher stage[NUM_VARIANTS][NUM_EQ][NUM_FLUX][NUM_RECON][3];
    ApplyLauncher apply[NUM_VARIANTS][NUM_EQ];
    ReconLauncher recon[NUM_VARIANTS][NUM_EQ][NUM_RECON];
    CheckLauncher check[NUM_VARIANTS][NUM_EQ];
    BatchLauncher batch[NUM_VARIANTS][NUM_EQ][NUM_FLUX][NUM_RECON][3];
    size_t stage_smem[NUM_VARIANTS][NUM_EQ][NUM_FLUX][NUM_RECON][3];
};

Registry& registry();

}  // namespace gbfv
