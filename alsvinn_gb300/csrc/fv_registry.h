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

// Single-grid stage launch; `maps` holds the tensor maps of a.in and a.l0
// for the TMA-staged kernels (null otherwise).
typedef int (*StageLauncher)(const StageArgs& a, const TmaMaps* maps, cudaStream_t s);
typedef int (*ApplyLauncher)(const StageArgs& a, cudaStream_t s);

typedef int (*ReconLauncher)(const ReconArgs& a, cudaStream_t s);

// The operator on a region of cells (a.rlo, a.rhi, a.vin, a.vout; MODE_L).
typedef int (*RegionLauncher)(const StageArgs& a, cudaStream_t s);

typedef int (*CheckLauncher)(const CheckArgs& a, cudaStream_t s);

// Persistent ensemble stage launch: grid = ctas (0: one wave of resident CTAs).
typedef int (*BatchLauncher)(const BatchArgs& a, int ctas, cudaStream_t s);

// One compiled configuration of a scheme's stage kernels: the tile shape,
// the threads per CTA (a thread owns cells / threads cells when the tile has
// more cells than threads) and how the tile + halo reaches shared memory
// (TMA box copies or per-thread loads). Candidate 0 of every scheme is the
// default; the autotuner times the others on the caller's grid.
struct StageCandidate {
    StageLauncher stage;
    BatchLauncher batch;
    int tile[3];
    int threads;
    int tma;      // 1: the kernels stage the halo by TMA (needs tensor maps)
    int halo[3];  // TMA box: the tile plus the ghost halo in each active dimension
    int nv;       // variables per cell (the box's fourth extent)
    int min_blocks;  // resident CTAs per SM the single-grid kernel is compiled for
};
constexpr int kMaxCandidates = 8;

struct Registry {
    // [variant][equation][flux][recon][dim-1][candidate]
    StageCandidate cand[NUM_VARIANTS][NUM_EQ][NUM_FLUX][NUM_RECON][3][kMaxCandidates];
    int ncand[NUM_VARIANTS][NUM_EQ][NUM_FLUX][NUM_RECON][3];
    RegionLauncher region[NUM_VARIANTS][NUM_EQ][NUM_FLUX][NUM_RECON][3];
    ApplyLauncher apply[NUM_VARIANTS][NUM_EQ];
    ReconLauncher recon[NUM_VARIANTS][NUM_EQ][NUM_RECON];
    CheckLauncher check[NUM_VARIANTS][NUM_EQ];
};

Registry& registry();

// The candidates of one scheme (candidate 0 first); *count = 0 when the
// scheme has no kernel.
const StageCandidate* candidates(int var, int eq, int fl, int rc, int dim, int* count);

}  // namespace gbfv
