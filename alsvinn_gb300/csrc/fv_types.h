// Types shared by the kernel translation units and the C-ABI layer: grid
// geometry, the device-resident step state and the launch argument blocks.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

namespace gbfv {

enum Recon { RC_NONE = 0, RC_WENO2 = 1, RC_ENO2 = 2, RC_ENO3 = 3, RC_ENO4 = 4, RC_MC = 5, RC_MM = 6, RC_WENOF2 = 7 };

enum Mode { MODE_L = 0, MODE_RK3_S1 = 1, MODE_RK3_S2 = 2, MODE_RK2_S1 = 3 };

// Device-resident step state shared by the per-step kernels (one per solve).
struct StepState {
    unsigned long long ws_bits[3];  // max face wave speed per direction (non-negative doubles)
    double t;                       // current time
    double dt;                      // dt of the step in flight
    double scale;                   // dt / dx.x
    long long steps;                // steps performed
    long long number_saved;         // FixedIntervalWriter counter (starts at 1)
    int status;                     // 0 ok, 1 constraint violated
    int failed_step;                // first step whose state broke the constraints
    int done;                       // 1: the advance has reached its end; kernels return at once
    int parity;                     // ensemble RK2: which of the two state buffers holds the state
    double end_time;                // advance target time
    long long step_limit;           // advance step limit (< 0: none)
    int just_done;                  // ensemble: reached end_time in the step just finished
    int group;                      // ensemble: statistics group (< 0: none)
    long long number_saved2;        // second save clamp's counter (FixedIntervalStatistics, starts at 1)
    int saved_mask;                 // bit k: save counter k advanced in the step just finished
    float scale_f;                  // scale rounded to float once, for the FP32 kernels
    int just_saved;                 // ensemble: save index reached in the step just finished (-1: none)
};

// The step's dt (Integrator::computeTimestep, alsfvm/src/integrator/
// Integrator.cpp:20-46: cfl over the sum of wave speed / cell length over the
// active directions) clamped to the next save time of up to two fixed
// intervals (FixedIntervalWriter::adjustTimestep, alsfvm/src/io/
// FixedIntervalWriter.cpp:45-53; FixedIntervalStatistics::adjustTimestep,
// alsuq/src/stats/FixedIntervalStatistics.cpp:33-41); stores dt and dt / dx.x.
__device__ __forceinline__ void set_step_dt(StepState& S, int dim, const double* cell_lengths, double cfl,
                                            double interval, double interval2) {
    double ws[3];
    for (int d = 0; d < 3; ++d) ws[d] = d < dim ? __longlong_as_double((long long)S.ws_bits[d]) : 0.0;
    double waveSpeedTotal = 0;
    for (int d = 0; d < 3; ++d) {
        if (cell_lengths[d] == 0) continue;
        waveSpeedTotal += ws[d] / cell_lengths[d];
    }
    double dt = cfl / waveSpeedTotal;
    if (interval > 0) {
        const double nextSaveTime = (double)S.number_saved * interval + 0.0;
        const double lim = nextSaveTime - S.t;
        dt = lim < dt ? lim : dt;
    }
    if (interval2 > 0) {
        const double nextSaveTime = (double)S.number_saved2 * interval2;
        const double lim = nextSaveTime - S.t;
        dt = lim < dt ? lim : dt;
    }
    S.dt = dt;
    S.scale = dt / cell_lengths[0];
    S.scale_f = (float)S.scale;
}

struct StepParams {
    double cfl;
    double cell_lengths[3];
    double end_time;
    double time_interval;       // 0: no save-time clamp
    int dim;
    double time_interval2 = 0;  // second clamp (statistics save times); 0: none
    int stop_at_save = 0;       // end the advance after a step that reached a save time
};

// Tile of one CTA of the stage kernels and the CTA's thread count, per
// dimension and arithmetic variant (0 fp64, 1 fp64 exact, 2 fp32, 3 fp64 state
// with double-float arithmetic). A tile of T cells per direction needs
// T_d + 2 reconstructions and T_d + 1 face fluxes along each direction d
// (times the other extents). These are the default configurations (candidate
// 0; the autotuner's other candidates are registered in fv_variant.cu): the
// FP64 and FP32 kernels use 32 x 8 tiles, one thread per cell; the
// double-float kernel, bound by barrier waits, uses a
// 16 x 12 tile on 256 threads, which keeps each reconstruction and flux phase
// within one pass of the threads (a second, nearly empty pass leaves most
// warps waiting at the next barrier). Threads past the tile's cells join the
// reconstruction and flux phases only.
template <int DIM, int VAR> struct TileShape;
// (1D: 160 threads for 128 cells, so the 130 reconstructions and 129 faces of
// a tile take one pass of the threads; on small grids the stage time is the
// per-thread chain of FP64 instructions, which a second pass would double)
template <int VAR> struct TileShape<1, VAR> { static constexpr int X = 128, Y = 1, Z = 1, THREADS = 160; };
template <int VAR> struct TileShape<2, VAR> { static constexpr int X = 32, Y = 8, Z = 1, THREADS = 256; };
template <> struct TileShape<2, 3> { static constexpr int X = 16, Y = 12, Z = 1, THREADS = 256; };
template <int VAR> struct TileShape<3, VAR> { static constexpr int X = 8, Y = 8, Z = 4, THREADS = 256; };

template <int VAR> inline int tile_extent_v(int dim, int axis) {
    const int shapes[3][3] = {{TileShape<1, VAR>::X, TileShape<1, VAR>::Y, TileShape<1, VAR>::Z},
                              {TileShape<2, VAR>::X, TileShape<2, VAR>::Y, TileShape<2, VAR>::Z},
                              {TileShape<3, VAR>::X, TileShape<3, VAR>::Y, TileShape<3, VAR>::Z}};
    return shapes[dim - 1][axis];
}
inline int tile_extent(int variant, int dim, int axis) {
    switch (variant) {
        case 0: return tile_extent_v<0>(dim, axis);
        case 1: return tile_extent_v<1>(dim, axis);
        case 2: return tile_extent_v<2>(dim, axis);
        default: return tile_extent_v<3>(dim, axis);
    }
}

struct Grid {
    int n[3];   // interior cells
    int g[3];   // ghosts per dimension (0 in inactive dimensions)
    int t[3];   // padded extents
    long long total;
    int dim;
};

// Padded index of (x, y, z). Arrays below 2^31 cells per variable (every
// grid up to ~1290^3) take 32-bit products: GB300 runs 64-bit integer
// multiplies on its narrow FP64 pipe, which the stage kernels otherwise keep
// free for FP64 arithmetic.
__device__ __forceinline__ long long gidx(const Grid& G, int x, int y, int z) {
    if (G.total < (1LL << 31)) return (long long)((z * G.t[1] + y) * G.t[0] + x);
    return ((long long)z * G.t[1] + y) * G.t[0] + x;
}

// Padded positions holding the value of interior cell i (interior
// coordinate) along one dimension: slot 0 the cell itself, slots 1 and 2 its
// ghost images (Neumann mirror: alsfvm/include/alsfvm/boundary/Neumann.hpp:
// 24-35; periodic wrap: Periodic.hpp:24-42). Returns the mask of valid slots
// (bit 0 always). Fixed slots keep the positions in registers.
__device__ __forceinline__ int images(int i, int n, int g, bool periodic, int pos[3]) {
    pos[0] = i + g;
    pos[1] = 0;
    pos[2] = 0;
    int mask = 1;
    if (g > 0) {
        if (i < g) {
            pos[1] = periodic ? i + g + n : g - 1 - i;
            mask |= 2;
        }
        if (i >= n - g) {
            pos[2] = periodic ? i + g - n : 2 * n + g - 1 - i;
            mask |= 4;
        }
    }
    return mask;
}

// Stores one cell's values at its position and every ghost image of it.
template <class R, int NV>
__device__ __forceinline__ void store_with_images(R* out, long long total, const Grid& G, int ix, int iy, int iz,
                                                  bool periodic, const R* v) {
    int px[3], py[3], pz[3];
    const int xm = images(ix, G.n[0], G.g[0], periodic, px);
    const int ym = images(iy, G.n[1], G.g[1], periodic, py);
    const int zm = images(iz, G.n[2], G.g[2], periodic, pz);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (!((zm >> a) & 1)) continue;
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            if (!((ym >> b) & 1)) continue;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                if (!((xm >> c) & 1)) continue;
                const long long gi = gidx(G, px[c], py[b], pz[a]);
#pragma unroll
                for (int k = 0; k < NV; ++k) out[k * total + gi] = v[k];
            }
        }
    }
}


// Tensor maps of one single-grid stage launch, passed by value as a
// __grid_constant__ kernel parameter (TMA halo staging): the stage input and,
// for the stage-1 modes, the stage-0 flux difference L0.
struct TmaMaps {
    CUtensorMap in;
    CUtensorMap l0;
};

struct StageArgs {
    const void* in;   // U (MODE_L, MODE_RK3_S2) or U0 (stage-1 modes)
    const void* u0;   // U0 for the combination
    const void* l0;   // L0 for stage-1 modes
    void* out;
    const CUtensorMap* tm_in;  // tensor maps of in and l0 (TMA staging; null: plain loads)
    const CUtensorMap* tm_l0;
    StepState* st;
    Grid G;
    double gamma;
    float gamma_f;    // gamma rounded to float once, for the FP32 kernels
    int mode;
    int periodic;
    int check;        // run the constraint check on the output
    // region calls of the operator (region_kernel, MODE_L only): the cells
    // [rlo, rhi) in interior coordinates, read from and written to one
    // array per variable
    int rlo[3];
    int rhi[3];
    const void* vin[5];
    void* vout[5];
    // single-grid TMA stages: bytes announced on the halo barrier beyond the
    // copies' (0; nonzero only in a test of the bounded wait's error path)
    unsigned tma_extra_tx;
    // single-grid stages reading / writing a host state in place (null:
    // none): MODE_L writes its input cells, with their ghost images, to
    // copy_in (the device copy of a state read from mapped host memory);
    // a combination stage writes its output to out2 as well as to out
    void* copy_in;
    void* out2;
};

// Reconstruction of one direction over the reference's cell range
// (cells [g-1, t-g+1) along dir, interior in the other dimensions; every cell
// for the "none" reconstruction, which copies the whole volume).
struct ReconArgs {
    const void* in;
    void* left;
    void* right;
    Grid G;
    int dir;
    double gamma;  // for reconstructions in primitive variables
    int start[3];  // offsets of the cell range's lower / upper ends (the
    int end[3];    // reference's start / end; 0: the whole range)
};

// Constraint check over every padded cell (ghosts included, as the reference
// scans the whole volume); sets *flag to 0 when a cell fails.
struct CheckArgs {
    const void* in;
    int* flag;
    Grid G;
    double gamma;
};

// One member of an ensemble: its grid and its three state-sized buffers.
struct BatchMember {
    void* u;  // state (padded)
    void* v;  // second state buffer
    void* l;  // stage-0 flux difference
    Grid G;
    int tma;  // the member's tensor maps (u, v, l) are valid for the launch's halo box
};

// Arguments of one ensemble stage launch. tiles[i] = (member, ox, oy, oz);
// the tile count is read from device memory so a captured graph stays valid
// when members join or leave.
struct BatchArgs {
    const BatchMember* members;
    StepState* states;
    const int4* tiles;
    const int* ntiles;
    const CUtensorMap* maps;  // per member slot s: maps[3 s + {0, 1, 2}] of u, v, l
    double gamma;
    float gamma_f;
    int mode;
    int periodic;
};

}  // namespace gbfv
