/* gbfv: GB300 finite-volume step and ensemble statistics, C ABI.
 *
 * A drop-in for the hot path of alsvinn's alsfvm explicit finite-volume step
 * (reconstruction, numerical flux, flux divergence, SSP Runge-Kutta stages,
 * ghost cells, CFL time step) and alsuq's mean/variance statistics, running on
 * one GB300 GPU. Plain pointers and sizes only; no C++ or torch types.
 *
 * Conventions
 *  - Every function returns 0 (GBFV_OK) or a negative gbfv_status; nothing
 *    throws across this boundary. gbfv_last_error() gives the message of the
 *    calling thread's last failure.
 *  - State layout is the reference Volume's: one padded array per conserved
 *    variable, x fastest, (nx+2g)(ny+2g)(nz+2g) values, ghost cells only in
 *    active dimensions, the nvar arrays back to back
 *    (alsfvm/src/volume/Volume.cpp:44-60, alsfvm/include/alsfvm/memory/View.hpp:116-118).
 *  - Host buffers are owned by the caller; device buffers named *_dev are
 *    device pointers owned by the caller; a handle owns its internal device
 *    state. A handle is used by one host thread at a time and issues its work
 *    on its own CUDA stream.
 *  - Names are the reference's XML spellings (alsfvm/src/config/SimulatorSetup.cpp:
 *    122-132): equation "euler1|euler2|euler3|burgers", flux "hll|hll3|godunov",
 *    reconstruction "none|weno2|eno2|eno3|eno4", integrator
 *    "forwardeuler|rungekutta2|rungekutta3", boundary "neumann|periodic".
 */
#ifndef GBFV_H
#define GBFV_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    GBFV_OK = 0,
    GBFV_ERR_ARGUMENT = -1,     /* bad name, size or pointer */
    GBFV_ERR_CUDA = -2,         /* a CUDA runtime call failed */
    GBFV_ERR_CONSTRAINT = -3,   /* the state broke rho > 0, p > 0 or finiteness */
    GBFV_ERR_MEMORY = -4,       /* device or host allocation failed */
    GBFV_ERR_UNSUPPORTED = -5   /* combination not provided */
} gbfv_status;

/* Arithmetic of the state and of the step. */
typedef enum {
    GBFV_FP64 = 0,        /* FP64 state, FP64 arithmetic: the drop-in path */
    GBFV_FP64_EXACT = 1,  /* FP64, reference operation order, no contraction:
                             bit-identical to the reference CPU path */
    GBFV_FP32 = 2,        /* FP32 state and arithmetic; dt, wave speeds and
                             statistics in FP64 */
    GBFV_FP64_DF = 3      /* FP64 state and FP64 Runge-Kutta update;
                             reconstruction and fluxes in double-float
                             (two FP32 numbers, ~48 bits) on the FP32 pipes */
} gbfv_precision;

typedef struct {
    const char* equation;
    const char* flux;
    const char* reconstruction;
    const char* integrator;
    const char* boundary;
    int n[3];             /* interior cells; 1 in inactive dimensions */
    double lower[3];      /* grid lower corner (Grid origin) */
    double upper[3];      /* grid upper corner */
    double gamma;         /* Euler gamma (EulerParameters, default 1.4) */
    double cfl;           /* CFL number */
    int precision;        /* gbfv_precision */
} gbfv_desc;

typedef struct gbfv_solver gbfv_solver;

const char* gbfv_last_error(void);
const char* gbfv_version(void);

/* Ghost cells the reference allocates for a reconstruction:
 * max(flux stencil - 1, reconstruction ghosts)
 * (replaces NumericalFluxCPU::getNumberOfGhostCells,
 * alsfvm/src/numflux/NumericalFluxCPU.cpp:226-231). */
int gbfv_ghost_cells(const char* reconstruction);

/* Number of conserved variables of an equation (3, 4, 5 or 1). */
int gbfv_num_variables(const char* equation);

/* ----------------------------------------------------------- solver */

/* Creates a solver: device state, scratch and stream for one grid
 * (replaces the Simulator construction, alsfvm/src/simulator/Simulator.cpp:26-64). */
int gbfv_create(const gbfv_desc* desc, gbfv_solver** out);
int gbfv_destroy(gbfv_solver* s);

/* Padded extents (t[3]) and total cells per variable. */
int gbfv_extents(const gbfv_solver* s, int t[3], long long* total);

/* Sets the state from interior primitive variables (rho, u..., p) or (u),
 * nvar * nx*ny*nz doubles, x fastest: converts to conserved variables and
 * fills the ghost cells (replaces Simulator::setInitialValue,
 * alsfvm/src/simulator/Simulator.cpp:117-162). Resets time and step count. */
int gbfv_set_primitive(gbfv_solver* s, const double* prim_host);

/* Sets / reads the padded conserved state (nvar * total doubles) from / to
 * host memory (replaces Simulator::setSimulationState, Simulator.cpp:104-107,
 * and the Volume copy to host). gbfv_set_state resets time and step count. */
int gbfv_set_state(gbfv_solver* s, const double* state_host);
int gbfv_get_state(gbfv_solver* s, double* state_host);

/* Device pointer of the current padded state (nvar * total values of the
 * solver's precision); valid until the next step. */
int gbfv_state_device(gbfv_solver* s, void** state_dev);

/* Advances up to max_steps time steps (max_steps <= 0: no step limit) or until
 * t >= end_time, whichever comes first (replaces the alsvinncli loop
 * `while (!atEnd()) performStep()`, alsvinncli/src/main.cpp:217-232, with
 * Simulator::performStep, Simulator.cpp:81-85, 191-214). number_of_saves > 0
 * attaches the FixedIntervalWriter dt clamp with interval end_time /
 * number_of_saves (alsfvm/src/io/FixedIntervalWriter.cpp:45-53); the clamp
 * persists across calls. Returns GBFV_ERR_CONSTRAINT if a step broke the
 * constraint check (CPUCellComputer::obeysConstraints). */
int gbfv_advance(gbfv_solver* s, double end_time, int number_of_saves, int max_steps);

/* A run schedule with the reference's two kinds of save-time clamp: the fvm
 * writer's FixedIntervalWriter (alsfvm/src/io/FixedIntervalWriter.cpp:32-53,
 * save k at k * save_interval[0]) and alsuq's FixedIntervalStatistics
 * (alsuq/src/stats/FixedIntervalStatistics.cpp:33-86, at k * save_interval[1]);
 * dt is clamped to the nearer next save time of each nonzero interval
 * (interval = endTime / numberOfSaves, as SimulatorSetup.cpp and Setup.cpp
 * form it). Both save counters start at 1 (the t = 0 write, when wanted, is
 * the caller's) and reset with the time. */
typedef struct gbfv_schedule {
    double end_time;
    double save_interval[2];
    int max_steps;    /* <= 0: no step limit */
    int stop_at_save; /* nonzero: return after the step at which a save time was reached */
} gbfv_schedule;

/* Advances under a schedule. *saved_mask receives, for the last step taken,
 * bit k set when save counter k advanced in it (the step after which the
 * reference calls that writer's write), 0 when no step was taken. Returns
 * GBFV_ERR_CONSTRAINT as gbfv_advance does. */
int gbfv_advance_schedule(gbfv_solver* s, const gbfv_schedule* schedule, int* saved_mask);

/* The CUDA stream (cudaStream_t) the solver issues its work on. */
int gbfv_stream(gbfv_solver* s, void** stream);

/* Per-launch timing of the step kernels with CUDA events on the solver's
 * stream (the GB300 counterpart of the reference's ALSVINN_TIME_BLOCK timers,
 * alsutils/include/alsutils/timer/Timer.hpp:9-50). While enabled, every stage
 * launch is bracketed by events; gbfv_profile_read sums their durations and
 * resets the record. kernel_launches counts every kernel the solver launched
 * since creation. */
int gbfv_profile(gbfv_solver* s, int enable);
int gbfv_profile_read(gbfv_solver* s, double* stage_ms, long long* stage_launches, long long* kernel_launches);

/* Time, step count and the dt of the last step. */
int gbfv_time(gbfv_solver* s, double* t, long long* steps, double* last_dt);

/* Stage kernel candidates and the autotuner (no counterpart in the
 * reference, whose CUDA kernels use fixed launch shapes). A scheme has one
 * or more compiled configurations of its stage kernels: tile shape, threads
 * per CTA (threads < cells: several cells per thread) and halo staging by TMA
 * box copies (tma = 1) or per-thread loads. Candidate 0 is the default. At
 * the first advance the autotuner times every eligible candidate on the
 * solver's state and keeps the fastest (cached per scheme and grid for the
 * process; GBFV_AUTOTUNE=0 in the environment keeps candidate 0); grids of
 * fewer than 4096 interior cells keep candidate 0 unless gbfv_autotune is
 * called. Every
 * candidate gives bit-identical states. TMA candidates need padded rows
 * (t_x * element size) that are multiples of 16 bytes.
 *   gbfv_select_candidate: pin candidate idx (-1: back to the autotuner);
 *     GBFV_ERR_UNSUPPORTED when the grid cannot be staged by TMA.
 *   gbfv_autotune: tune now; ms[i] = the candidate's mean time per stage
 *     launch of one step (SSP-RK3: (MODE_L + 2 x stage 1) / 3; otherwise
 *     MODE_L; -1: not eligible), *chosen = the candidate kept.
 *   gbfv_current_candidate: the candidate in use (-1: not chosen yet). */
int gbfv_candidate_count(gbfv_solver* s, int* count);
int gbfv_candidate_info(gbfv_solver* s, int idx, int tile[3], int* threads, int* tma);
int gbfv_select_candidate(gbfv_solver* s, int idx);
int gbfv_autotune(gbfv_solver* s, int* chosen, double* ms, int capacity);
int gbfv_current_candidate(gbfv_solver* s, int* idx);

/* Same as gbfv_advance, reading the state from host memory first and writing
 * it back after: the call a host-side Volume owner makes per step. For one
 * step (max_steps == 1) of an FP64 / FP64-exact RK2 or RK3 solver on pinned
 * host memory the GPU can address (cudaHostAlloc / pinned allocations; on a
 * GB300 node reached over NVLink-C2C), the first stage reads the host state
 * in place and the last stage writes the result back, with no copies around
 * the step; other calls copy the state in and out. Both give the same bits,
 * and the solver's device state afterwards is the host's. */
int gbfv_advance_host(gbfv_solver* s, double* state_host_inout, double end_time, int number_of_saves,
                      int max_steps);

/* --------------------------------------------------- operator level */

/* One evaluation of the spatial operator on a caller state: out_dev gets
 * sum_d (F_{i-1/2} - F_{i+1/2}) (unscaled) on interior cells and its ghost
 * images, ws the maximum face wave speed per direction (0 for inactive
 * directions). state_dev and out_dev are padded device arrays of the solver's
 * precision (replaces NumericalFlux::computeFlux,
 * alsfvm/include/alsfvm/numflux/NumericalFlux.hpp:44-48, as called by
 * ConservedSystem::operator(), alsfvm/src/simulator/ConservedSystem.cpp:31-103). */
int gbfv_compute_flux(gbfv_solver* s, const void* state_dev, void* out_dev, double ws[3]);

/* Reconstruction in one direction (indicator variable 0) over the reference's
 * cell range; left_dev / right_dev padded device arrays (replaces
 * Reconstruction::performReconstruction,
 * alsfvm/include/alsfvm/reconstruction/Reconstruction.hpp:46-51). */
int gbfv_reconstruct(gbfv_solver* s, int direction, const void* state_dev, void* left_dev, void* right_dev);

/* Ghost-cell fill of a padded device state in place (replaces
 * Boundary::applyBoundaryConditions, alsfvm/include/alsfvm/boundary/Boundary.hpp:30-31). */
int gbfv_apply_boundary(gbfv_solver* s, void* state_dev);

/* Constraint check over a padded device state: *ok = 1 if every cell is finite
 * with rho > 0, p > 0 (replaces CellComputer::obeysConstraints,
 * alsfvm/include/alsfvm/equation/CellComputer.hpp:61). */
int gbfv_obeys_constraints(gbfv_solver* s, const void* state_dev, int* ok);

/* The operator-level calls on a reference Volume as it is laid out: one
 * padded device array per conserved variable (vars[k], k < nvar; separate
 * allocations or one block), issued on `stream` (NULL: the solver's), and
 * synchronous on return like the reference's CUDA path. */

/* NumericalFlux::computeFlux(U, waveSpeed, computeWaveSpeed, out, start,
 * end) (alsfvm/include/alsfvm/numflux/NumericalFlux.hpp:44-52,
 * alsfvm/src/numflux/NumericalFluxCPU.cpp:167-221) on the region of cells
 * [start, n + end) per active dimension (interior coordinates; start[d] >=
 * 0, end[d] <= 0; inactive dimensions 0): out gets, on those cells only,
 * sum_d (F_{i-1/2} - F_{i+1/2}) (unscaled); the other cells of out keep
 * their values; ws[d] = the maximum wave speed of the faces from the
 * region's lower to its upper face in direction d. ConservedSystem splits a
 * stage into the interior and 2 x dim side strips
 * (alsfvm/src/simulator/ConservedSystem.cpp:59-96): each call costs its
 * region. start / end NULL: the whole interior. */
int gbfv_compute_flux_region(gbfv_solver* s, const void* const* state_vars, void* const* out_vars, double ws[3],
                             const int start[3], const int end[3], void* stream);

/* Reconstruction::performReconstruction(in, direction, 0, left, right,
 * start, end) (alsfvm/include/alsfvm/reconstruction/Reconstruction.hpp:
 * 46-58, cell range of alsfvm/src/reconstruction/ReconstructionCPU.cpp:
 * 64-72 shifted by start / end; "none" copies every cell). */
int gbfv_reconstruct_vars(gbfv_solver* s, int direction, const void* const* state_vars, void* const* left_vars,
                          void* const* right_vars, const int start[3], const int end[3], void* stream);

/* Boundary::applyBoundaryConditions (alsfvm/include/alsfvm/boundary/
 * Boundary.hpp:30-31) on one array per variable. */
int gbfv_apply_boundary_vars(gbfv_solver* s, void* const* vars, void* stream);

/* CellComputer::obeysConstraints on one array per variable. */
int gbfv_obeys_constraints_vars(gbfv_solver* s, const void* const* vars, int* ok, void* stream);

/* The other CellComputer maps (alsfvm/include/alsfvm/equation/CellComputer.hpp:
 * 35-70, as CPUCellComputer computes them over every cell of the volume,
 * alsfvm/src/equation/CPUCellComputer.cpp:31-140):
 *   gbfv_prim_to_cons_vars      computeFromPrimitive (rho, u..., p) -> conserved
 *   gbfv_extra_variables_vars   computeExtraVariables: p, then u (Euler; Burgers
 *                               has none)
 *   gbfv_max_wave_speed_vars    computeMaxWaveSpeed in one direction (cells whose
 *                               speed is not a number are passed over) */
int gbfv_prim_to_cons_vars(gbfv_solver* s, const void* const* prim_vars, void* const* cons_vars, void* stream);
int gbfv_extra_variables_vars(gbfv_solver* s, const void* const* cons_vars, void* const* extra_vars, void* stream);
int gbfv_max_wave_speed_vars(gbfv_solver* s, const void* const* cons_vars, int direction, double* speed,
                             void* stream);

/* ------------------------------------------------ device array arithmetic */

/* Elementwise arithmetic on device arrays of `count` values (float for
 * GBFV_FP32, double otherwise), issued on `stream` (a cudaStream_t; NULL:
 * the default stream): what a device Memory<real> of the "gb300" platform
 * needs so that the reference's own integrators and statistics run on
 * device state (replaces memory::Memory<real>'s arithmetic,
 * alsfvm/include/alsfvm/memory/Memory.hpp:166-302, which the reference's
 * cuda platform implements in alsfvm/src/cuda/CudaMemory.cpp and
 * alsfvm/src/cuda/vector_operations.cu). Operations run in the element type
 * in the order of the reference's HostMemory loops
 * (alsfvm/src/memory/HostMemory.cpp:97-311) without multiply-add
 * contraction, so double results equal the reference CPU path's bit for bit
 * (a power other than 1 or 2 uses CUDA's pow). A scalar is a double, as the
 * reference's `real`: float elements are widened, operated on and rounded. */
typedef enum {
    GBFV_MEMORY_ADD = 0,      /* a += b  (Memory::operator+=) */
    GBFV_MEMORY_SUBTRACT = 1, /* a -= b  (operator-=) */
    GBFV_MEMORY_MULTIPLY = 2, /* a *= b  (operator*=) */
    GBFV_MEMORY_DIVIDE = 3    /* a /= b  (operator/=) */
} gbfv_memory_op_kind;

int gbfv_memory_op(int op, void* a_dev, const void* b_dev, long long count, int precision, void* stream);
/* a op= scalar (Memory::operator+=(real) etc.). */
int gbfv_memory_op_scalar(int op, void* a_dev, double scalar, long long count, int precision, void* stream);
/* a = 0 (Memory::makeZero). */
int gbfv_memory_make_zero(void* a_dev, long long count, int precision, void* stream);
/* v1 = a1 v1 + a2 v2 + a3 v3 + a4 v4 + a5 v5, left to right, coefficients in
 * the element type (Memory::addLinearCombination). */
int gbfv_memory_add_linear_combination(void* v1_dev, double a1, double a2, const void* v2_dev, double a3,
                                       const void* v3_dev, double a4, const void* v4_dev, double a5,
                                       const void* v5_dev, long long count, int precision, void* stream);
/* a += factor * pow(b, power) (Memory::addPower; factor 1 for its
 * two-argument form) and a -= pow(b, power) (Memory::subtractPower). */
int gbfv_memory_add_power(void* a_dev, const void* b_dev, double power, double factor, long long count, int precision,
                          void* stream);
int gbfv_memory_subtract_power(void* a_dev, const void* b_dev, double power, long long count, int precision,
                               void* stream);
/* Total variation of a padded array with extents[3] (x fastest) over
 * [start, end) (Memory::getTotalVariation, HostMemory.cpp:323-392):
 * direction -1: sum of pow(sqrt((u - u(y-1))^2 + (u - u(x-1))^2), p) with
 * x from start.x + 1, y from start.y + 1 (2D) and z from 0 (1D / 2D only);
 * direction d: sum of pow(|u - u(-e_d)|, p) from start + e_d. Summed in FP64
 * in a fixed order (equal to the reference's sequential sum to rounding);
 * *result is written after the stream synchronises. */
int gbfv_memory_total_variation(const void* a_dev, const int extents[3], int p, int direction, const int start[3],
                                const int end[3], int precision, double* result, void* stream);

/* ------------------------------------------------------- statistics */

typedef struct gbfv_stats gbfv_stats;

/* Streaming FP64 Welford mean / variance over `count` values per sample
 * (replaces alsuq's MeanVariance with StatisticsHelper::combineStatistics on
 * one rank, alsuq/src/stats/MeanVariance.cpp:30-67,
 * alsuq/src/stats/StatisticsHelper.cpp:35-79; the variance is the population
 * variance). */
int gbfv_stats_create(long long count, gbfv_stats** out);
int gbfv_stats_destroy(gbfv_stats* st);
int gbfv_stats_reset(gbfv_stats* st);
/* Adds one sample from device memory (precision 0: double, 2: float). */
int gbfv_stats_add_device(gbfv_stats* st, const void* sample_dev, int precision);
/* Adds one sample from host memory. */
int gbfv_stats_add_host(gbfv_stats* st, const double* sample_host);
/* Merges another accumulator into st (Chan et al. pairwise combination). */
int gbfv_stats_merge(gbfv_stats* st, const gbfv_stats* other);
/* Writes mean and variance to host arrays of `count` doubles. */
int gbfv_stats_result(gbfv_stats* st, double* mean_host, double* var_host, long long* samples);
/* Writes the raw Welford triple (sample count, mean, M2 = sum of squared
 * deviations) for a cross-rank merge; the rank-level counterpart of the
 * per-rank sums that alsuq/src/stats/StatisticsHelper.cpp:65-68 reduces. An
 * empty accumulator gives samples = 0 and zero arrays. */
int gbfv_stats_export(gbfv_stats* st, double* mean_host, double* m2_host, long long* samples);

/* Cube structure functions (alsuq's "structure_cube" statistic,
 * alsuq/src/stats/StructureCube.cpp:36-76, kernel
 * alsfvm/include/alsfvm/functional/structure_common.hpp:37-154). Each sample
 * adds, per variable and h = 1 .. number_of_h - 1, the sum over cells and
 * over the points of the cube surface at distance h of |u(x) - u(y)|^p /
 * (nx ny nz), points outside the grid wrapped ("periodic") or clamped
 * ("neumann"); entry 0 stays 0. The result is the mean over the samples;
 * gbfv_structure_export gives the raw sums for a cross-rank merge (sums and
 * sample counts add). Arrays are nvar x number_of_h doubles. */
typedef struct gbfv_structure gbfv_structure;
int gbfv_structure_create(const char* boundary, const int n[3], int ghosts, int nvar, int number_of_h, double p,
                          gbfv_structure** out);
int gbfv_structure_destroy(gbfv_structure* s);
/* Adds one sample: a padded device state of nvar variables (precision 0 or 1:
 * double, 2: float). */
int gbfv_structure_add_device(gbfv_structure* s, const void* state_dev, int precision);
int gbfv_structure_result(gbfv_structure* s, double* mean_host, long long* samples);
int gbfv_structure_export(gbfv_structure* s, double* sums_host, long long* samples);
/* Zeroes the sums and the sample count. */
int gbfv_structure_reset(gbfv_structure* s);
/* The axis structure function of alsuq's StructureBasic
 * (alsuq/src/stats/StructureBasic.cpp:50-92): per variable and h = 0 ..
 * number_of_h - 1, the sum over cells of |u(x) - u(x + h e_direction)|^p /
 * (nx ny nz), the shifted point wrapped (periodic) or clamped (Neumann).
 * The other gbfv_structure_* calls apply unchanged. */
int gbfv_structure_create_basic(const char* boundary, const int n[3], int ghosts, int nvar, int number_of_h,
                                double p, int direction, gbfv_structure** out);

/* ------------------------------------------------------- functionals */

/* Functionals of one state (alsfvm::functional::Functional::operator(),
 * alsfvm/include/alsfvm/functional/Functional.hpp:26-60, the set the
 * reference's FunctionalFactory registers for its cuda platform): a map from a
 * padded state to a small volume of nvar variables that gbfv_functional_apply
 * adds, times a weight, into an FP64 accumulator on the device. Names and
 * parameters as in the reference's XML:
 *   identity                      the interior state              (Identity.cpp)
 *   moment (degree)               pow(u, degree), interior         (Moment.cpp)
 *   legendre_pointwise (degree, min_value, max_value, variable_mask)
 *                                 P_degree((u - min) / (max - min)) of the
 *                                 selected variables (bit k: variable k; 0:
 *                                 all); 2D grids only, and the scaled value
 *                                 must lie in [-1, 1]             (LegendrePointWise.cpp)
 *   log_entropy (gamma)           one value, in the energy variable: the
 *                                 integral of -rho s / (gamma - 1),
 *                                 s = log p - gamma log rho; Euler   (LogEntropy.cpp)
 *   bv (degree)                   one value per variable: the total
 *                                 variation sum (sqrt(du_y^2 + du_x^2))^degree;
 *                                 1D / 2D                          (BoundedVariation.cpp)
 *   bv_direction (degree, direction)
 *                                 one value per variable: the sum of
 *                                 |u - u(-e_direction)|^degree     (HostMemory::getTotalVariation)
 *   structure_cube (p, number_of_h)
 *                                 number_of_h values per variable: this
 *                                 state's cube structure function, which
 *                                 replaces the output (weight unused; the
 *                                 reference zeroes its output first) (StructureCube.cpp)
 * n, ghosts, lower, upper: the state's grid (cell lengths enter log_entropy
 * and the 2D checks). gbfv_functional_size gives the output extents;
 * gbfv_functional_result copies nvar x (extent product) values, x fastest. */
typedef struct gbfv_functional gbfv_functional;
typedef struct {
    int degree;
    double min_value, max_value;
    unsigned variable_mask;
    double gamma;
    double p;
    int number_of_h;
    int direction;
} gbfv_functional_params;

int gbfv_functional_create(const char* name, const char* equation, const char* boundary, const int n[3], int ghosts,
                           const double lower[3], const double upper[3], const gbfv_functional_params* params,
                           gbfv_functional** out);
int gbfv_functional_destroy(gbfv_functional* f);
int gbfv_functional_size(const gbfv_functional* f, int size[3], int* nvar);
int gbfv_functional_reset(gbfv_functional* f);
int gbfv_functional_apply(gbfv_functional* f, const void* state_dev, int precision, double weight);
int gbfv_functional_result(gbfv_functional* f, double* out_host);

/* --------------------------------------------------------- ensembles */

/* Many grids (members) of one scheme advanced together: the UQ ensemble of
 * alsuq's Runner (alsuq/src/run/Runner.cpp:39-90), which the reference runs
 * one sample after another. Each RK stage of the whole ensemble is one
 * persistent launch over the tiles of every member; each member has its own
 * dt (from its own wave-speed maximum) and its own time; a time step of the
 * ensemble is replayed as a CUDA graph. Members may have different grid sizes
 * but share the equation, scheme, precision and dimension. Member memory comes
 * from one pool allocated at creation (the HBM budget). The integrator must be
 * rungekutta2 or rungekutta3. */
typedef struct gbfv_batch gbfv_batch;

/* scheme: names, gamma, cfl, precision (its grid fields are ignored). */
int gbfv_batch_create(const gbfv_desc* scheme, long long pool_bytes, int max_members, gbfv_batch** out);
int gbfv_batch_destroy(gbfv_batch* b);

/* Pool bytes a member with this grid needs (three padded state arrays), or a
 * negative status. */
long long gbfv_batch_member_bytes(const gbfv_batch* b, const int n[3]);
int gbfv_batch_free_bytes(const gbfv_batch* b, long long* free_total, long long* largest_block);

/* Adds a member from interior primitive initial data (as gbfv_set_primitive).
 * group >= 0 folds the member's state at end_time into that group's FP64
 * Welford mean / variance (every member of a group shares its grid); < 0: no
 * statistics. GBFV_ERR_MEMORY when the pool or the slots are full. */
int gbfv_batch_add(gbfv_batch* b, const int n[3], const double lower[3], const double upper[3],
                   const double* prim_host, int group, int* slot);
int gbfv_batch_remove(gbfv_batch* b, int slot);

/* Advances every member until it reaches end_time with its own dt (the
 * number_of_saves > 0 clamp lands each member exactly on the save times), or
 * until max_steps more steps (max_steps <= 0: no limit). Members that reach
 * end_time stop; their states are folded into their statistics group. */
int gbfv_batch_advance(gbfv_batch* b, double end_time, int number_of_saves, int max_steps);

/* A member's own end time: it stops at min(end_time, the end time of the
 * advance) and, with number_of_saves > 0, its dt is clamped to the save times
 * k * end_time / number_of_saves (the FixedIntervalWriter clamp, alsfvm/src/
 * io/FixedIntervalWriter.cpp:45-53), so it lands exactly on end_time. The
 * advance's number_of_saves no longer applies to it. A reference run's end
 * time belongs to its configuration (alsfvm/src/config/SimulatorSetup.cpp:
 * 102-232), so members of one ensemble may each have their own. */
int gbfv_batch_set_member_end(gbfv_batch* b, int slot, double end_time, int number_of_saves);

/* The second save clamp of a member, the fvm writer's FixedIntervalWriter
 * (alsfvm/src/io/FixedIntervalWriter.cpp:45-53): dt is also clamped to the
 * next k * interval (0: none), beside the statistics clamp. With it an
 * advance to end_time = k * interval stops every member exactly at its k-th
 * writer save, where the host reads its state for the writer (alsuq's
 * Runner attaches the writers to every sample's simulator,
 * alsuq/src/run/Runner.cpp:55-73). With one statistics save, a member with a
 * statistics clamp is folded at that clamp's save, not at the end of an
 * advance that stopped earlier. */
int gbfv_batch_set_member_write_interval(gbfv_batch* b, int slot, double interval);

/* A member's status: 0 running or finished, 1 its state broke the constraint
 * check (CPUCellComputer::obeysConstraints; the member stopped at
 * *failed_step while the others went on), 2 a halo copy timed out. */
int gbfv_batch_member_status(gbfv_batch* b, int slot, int* status, int* failed_step);

int gbfv_batch_member_time(gbfv_batch* b, int slot, double* t, long long* steps);
int gbfv_batch_member_state(gbfv_batch* b, int slot, double* state_host);

/* Mean and (population) variance of a statistics group over the whole padded
 * state (the reference's statistics volumes include the ghost cells), as
 * nvar * total doubles each; *count = members folded in. */
int gbfv_batch_stats_result(gbfv_batch* b, int group, double* mean_host, double* var_host, long long* count);
/* The raw Welford triple of one group (see gbfv_stats_export). */
int gbfv_batch_stats_export(gbfv_batch* b, int group, double* mean_host, double* m2_host, long long* count);
int gbfv_batch_stats_reset(gbfv_batch* b);
/* Statistics at several save times (FixedIntervalStatistics with
 * numberOfSaves = saves, alsuq/src/stats/FixedIntervalStatistics.cpp:33-86):
 * set before the first member joins; each group then holds one accumulator
 * per save k, into which a member is folded when its save clamp stops it at
 * t = (k + 1) end_time / saves (advance with number_of_saves = saves). The
 * functions above read the last save; _save reads save k. */
int gbfv_batch_set_statistics_saves(gbfv_batch* b, int saves);
int gbfv_batch_stats_export_save(gbfv_batch* b, int group, int save, double* mean_host, double* m2_host,
                                 long long* count);

/* Slots whose member has reached the end time of the last advance (up to
 * capacity written; *count = all of them), and the number of members. */
int gbfv_batch_finished(gbfv_batch* b, int* slots, int capacity, int* count);
int gbfv_batch_active(const gbfv_batch* b, int* count);

/* Kernels launched by the ensemble since creation, and its CUDA stream. */
int gbfv_batch_launches(gbfv_batch* b, long long* launches);
int gbfv_batch_stream(gbfv_batch* b, void** stream);

/* Stage kernel candidates of the ensemble (the same set as the single-grid
 * solver's for the scheme). The autotuner runs at the first advance whose
 * running members hold at least 2^22 cells (or finds the process's cached
 * choice for the scheme); smaller ensembles keep candidate 0 until then.
 * Members whose arrays break a TMA rule stage their halo with per-thread
 * loads inside a TMA candidate.
 *   gbfv_batch_select_candidate: pin candidate idx (-1: back to the autotuner).
 *   gbfv_batch_current_candidate: the candidate in use; *member_tma = members
 *     staged by TMA.
 *   gbfv_batch_autotune_result: per candidate the mean time per stage
 *     launch of one step over the running members (SSP-RK3: (MODE_L + 2 x
 *     stage 1) / 3; otherwise MODE_L) when the autotuner ran (-1: not
 *     timed). */
int gbfv_batch_select_candidate(gbfv_batch* b, int idx);
int gbfv_batch_current_candidate(gbfv_batch* b, int* idx, int* member_tma);
int gbfv_batch_autotune_result(gbfv_batch* b, double* ms, int capacity);

/* ----------------------------------------------------------- serving */

/* A continuous-batching request loop over two ensembles (no counterpart in
 * the reference, whose alsuq runs a fixed list of samples). A request is a
 * solve (equation, grid, end time, initial-data seed). Requests arrive at
 * their `arrival` time (seconds after gbfv_server_run starts), are admitted
 * once their grid fits the HBM budget (first fit in arrival order), run next
 * to the requests already in flight with their own dt and their own end
 * time, fold their final state into the FP64 statistics of their (kind,
 * grid, end time) group and leave, freeing their memory. A request whose
 * state breaks the constraint check fails alone (status 3) and leaves; the
 * others run on. Burgers and Kelvin-Helmholtz requests run in two ensembles
 * driven by two host threads on two streams. */
typedef enum { GBFV_REQUEST_BURGERS = 0, GBFV_REQUEST_KELVIN_HELMHOLTZ = 1 } gbfv_request_kind;

typedef struct {
    int kind;         /* gbfv_request_kind: the equation and its scheme */
    int n;            /* cells per dimension (Burgers: nx; KH: nx = ny) */
    double end_time;  /* the request's own end time */
    double phase;     /* Burgers: u0 = sin(2 pi x) + 0.5 phase, phase in [-1, 1] */
    int sample;       /* KH: generator sample of the interface perturbation */
    double arrival;   /* seconds after the start of gbfv_server_run */
    int keep;         /* 1: keep the final state for gbfv_server_final_state */
    /* NULL: the kind's initial data from phase / sample. Otherwise the
     * caller's interior primitive variables (Burgers n values, KH 4 n^2),
     * copied by gbfv_server_submit. */
    const double* initial_primitive;
} gbfv_request;

typedef struct gbfv_server gbfv_server;

/* budget_bytes: device memory for the two ensembles' member states;
 * precision: gbfv_precision of the states; max_slots: members per ensemble. */
int gbfv_server_create(long long budget_bytes, int precision, int max_slots, gbfv_server** out);
int gbfv_server_destroy(gbfv_server* s);
/* Queue requests before gbfv_server_run; their arrival times pace admission. */
int gbfv_server_submit(gbfv_server* s, const gbfv_request* r, int* id);
/* Serves every submitted request, advancing each ensemble in chunks of
 * steps_per_chunk time steps between admissions. A request that fails does
 * not stop the run; a CUDA error does (every request in flight fails). */
int gbfv_server_run(gbfv_server* s, int steps_per_chunk);
/* Times in seconds after the start of the run; status 2 done, 3 failed. */
int gbfv_server_result(gbfv_server* s, int id, double* arrival_s, double* admit_s, double* finish_s,
                       long long* steps, int* status);
int gbfv_server_final_state(gbfv_server* s, int id, double* state_host, long long capacity);
/* FP64 mean / variance of the final states of every request of a (kind, n,
 * end_time) group; gbfv_server_stats needs the (kind, n) requests to share
 * one end time. */
int gbfv_server_stats_at(gbfv_server* s, int kind, int n, double end_time, double* mean_host, double* var_host,
                         long long* count);
int gbfv_server_stats(gbfv_server* s, int kind, int n, double* mean_host, double* var_host, long long* count);
int gbfv_server_launches(gbfv_server* s, long long* launches);

/* ---------------------------------------------------- initial data */

/* Interior primitive variables of the benchmark workloads at the cell
 * midpoints origin + dx*i + dx/2 (Grid::getCellMidpoints,
 * alsfvm/src/grid/Grid.cpp:148-165), x fastest, one block per variable, ready
 * for gbfv_set_primitive / gbfv_batch_add. They replace the reference's
 * Python initial-data scripts for these workloads (PythonInitialData,
 * alsfvm/src/init/PythonInitialData.cpp:84-281). */
/* Sod: (rho,u,p) = (1,0,1) for x < 0, (0.125,0,0.1) otherwise. */
int gbfv_init_sod(const int n[3], const double lower[3], const double upper[3], double* prim);
/* Kelvin-Helmholtz: rho=2, u=-0.5 inside 0.25+d1(x) < y < 0.75+d2(x), else
 * rho=1, u=0.5; v=0, p=2.5; d(x) = 0.01 sum_j a_j cos(b_j + 2 pi j x) with
 * a = X[0:10] (d1), X[20:30] (d2) normalised to sum 1 and b = 2 pi X[10:20]
 * (d1), 2 pi X[30:40] (d2); X are 40 draws of gbfv_uniform. */
int gbfv_init_kelvin_helmholtz(const int n[3], const double lower[3], const double upper[3], const double X[40],
                               double* prim);
/* Taylor-Green: rho=1, u=sin x cos y cos z, v=-cos x sin y cos z, w=0,
 * p = 100 + ((cos 2x + cos 2y)(cos 2z + 2) - 2)/16. */
int gbfv_init_taylor_green(const int n[3], const double lower[3], const double upper[3], double* prim);
/* Burgers: u = sin(2 pi x) + 0.5 * phase. */
int gbfv_init_burgers_sine(const int n[3], const double lower[3], const double upper[3], double phase,
                           double* prim);

/* ------------------------------------------------------- generator */

/* Uniform draws of the reference's sample generator: draw number
 * sample * dimension + c of the default-seeded mt19937_64 through
 * uniform_real_distribution(0,1), scaled to [lower, upper]
 * (replaces STLMersenne + Uniform, alsuq/src/generator/STLMersenne.cpp:38-85,
 * alsuq/src/distribution/Uniform.cpp:27-34). */
int gbfv_uniform(int dimension, int sample, double lower, double upper, double* out);

/* The stateful generator behind alsuq's sample parameters: one default-seeded
 * mt19937_64 shared by every parameter of a run (the reference keeps it
 * process-wide). gbfv_generator_uniform is STLMersenne::generate(component,
 * sample) for a parameter of `dimension` components -- discard forward to
 * draw sample * dimension, then to the component, never backwards -- followed
 * by Uniform's x * (upper - lower) + lower (alsuq/src/generator/
 * STLMersenne.cpp:38-85, alsuq/src/distribution/Uniform.cpp:27-34). Requests
 * in the reference's order (samples ascending; per sample the parameters in
 * name order, components ascending) reproduce its parameter values. */
typedef struct gbfv_generator gbfv_generator;
int gbfv_generator_create(gbfv_generator** out);
int gbfv_generator_destroy(gbfv_generator* g);
int gbfv_generator_uniform(gbfv_generator* g, int dimension, int component, long long sample, double lower,
                           double upper, double* out);

/* ------------------------------------------------- failure-path testing */

/* Makes the solver's TMA-staged stage launches announce extra_bytes more on
 * their halo barrier than their copies deliver (0 restores the normal
 * launches). Every halo wait then runs out its time limit (about a second
 * per CTA, twice), the kernel records status 2 in the step state and
 * returns without writing, and the advance reports GBFV_ERR_CUDA; the
 * copies themselves complete, the context stays usable and the solver's
 * state is the one before the step. For tests of that error path only:
 * nothing faults and nothing waits without a limit. No counterpart in the
 * reference. */
int gbfv_test_tma_wait_limit(gbfv_solver* s, unsigned extra_bytes);

/* ----------------------------------------------- allocation-free stepping */

/* Size of the library's built-in scratch array for gbfv_advance_noalloc. */
#define GBFV_NOALLOC_SCRATCH_BYTES (32u << 20)

/* gbfv_advance without any allocation, for callers that cannot call
 * cudaMalloc (an application whose device memory belongs to a pool or arena
 * it does not expose, a plug-in that may not allocate after start-up, a host
 * that works inside a fixed memory budget). No counterpart in the reference:
 * alsvinn always allocates its scratch volumes.
 *
 * The caller owns the padded device state (state_dev, nvar * total values of
 * desc->precision, ghosts filled), the stream (NULL: the default stream), the
 * time *t_inout and the step count *steps_inout, which the call advances like
 * gbfv_advance (the same results, bit for bit). It always runs the scheme's
 * default stage kernels (candidate 0: per-thread halo loads; no tensor maps
 * are encoded on the caller's buffers and nothing is autotuned), which on
 * KH 1024^2 FP64 take 0.653 against 0.601 ms per stage launch of the tuned
 * TMA candidate that gbfv_advance picks. Scratch -- the stage-0 flux
 * difference, the second state buffer and the step state -- comes from one
 * static device array of GBFV_NOALLOC_SCRATCH_BYTES that every GPU loading the
 * library holds until exit; grids needing more (2 * nvar * total * element
 * size plus under 1 KiB of step state and alignment) are rejected with GBFV_ERR_UNSUPPORTED. The call makes no
 * cudaMalloc, cudaFree or other allocating call.
 *  - The first call on a device looks up the array's device address
 *    (cudaGetSymbolAddress) with that device current, and so does the first
 *    call in a new context of the device (after a cudaDeviceReset); make the
 *    first call before any stream capture. Host threads share the looked-up
 *    address under a lock.
 *  - All calls share the one array and it keeps the last call's contents;
 *    calls that overlap on the GPU (other streams, other host threads) race.
 *  - The save-time clamp restarts from *t_inout on every call. */
int gbfv_advance_noalloc(const gbfv_desc* desc, void* state_dev, double* t_inout, long long* steps_inout,
                         double end_time, int number_of_saves, int max_steps, void* stream);

#ifdef __cplusplus
}
#endif
#endif
