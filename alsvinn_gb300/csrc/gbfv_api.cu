// C ABI of the GB300 finite-volume step (include/gbfv.h): solver handles, the
// per-step driver and the operator-level entry points. Built with -fmad=false
// (device) and -ffp-contract=off (host) so the time-step arithmetic and the
// primitive-to-conserved conversion round exactly as the reference does.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <random>
#include <string>
#include <vector>

#include "fv_registry.h"
#include "fv_tma.cuh"
#include "gbfv.h"
#include "gbfv_internal.h"

#define GBFV_REGISTER_DECL(v, e) extern "C" void gbfv_register_v##v##_e##e(gbfv::Registry*);
GBFV_REGISTER_DECL(0, 0) GBFV_REGISTER_DECL(0, 1) GBFV_REGISTER_DECL(0, 2) GBFV_REGISTER_DECL(0, 3)
GBFV_REGISTER_DECL(1, 0) GBFV_REGISTER_DECL(1, 1) GBFV_REGISTER_DECL(1, 2) GBFV_REGISTER_DECL(1, 3)
GBFV_REGISTER_DECL(2, 0) GBFV_REGISTER_DECL(2, 1) GBFV_REGISTER_DECL(2, 2) GBFV_REGISTER_DECL(2, 3)
GBFV_REGISTER_DECL(3, 0) GBFV_REGISTER_DECL(3, 1) GBFV_REGISTER_DECL(3, 2) GBFV_REGISTER_DECL(3, 3)
#define GBFV_TUNE_DECL(v, e) extern "C" void gbfv_tune_v##v##_e##e(gbfv::Registry*);
GBFV_TUNE_DECL(0, 0) GBFV_TUNE_DECL(0, 1) GBFV_TUNE_DECL(0, 2) GBFV_TUNE_DECL(0, 3)
GBFV_TUNE_DECL(1, 0) GBFV_TUNE_DECL(1, 1) GBFV_TUNE_DECL(1, 2) GBFV_TUNE_DECL(1, 3)
GBFV_TUNE_DECL(2, 0) GBFV_TUNE_DECL(2, 1) GBFV_TUNE_DECL(2, 2) GBFV_TUNE_DECL(2, 3)
GBFV_TUNE_DECL(3, 0) GBFV_TUNE_DECL(3, 1) GBFV_TUNE_DECL(3, 2) GBFV_TUNE_DECL(3, 3)
#define GBFV_REGION_DECL(v, e) extern "C" void gbfv_region_v##v##_e##e(gbfv::Registry*);
GBFV_REGION_DECL(0, 0) GBFV_REGION_DECL(0, 1) GBFV_REGION_DECL(0, 2) GBFV_REGION_DECL(0, 3)
GBFV_REGION_DECL(1, 0) GBFV_REGION_DECL(1, 1) GBFV_REGION_DECL(1, 2) GBFV_REGION_DECL(1, 3)
GBFV_REGION_DECL(2, 0) GBFV_REGION_DECL(2, 1) GBFV_REGION_DECL(2, 2) GBFV_REGION_DECL(2, 3)
GBFV_REGION_DECL(3, 0) GBFV_REGION_DECL(3, 1) GBFV_REGION_DECL(3, 2) GBFV_REGION_DECL(3, 3)

namespace gbfv {

Registry& registry() {
    // ~1 MB of launcher table: built once on the heap
    static Registry* R = [] {
        Registry* r = new Registry();
        std::memset(r, 0, sizeof *r);
        gbfv_register_v0_e0(r); gbfv_register_v0_e1(r); gbfv_register_v0_e2(r); gbfv_register_v0_e3(r);
        gbfv_register_v1_e0(r); gbfv_register_v1_e1(r); gbfv_register_v1_e2(r); gbfv_register_v1_e3(r);
        gbfv_register_v2_e0(r); gbfv_register_v2_e1(r); gbfv_register_v2_e2(r); gbfv_register_v2_e3(r);
        gbfv_register_v3_e0(r); gbfv_register_v3_e1(r); gbfv_register_v3_e2(r); gbfv_register_v3_e3(r);
        // autotuning candidates after every default
        gbfv_tune_v0_e0(r); gbfv_tune_v0_e1(r); gbfv_tune_v0_e2(r); gbfv_tune_v0_e3(r);
        gbfv_tune_v1_e0(r); gbfv_tune_v1_e1(r); gbfv_tune_v1_e2(r); gbfv_tune_v1_e3(r);
        gbfv_tune_v2_e0(r); gbfv_tune_v2_e1(r); gbfv_tune_v2_e2(r); gbfv_tune_v2_e3(r);
        gbfv_tune_v3_e0(r); gbfv_tune_v3_e1(r); gbfv_tune_v3_e2(r); gbfv_tune_v3_e3(r);
        // region kernels of the operator-level calls
        gbfv_region_v0_e0(r); gbfv_region_v0_e1(r); gbfv_region_v0_e2(r); gbfv_region_v0_e3(r);
        gbfv_region_v1_e0(r); gbfv_region_v1_e1(r); gbfv_region_v1_e2(r); gbfv_region_v1_e3(r);
        gbfv_region_v2_e0(r); gbfv_region_v2_e1(r); gbfv_region_v2_e2(r); gbfv_region_v2_e3(r);
        gbfv_region_v3_e0(r); gbfv_region_v3_e1(r); gbfv_region_v3_e2(r); gbfv_region_v3_e3(r);

        return r;
    }();
    return *R;
}

const StageCandidate* candidates(int var, int eq, int fl, int rc, int dim, int* count) {
    Registry& R = registry();
    *count = R.ncand[var][eq][fl][rc][dim - 1];
    return R.cand[var][eq][fl][rc][dim - 1];
}

// ------------------------------------------------------- step kernels

// dt = cfl / sum_d ws_d / dx_d, then the save-time clamp
// (Integrator::computeTimestep, alsfvm/src/integrator/Integrator.cpp:20-46;
// FixedIntervalWriter::adjustTimestep, alsfvm/src/io/FixedIntervalWriter.cpp:45-53).
__global__ void dt_kernel(StepState* st, StepParams P) {
    if (st->done) return;
    set_step_dt(*st, P.dim, P.cell_lengths, P.cfl, P.time_interval, P.time_interval2);
}

// t += dt (TimestepInformation::incrementTime), the writer's save counter, and
// the loop condition t < end_time (Simulator::atEnd, Simulator.cpp:77-79).
__global__ void finish_kernel(StepState* st, StepParams P) {
    if (st->done) return;
    st->t = st->t + st->dt;
    st->steps += 1;
    // the writers' save counters (FixedIntervalWriter::write, FixedIntervalWriter.cpp:32-42;
    // FixedIntervalStatistics::computeStatistics, FixedIntervalStatistics.cpp:71-86)
    int saved = 0;
    if (P.time_interval > 0 && st->t >= (double)st->number_saved * P.time_interval + 0.0) {
        st->number_saved += 1;
        saved |= 1;
    }
    if (P.time_interval2 > 0 && st->t >= (double)st->number_saved2 * P.time_interval2) {
        st->number_saved2 += 1;
        saved |= 2;
    }
    st->saved_mask = saved;
    st->ws_bits[0] = st->ws_bits[1] = st->ws_bits[2] = 0ull;
    if (!(st->t < st->end_time) || (st->step_limit >= 0 && st->steps >= st->step_limit) || st->status != 0 ||
        (P.stop_at_save && saved))
        st->done = 1;
}

__global__ void begin_kernel(StepState* st, double end_time, long long step_limit) {
    st->end_time = end_time;
    st->step_limit = step_limit;
    st->ws_bits[0] = st->ws_bits[1] = st->ws_bits[2] = 0ull;
    st->done = (!(st->t < end_time) || (step_limit >= 0 && st->steps >= step_limit) || st->status != 0) ? 1 : 0;
}

// Copies V into U (end of an RK2 step), skipped once the advance is done.
template <class R>
__global__ void copy_state_kernel(const StepState* st, const R* __restrict__ src, R* __restrict__ dst, long long n) {
    if (st->done) return;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        dst[i] = src[i];
}

// Ghost fill: every ghost cell copies the interior cell its per-dimension index
// maps select; the composition equals the reference's dimension-by-dimension
// fill (alsfvm/src/boundary/BoundaryCPU.cpp:30-106).
__device__ __forceinline__ int src_index(int p, int n, int g, bool periodic) {
    if (p < g) return periodic ? p + n : 2 * g - 1 - p;
    if (p >= n + g) return periodic ? p - n : 2 * (n + g) - 1 - p;
    return p;
}

template <class R>
__global__ void boundary_kernel(R* U, Grid G, int nvar, int periodic) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= G.total) return;
    const int x = (int)(i % G.t[0]);
    const int y = (int)((i / G.t[0]) % G.t[1]);
    const int z = (int)(i / ((long long)G.t[0] * G.t[1]));
    const bool per = periodic != 0;
    const int sx = src_index(x, G.n[0], G.g[0], per);
    const int sy = src_index(y, G.n[1], G.g[1], per);
    const int sz = src_index(z, G.n[2], G.g[2], per);
    if (sx == x && sy == y && sz == z) return;
    const long long s = gidx(G, sx, sy, sz);
    for (int k = 0; k < nvar; ++k) U[k * G.total + i] = U[k * G.total + s];
}

}  // namespace gbfv

using namespace gbfv;

// ---------------------------------------------------------------- errors

static thread_local std::string g_err;

static int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

int gbfv_internal_fail(int code, const char* msg) { return fail(code, msg); }

#define CUDA_TRY(x)                                                                          \
    do {                                                                                     \
        cudaError_t e_ = (x);                                                                \
        if (e_ != cudaSuccess)                                                               \
            return fail(GBFV_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_));     \
    } while (0)

#define LAUNCH_TRY(x)                                                                        \
    do {                                                                                     \
        int r_ = (x);                                                                        \
        if (r_ != 0)                                                                         \
            return fail(GBFV_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString((cudaError_t)r_)); \
    } while (0)

// ---------------------------------------------------------------- names

static int parse_eq(const char* s) {
    if (!s) return -1;
    if (!strcmp(s, "burgers")) return EQ_BURGERS;
    if (!strcmp(s, "euler1")) return EQ_EULER1;
    if (!strcmp(s, "euler2")) return EQ_EULER2;
    if (!strcmp(s, "euler3")) return EQ_EULER3;
    return -1;
}
static int parse_flux(const char* s) {
    if (!s) return -1;
    if (!strcmp(s, "hll")) return FL_HLL;
    if (!strcmp(s, "hll3")) return FL_HLL3;
    if (!strcmp(s, "godunov")) return FL_GODUNOV;
    if (!strcmp(s, "central")) return FL_CENTRAL;
    if (!strcmp(s, "rusanov")) return FL_RUSANOV;
    if (!strcmp(s, "roe")) return FL_ROE;
    return -1;
}
static int parse_recon(const char* s) {
    if (!s) return -1;
    if (!strcmp(s, "none")) return RC_NONE;
    if (!strcmp(s, "weno2")) return RC_WENO2;
    if (!strcmp(s, "eno2")) return RC_ENO2;
    if (!strcmp(s, "eno3")) return RC_ENO3;
    if (!strcmp(s, "eno4")) return RC_ENO4;
    if (!strcmp(s, "mc")) return RC_MC;
    if (!strcmp(s, "mm")) return RC_MM;
    if (!strcmp(s, "wenof2")) return RC_WENOF2;
    return -1;
}
enum { IN_FE = 0, IN_RK2 = 1, IN_RK3 = 2 };
static int parse_integrator(const char* s) {
    if (!s) return -1;
    if (!strcmp(s, "forwardeuler")) return IN_FE;
    if (!strcmp(s, "rungekutta2")) return IN_RK2;
    if (!strcmp(s, "rungekutta3")) return IN_RK3;
    return -1;
}
static int parse_bc(const char* s) {
    if (!s) return -1;
    if (!strcmp(s, "neumann")) return 0;
    if (!strcmp(s, "periodic")) return 1;
    return -1;
}
static const int kReconGhosts[8] = {1, 2, 2, 3, 4, 2, 2, 2};

// ---------------------------------------------------------------- solver

struct gbfv_solver {
    int eq, fl, rc, in, periodic, var, nvar, elem;
    double gamma, cfl;
    double cell_lengths[3];
    Grid G;
    void* U = nullptr;  // current state (padded)
    void* V = nullptr;  // second state buffer
    void* L = nullptr;  // stage-0 flux difference
    StepState* st = nullptr;     // device step state
    StepState* st_op = nullptr;  // device scratch for operator-level calls
    StepState* st_host = nullptr;  // pinned mirror
    int* flag = nullptr;           // device scratch flag
    int* flag_host = nullptr;
    void* staging = nullptr;       // pinned host staging (FP32 conversions)
    cudaStream_t stream = nullptr;
    double time_interval = 0;
    long long launches = 0;         // kernels launched since creation
    bool profiling = false;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> events;  // stage launches while profiling
    std::vector<cudaEvent_t> event_pool;
    // stage kernel configuration: the candidate in use (-1: chosen by the
    // autotuner at the first advance) and its tensor maps of U, V, L
    int cand = -1;
    bool pinned = false;  // set by gbfv_select_candidate: the autotuner leaves it alone
    CUtensorMap tm[3];
    bool tm_ok = false;
    std::vector<double> tune_ms;  // the autotuner's MODE_L time per candidate (-1: not eligible)
    void* op_block = nullptr;     // scratch of the per-variable operator calls (allocated at first use)
    unsigned tma_extra_tx = 0;    // gbfv_test_tma_wait_limit: extra bytes announced on the halo barrier
    // st_host mirrors st: set after each copy back, cleared while step kernels
    // may be in flight (an advance skips its opening copy when it is set)
    bool st_host_valid = false;
    // kGraphSteps time steps captured as one CUDA graph, replayed for the
    // long stretches of an advance (valid for graph_params and graph_cand)
    cudaGraphExec_t step_graph = nullptr;
    StepParams graph_params;
    int graph_cand = -2;
    long long graph_launches = 0;  // kernels in one replay
};

static size_t state_bytes(const gbfv_solver* s) { return (size_t)s->nvar * s->G.total * s->elem; }

static void release(gbfv_solver* s) {
    if (!s) return;
    if (s->step_graph) cudaGraphExecDestroy(s->step_graph);
    for (auto& e : s->events) {
        cudaEventDestroy(e.first);
        cudaEventDestroy(e.second);
    }
    for (auto e : s->event_pool) cudaEventDestroy(e);
    if (s->U) cudaFree(s->U);
    if (s->V) cudaFree(s->V);
    if (s->L) cudaFree(s->L);
    if (s->st) cudaFree(s->st);
    if (s->st_op) cudaFree(s->st_op);
    if (s->flag) cudaFree(s->flag);
    if (s->st_host) cudaFreeHost(s->st_host);
    if (s->flag_host) cudaFreeHost(s->flag_host);
    if (s->staging) cudaFreeHost(s->staging);
    if (s->op_block) cudaFree(s->op_block);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
}

extern "C" {

const char* gbfv_last_error(void) { return g_err.c_str(); }
const char* gbfv_version(void) { return "gbfv 0.1 sm_103a"; }

int gbfv_ghost_cells(const char* reconstruction) {
    const int rc = parse_recon(reconstruction);
    if (rc < 0) return fail(GBFV_ERR_ARGUMENT, "unknown reconstruction");
    return kReconGhosts[rc];
}

int gbfv_num_variables(const char* equation) {
    const int eq = parse_eq(equation);
    if (eq < 0) return fail(GBFV_ERR_ARGUMENT, "unknown equation");
    return eq == EQ_BURGERS ? 1 : eq + 2;
}

int gbfv_create(const gbfv_desc* d, gbfv_solver** out) {
    if (!d || !out) return fail(GBFV_ERR_ARGUMENT, "null argument");
    *out = nullptr;
    const int eq = parse_eq(d->equation), fl = parse_flux(d->flux), rc = parse_recon(d->reconstruction);
    const int in = parse_integrator(d->integrator), bc = parse_bc(d->boundary);
    if (eq < 0) return fail(GBFV_ERR_ARGUMENT, "unknown equation");
    if (fl < 0) return fail(GBFV_ERR_ARGUMENT, "unknown flux");
    if (rc < 0) return fail(GBFV_ERR_ARGUMENT, "unknown reconstruction");
    if (in < 0) return fail(GBFV_ERR_ARGUMENT, "unknown integrator");
    if (bc < 0) return fail(GBFV_ERR_ARGUMENT, "unknown boundary");
    if (!flux_applies(eq, fl))
        return fail(GBFV_ERR_UNSUPPORTED, "flux does not apply to this equation");
    if (d->precision < 0 || d->precision >= NUM_VARIANTS) return fail(GBFV_ERR_ARGUMENT, "bad precision");
    for (int k = 0; k < 3; ++k)
        if (d->n[k] < 1) return fail(GBFV_ERR_ARGUMENT, "grid dimensions must be >= 1");
    const int dim = d->n[2] > 1 ? 3 : (d->n[1] > 1 ? 2 : 1);
    if (eq != EQ_BURGERS && eq != dim)
        return fail(GBFV_ERR_UNSUPPORTED, "euler<d> needs a d-dimensional grid");
    const int g = kReconGhosts[rc];
    for (int k = 0; k < dim; ++k)
        if (d->n[k] < g) return fail(GBFV_ERR_UNSUPPORTED, "every active dimension needs at least as many cells as ghost cells");
    int ncand = 0;
    candidates(d->precision, eq, fl, rc, dim, &ncand);
    if (ncand == 0) return fail(GBFV_ERR_UNSUPPORTED, "no kernel for this combination");

    gbfv_solver* s = new gbfv_solver();
    s->eq = eq; s->fl = fl; s->rc = rc; s->in = in; s->periodic = bc; s->var = d->precision;
    s->nvar = eq == EQ_BURGERS ? 1 : eq + 2;
    s->elem = d->precision == VAR_F32 ? 4 : 8;
    s->gamma = d->gamma;
    s->cfl = d->cfl;
    s->G.dim = dim;
    long long total = 1;
    for (int k = 0; k < 3; ++k) {
        s->G.n[k] = d->n[k];
        s->G.g[k] = k < dim ? g : 0;
        s->G.t[k] = d->n[k] + 2 * s->G.g[k];
        total *= s->G.t[k];
    }
    s->G.total = total;
    // Grid cell lengths; inactive dimensions get 1 (alsfvm/src/grid/Grid.cpp:24-42).
    for (int k = 0; k < 3; ++k) s->cell_lengths[k] = (d->upper[k] - d->lower[k]) / d->n[k];
    if (d->n[1] == 1) s->cell_lengths[1] = 1;
    if (d->n[2] == 1) s->cell_lengths[2] = 1;

    const size_t bytes = state_bytes(s);
    cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&s->U, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&s->V, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&s->L, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&s->st, sizeof(StepState));
    if (e == cudaSuccess) e = cudaMalloc(&s->st_op, sizeof(StepState));
    if (e == cudaSuccess) e = cudaMalloc(&s->flag, sizeof(int));
    if (e == cudaSuccess) e = cudaMallocHost(&s->st_host, sizeof(StepState));
    if (e == cudaSuccess) e = cudaMallocHost(&s->flag_host, sizeof(int));
    if (e == cudaSuccess) e = cudaMemsetAsync(s->U, 0, bytes, s->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->V, 0, bytes, s->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->L, 0, bytes, s->stream);
    if (e == cudaSuccess) {
        StepState z;
        std::memset(&z, 0, sizeof z);
        z.number_saved = 1;
        z.number_saved2 = 1;
        z.done = 1;
        *s->st_host = z;
        e = cudaMemcpyAsync(s->st, s->st_host, sizeof z, cudaMemcpyHostToDevice, s->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        if (e == cudaSuccess) s->st_host_valid = true;
    }
    if (e != cudaSuccess) {
        const int code = (e == cudaErrorMemoryAllocation) ? GBFV_ERR_MEMORY : GBFV_ERR_CUDA;
        release(s);
        return fail(code, std::string("gbfv_create: ") + cudaGetErrorString(e));
    }
    *out = s;
    return GBFV_OK;
}

int gbfv_destroy(gbfv_solver* s) {
    if (!s) return GBFV_OK;
    if (s->stream) cudaStreamSynchronize(s->stream);
    release(s);
    return GBFV_OK;
}

int gbfv_extents(const gbfv_solver* s, int t[3], long long* total) {
    if (!s) return fail(GBFV_ERR_ARGUMENT, "null solver");
    if (t)
        for (int k = 0; k < 3; ++k) t[k] = s->G.t[k];
    if (total) *total = s->G.total;
    return GBFV_OK;
}

static int reset_time(gbfv_solver* s) {
    StepState z;
    std::memset(&z, 0, sizeof z);
    z.number_saved = 1;
    z.number_saved2 = 1;
    z.done = 1;
    *s->st_host = z;
    s->st_host_valid = false;
    CUDA_TRY(cudaMemcpyAsync(s->st, s->st_host, sizeof z, cudaMemcpyHostToDevice, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    s->st_host_valid = true;
    return GBFV_OK;
}

static int upload(gbfv_solver* s, const double* host) {
    const size_t n = (size_t)s->nvar * s->G.total;
    if (s->elem == 8) {
        CUDA_TRY(cudaMemcpyAsync(s->U, host, n * 8, cudaMemcpyHostToDevice, s->stream));
    } else {
        if (!s->staging) CUDA_TRY(cudaMallocHost(&s->staging, n * 4));
        CUDA_TRY(cudaStreamSynchronize(s->stream));
        float* f = static_cast<float*>(s->staging);
        for (size_t i = 0; i < n; ++i) f[i] = (float)host[i];
        CUDA_TRY(cudaMemcpyAsync(s->U, f, n * 4, cudaMemcpyHostToDevice, s->stream));
    }
    return GBFV_OK;
}

static int download(gbfv_solver* s, double* host) {
    const size_t n = (size_t)s->nvar * s->G.total;
    if (s->elem == 8) {
        CUDA_TRY(cudaMemcpyAsync(host, s->U, n * 8, cudaMemcpyDeviceToHost, s->stream));
        CUDA_TRY(cudaStreamSynchronize(s->stream));
    } else {
        if (!s->staging) CUDA_TRY(cudaMallocHost(&s->staging, n * 4));
        CUDA_TRY(cudaMemcpyAsync(s->staging, s->U, n * 4, cudaMemcpyDeviceToHost, s->stream));
        CUDA_TRY(cudaStreamSynchronize(s->stream));
        const float* f = static_cast<const float*>(s->staging);
        for (size_t i = 0; i < n; ++i) host[i] = (double)f[i];
    }
    return GBFV_OK;
}

static int launch_boundary(gbfv_solver* s, void* U) {
    const int bs = 256;
    const unsigned nb = (unsigned)((s->G.total + bs - 1) / bs);
    if (s->elem == 8)
        boundary_kernel<double><<<nb, bs, 0, s->stream>>>((double*)U, s->G, s->nvar, s->periodic);
    else
        boundary_kernel<float><<<nb, bs, 0, s->stream>>>((float*)U, s->G, s->nvar, s->periodic);
    CUDA_TRY(cudaGetLastError());
    return GBFV_OK;
}

int gbfv_set_state(gbfv_solver* s, const double* host) {
    if (!s || !host) return fail(GBFV_ERR_ARGUMENT, "null argument");
    int r = upload(s, host);
    if (r) return r;
    return reset_time(s);
}

int gbfv_get_state(gbfv_solver* s, double* host) {
    if (!s || !host) return fail(GBFV_ERR_ARGUMENT, "null argument");
    return download(s, host);
}

int gbfv_state_device(gbfv_solver* s, void** dev) {
    if (!s || !dev) return fail(GBFV_ERR_ARGUMENT, "null argument");
    *dev = s->U;
    return GBFV_OK;
}

// Primitive -> conserved for the interior cells of a padded array (ghosts
// untouched): CPUCellComputer::computeFromPrimitive with
// Euler::computeConserved (Euler.hpp:236-245) in the reference's operand
// order; Burgers copies u.
static void prim_to_cons(int eq, double gamma, const Grid& G, const double* prim, double* cons) {
    const long long total = G.total;
    const long long cells = (long long)G.n[0] * G.n[1] * G.n[2];
    const int nsd = eq == EQ_BURGERS ? 1 : eq;
    for (int z = 0; z < G.n[2]; ++z)
        for (int y = 0; y < G.n[1]; ++y)
            for (int x = 0; x < G.n[0]; ++x) {
                const long long ic = ((long long)z * G.n[1] + y) * G.n[0] + x;
                const long long ip = ((long long)(z + G.g[2]) * G.t[1] + (y + G.g[1])) * G.t[0] + (x + G.g[0]);
                if (eq == EQ_BURGERS) {
                    cons[ip] = prim[ic];
                    continue;
                }
                const double rho = prim[ic];
                double u[3] = {0.0, 0.0, 0.0};
                for (int k = 0; k < nsd; ++k) u[k] = prim[(1 + k) * cells + ic];
                const double p = prim[(1 + nsd) * cells + ic];
                double dot = u[0] * u[0];
                for (int k = 1; k < nsd; ++k) dot = dot + u[k] * u[k];
                cons[ip] = rho;
                for (int k = 0; k < nsd; ++k) cons[(1 + k) * total + ip] = u[k] * rho;
                cons[(1 + nsd) * total + ip] = p / (gamma - 1) + 0.5 * rho * dot;
            }
}

// Primitive -> conserved for interior cells, then the ghost fill: the values
// Simulator::setInitialValue produces (conversion CPUCellComputer::
// computeFromPrimitive with Euler::computeConserved, Euler.hpp:236-245).
int gbfv_set_primitive(gbfv_solver* s, const double* prim) {
    if (!s || !prim) return fail(GBFV_ERR_ARGUMENT, "null argument");
    std::vector<double> cons((size_t)s->nvar * s->G.total, 0.0);
    prim_to_cons(s->eq, s->gamma, s->G, prim, cons.data());
    int r = upload(s, cons.data());
    if (r) return r;
    r = launch_boundary(s, s->U);
    if (r) return r;
    return reset_time(s);
}

static StageArgs stage_args(gbfv_solver* s, StepState* st, const void* in, const void* u0, const void* l0,
                            void* out, int mode, int check) {
    StageArgs a;
    std::memset(&a, 0, sizeof a);
    a.in = in;
    a.u0 = u0;
    a.l0 = l0;
    a.out = out;
    a.st = st;
    a.G = s->G;
    a.gamma = s->gamma;
    a.gamma_f = (float)s->gamma;
    a.tm_in = nullptr;
    a.tm_l0 = nullptr;
    a.mode = mode;
    a.periodic = s->periodic;
    a.check = check;
    a.tma_extra_tx = s->tma_extra_tx;
    return a;
}

static cudaEvent_t take_event(gbfv_solver* s) {
    if (!s->event_pool.empty()) {
        cudaEvent_t e = s->event_pool.back();
        s->event_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

// Tensor maps of a stage launch on the solver's own buffers (U, V, L).
static const CUtensorMap* solver_map(const gbfv_solver* s, const void* p) {
    if (p == s->U) return &s->tm[0];
    if (p == s->V) return &s->tm[1];
    if (p == s->L) return &s->tm[2];
    return nullptr;
}

// Launches candidate c of the solver's scheme; TMA candidates get the maps of
// a.in and a.l0 (which must be the solver's buffers).
static int launch_candidate(gbfv_solver* s, const StageCandidate& c, const StageArgs& a) {
    if (!c.tma) return c.stage(a, nullptr, s->stream);
    const CUtensorMap* mi = solver_map(s, a.in);
    const CUtensorMap* ml = a.l0 ? solver_map(s, a.l0) : mi;
    if (!s->tm_ok || !mi || !ml) return (int)cudaErrorInvalidValue;
    TmaMaps m;
    m.in = *mi;
    m.l0 = *ml;
    return c.stage(a, &m, s->stream);
}

// One stage launch, bracketed by events while profiling.
static int launch_stage(gbfv_solver* s, const StageCandidate& c, const StageArgs& a) {
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (s->profiling) {
        e0 = take_event(s);
        e1 = take_event(s);
        CUDA_TRY(cudaEventRecord(e0, s->stream));
    }
    LAUNCH_TRY(launch_candidate(s, c, a));
    s->launches += 1;
    if (s->profiling) {
        CUDA_TRY(cudaEventRecord(e1, s->stream));
        s->events.emplace_back(e0, e1);
    }
    return GBFV_OK;
}

#define STAGE_TRY(x)       \
    do {                   \
        int r_ = (x);      \
        if (r_) return r_; \
    } while (0)

// Enqueues one time step; every kernel returns at once when st->done is set.
static int enqueue_step(gbfv_solver* s, const StepParams& P) {
    Registry& R = registry();
    int ncand = 0;
    const StageCandidate& stage = candidates(s->var, s->eq, s->fl, s->rc, s->G.dim, &ncand)[s->cand < 0 ? 0 : s->cand];
    cudaStream_t q = s->stream;
    STAGE_TRY(launch_stage(s, stage, stage_args(s, s->st, s->U, s->U, nullptr, s->L, MODE_L, 0)));
    dt_kernel<<<1, 1, 0, q>>>(s->st, P);
    CUDA_TRY(cudaGetLastError());
    s->launches += 2;  // dt + finish
    if (s->in == IN_RK3) {
        STAGE_TRY(launch_stage(s, stage, stage_args(s, s->st, s->U, s->U, s->L, s->V, MODE_RK3_S1, 0)));
        STAGE_TRY(launch_stage(s, stage, stage_args(s, s->st, s->V, s->U, nullptr, s->U, MODE_RK3_S2, 1)));
    } else if (s->in == IN_RK2) {
        STAGE_TRY(launch_stage(s, stage, stage_args(s, s->st, s->U, s->U, s->L, s->V, MODE_RK2_S1, 1)));
        s->launches += 1;
        const long long n = (long long)s->nvar * s->G.total;
        if (s->elem == 8)
            copy_state_kernel<double><<<1184, 256, 0, q>>>(s->st, (const double*)s->V, (double*)s->U, n);
        else
            copy_state_kernel<float><<<1184, 256, 0, q>>>(s->st, (const float*)s->V, (float*)s->U, n);
        CUDA_TRY(cudaGetLastError());
    } else {
        LAUNCH_TRY(R.apply[s->var][s->eq](stage_args(s, s->st, s->U, s->U, s->L, s->U, MODE_L, 1), q));
        s->launches += 1;
    }
    finish_kernel<<<1, 1, 0, q>>>(s->st, P);
    CUDA_TRY(cudaGetLastError());
    return GBFV_OK;
}

static int tune(gbfv_solver* s, bool force);

constexpr int kGraphSteps = 16;

static bool same_params(const StepParams& a, const StepParams& b) {
    return a.cfl == b.cfl && a.cell_lengths[0] == b.cell_lengths[0] && a.cell_lengths[1] == b.cell_lengths[1] &&
           a.cell_lengths[2] == b.cell_lengths[2] && a.end_time == b.end_time && a.time_interval == b.time_interval &&
           a.dim == b.dim && a.time_interval2 == b.time_interval2 && a.stop_at_save == b.stop_at_save;
}

// Enqueues n time steps: groups of kGraphSteps replay one captured graph
// (one launch instead of five per step; steps past the end of the advance
// return at once, as in the direct path), the rest are launched directly.
// Profiling keeps the direct path (per-launch events).
static int enqueue_steps(gbfv_solver* s, const StepParams& P, int n) {
    if (!s->profiling && n >= kGraphSteps) {
        if (!s->step_graph || !same_params(s->graph_params, P) || s->graph_cand != s->cand) {
            if (s->step_graph) cudaGraphExecDestroy(s->step_graph);
            s->step_graph = nullptr;
            cudaGraph_t g = nullptr;
            CUDA_TRY(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
            const long long before = s->launches;
            int r = GBFV_OK;
            for (int i = 0; i < kGraphSteps && !r; ++i) r = enqueue_step(s, P);
            const cudaError_t ce = cudaStreamEndCapture(s->stream, &g);
            s->graph_launches = s->launches - before;
            s->launches = before;
            if (r) {
                if (g) cudaGraphDestroy(g);
                return r;
            }
            if (ce != cudaSuccess) return fail(GBFV_ERR_CUDA, std::string("step graph capture: ") + cudaGetErrorString(ce));
            const cudaError_t ie = cudaGraphInstantiate(&s->step_graph, g, 0);
            cudaGraphDestroy(g);
            if (ie != cudaSuccess) return fail(GBFV_ERR_CUDA, std::string("step graph: ") + cudaGetErrorString(ie));
            s->graph_params = P;
            s->graph_cand = s->cand;
        }
        for (; n >= kGraphSteps; n -= kGraphSteps) {
            CUDA_TRY(cudaGraphLaunch(s->step_graph, s->stream));
            s->launches += s->graph_launches;
        }
    }
    for (int i = 0; i < n; ++i) {
        const int r = enqueue_step(s, P);
        if (r) return r;
    }
    return GBFV_OK;
}

static int drive(gbfv_solver* s, const StepParams& P, long long limit) {
    if (s->cand < 0 && !s->pinned) {
        const int r = tune(s, false);
        if (r) return r;
    }
    s->st_host_valid = false;
    begin_kernel<<<1, 1, 0, s->stream>>>(s->st, P.end_time, limit);
    CUDA_TRY(cudaGetLastError());
    s->launches += 1;
    int chunk = 1;
    for (;;) {
        const int r = enqueue_steps(s, P, chunk);
        if (r) return r;
        CUDA_TRY(cudaMemcpyAsync(s->st_host, s->st, sizeof(StepState), cudaMemcpyDeviceToHost, s->stream));
        CUDA_TRY(cudaStreamSynchronize(s->stream));
        s->st_host_valid = true;
        if (s->st_host->done) break;
        s->st_host_valid = false;
        // steps queued after the one that ended the advance return at once
        // (done), leaving the state and the saved mask as that step left them
        if (chunk < 64) chunk *= 2;
    }
    if (s->st_host->status == kStatusTmaTimeout) {
        char msg[256];
        snprintf(msg, sizeof msg, "a TMA halo copy did not complete within the time limit (step %d)",
                 s->st_host->failed_step);
        return fail(GBFV_ERR_CUDA, msg);
    }
    if (s->st_host->status != 0) {
        char msg[256];
        snprintf(msg, sizeof msg,
                 "Simulation state does not obey constraints! At time %.17g, number of timesteps performed %d",
                 s->st_host->t, s->st_host->failed_step);
        return fail(GBFV_ERR_CONSTRAINT, msg);
    }
    return GBFV_OK;
}

// Makes candidate idx current: encodes its tensor maps of U, V, L. False
// (nothing changed) when the grid cannot be staged by TMA.
static bool try_candidate(gbfv_solver* s, int idx) {
    int n = 0;
    const StageCandidate* c = candidates(s->var, s->eq, s->fl, s->rc, s->G.dim, &n);
    if (c[idx].tma) {
        CUtensorMap m[3];
        void* bufs[3] = {s->U, s->V, s->L};
        for (int k = 0; k < 3; ++k)
            if (!gbfv_encode_state_map(&m[k], bufs[k], s->G, s->nvar, s->elem, c[idx].halo[0], c[idx].halo[1],
                                       c[idx].halo[2]))
                return false;
        std::memcpy(s->tm, m, sizeof m);
        s->tm_ok = true;
    }
    s->cand = idx;
    return true;
}

static int use_candidate(gbfv_solver* s, int idx) {
    int n = 0;
    candidates(s->var, s->eq, s->fl, s->rc, s->G.dim, &n);
    if (idx < 0 || idx >= n) return fail(GBFV_ERR_ARGUMENT, "no such stage kernel candidate");
    if (!try_candidate(s, idx))
        return fail(GBFV_ERR_UNSUPPORTED,
                    "this grid cannot be staged by TMA (padded rows must be multiples of 16 bytes)");
    return GBFV_OK;
}

// The autotuner: times MODE_L launches of every candidate on the solver's
// current state (out = L, a scratch step state: no effect on the solve) and
// keeps the fastest; the choice is cached per scheme and grid for the
// process. GBFV_AUTOTUNE=0 in the environment keeps candidate 0.
constexpr long long kTuneFloorCells = 4096;

static int tune(gbfv_solver* s, bool force) {
    int n = 0;
    const StageCandidate* c = candidates(s->var, s->eq, s->fl, s->rc, s->G.dim, &n);
    s->tune_ms.assign(n, -1.0);
    char key[160];
    snprintf(key, sizeof key, "solver:%d:%d:%d:%d:%d:%d:%d:%d", s->var, s->eq, s->fl, s->rc, s->in, s->G.n[0],
             s->G.n[1], s->G.n[2]);
    int best = 0;
    if (n <= 1 || !gbfv_autotune_enabled()) return use_candidate(s, 0);
    // grids below kTuneFloorCells interior cells launch a handful of CTAs per
    // stage: every candidate times the same within the launch latency, and
    // timing them would cost more launches than a short solve makes
    const long long cells = (long long)s->G.n[0] * s->G.n[1] * s->G.n[2];
    if (!force && cells < kTuneFloorCells) return use_candidate(s, 0);
    if (!force && gbfv_tune_cache_get(key, &best) && best < n && try_candidate(s, best)) return GBFV_OK;
    StepState z;
    std::memset(&z, 0, sizeof z);
    cudaEvent_t e0, e1;
    CUDA_TRY(cudaEventCreate(&e0));
    CUDA_TRY(cudaEventCreate(&e1));
    double best_ms = 0;
    best = 0;
    const int kTimed = 3;
    int err = GBFV_OK;
    for (int i = 0; i < n && err == GBFV_OK; ++i) {
        if (!try_candidate(s, i)) continue;  // not eligible (TMA rules)
        cudaError_t e = cudaMemcpyAsync(s->st_op, &z, sizeof z, cudaMemcpyHostToDevice, s->stream);
        int r = e == cudaSuccess ? 0 : (int)e;
        // SSP-RK3: one step is MODE_L plus two combination stages, timed as
        // L + 2 x stage 1 (stage 1 writes the V scratch; dt = 0 in st_op)
        const int nmodes = s->in == IN_RK3 ? 2 : 1;
        double step_ms = 0;
        for (int m = 0; m < nmodes && !r; ++m) {
            const StageArgs a = m == 0 ? stage_args(s, s->st_op, s->U, s->U, nullptr, s->L, MODE_L, 0)
                                       : stage_args(s, s->st_op, s->U, s->U, s->L, s->V, MODE_RK3_S1, 0);
            r = launch_candidate(s, c[i], a);  // warm-up
            if (!r) r = (int)cudaEventRecord(e0, s->stream);
            for (int k = 0; k < kTimed && !r; ++k) r = launch_candidate(s, c[i], a);
            if (!r) r = (int)cudaEventRecord(e1, s->stream);
            if (!r) r = (int)cudaEventSynchronize(e1);
            float ms = 0;
            if (!r) r = (int)cudaEventElapsedTime(&ms, e0, e1);
            step_ms += (m == 0 ? 1.0 : 2.0) * ms / kTimed;
            s->launches += 1 + kTimed;
        }
        if (r) {
            err = fail(GBFV_ERR_CUDA, std::string("autotuning launch: ") + cudaGetErrorString((cudaError_t)r));
            break;
        }
        // per stage launch of one step
        s->tune_ms[i] = step_ms / (nmodes == 2 ? 3.0 : 1.0);
        if (i == 0 || s->tune_ms[i] < best_ms) {
            best_ms = s->tune_ms[i];
            best = i;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (err) return err;
    gbfv_tune_cache_put(key, best);
    return use_candidate(s, best);
}

static StepParams step_params(const gbfv_solver* s, double end_time) {
    StepParams P;
    P.cfl = s->cfl;
    for (int k = 0; k < 3; ++k) P.cell_lengths[k] = s->cell_lengths[k];
    P.end_time = end_time;
    P.time_interval = 0.0;
    P.dim = s->G.dim;
    return P;
}

// The host copy of the step state, fetched unless it is current.
static int sync_step_state(gbfv_solver* s) {
    if (s->st_host_valid) return GBFV_OK;
    CUDA_TRY(cudaMemcpyAsync(s->st_host, s->st, sizeof(StepState), cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    s->st_host_valid = true;
    return GBFV_OK;
}

int gbfv_advance(gbfv_solver* s, double end_time, int number_of_saves, int max_steps) {
    if (!s) return fail(GBFV_ERR_ARGUMENT, "null solver");
    {
        const int r = sync_step_state(s);
        if (r) return r;
    }
    const long long limit = max_steps > 0 ? s->st_host->steps + max_steps : -1;
    if (number_of_saves > 0) s->time_interval = end_time / number_of_saves;
    StepParams P = step_params(s, end_time);
    P.time_interval = number_of_saves > 0 ? s->time_interval : 0.0;
    return drive(s, P, limit);
}

int gbfv_advance_schedule(gbfv_solver* s, const gbfv_schedule* sch, int* saved_mask) {
    if (!s || !sch) return fail(GBFV_ERR_ARGUMENT, "null argument");
    if (!(sch->save_interval[0] >= 0) || !(sch->save_interval[1] >= 0))
        return fail(GBFV_ERR_ARGUMENT, "save intervals must be non-negative");
    if (saved_mask) *saved_mask = 0;
    {
        const int r = sync_step_state(s);
        if (r) return r;
    }
    const long long steps0 = s->st_host->steps;
    const long long limit = sch->max_steps > 0 ? steps0 + sch->max_steps : -1;
    StepParams P = step_params(s, sch->end_time);
    P.time_interval = sch->save_interval[0];
    P.time_interval2 = sch->save_interval[1];
    P.stop_at_save = sch->stop_at_save != 0;
    const int r = drive(s, P, limit);
    if (saved_mask && s->st_host->steps > steps0) *saved_mask = s->st_host->saved_mask;
    return r;
}

int gbfv_stream(gbfv_solver* s, void** stream) {
    if (!s || !stream) return fail(GBFV_ERR_ARGUMENT, "null argument");
    *stream = (void*)s->stream;
    return GBFV_OK;
}

int gbfv_candidate_count(gbfv_solver* s, int* count) {
    if (!s || !count) return fail(GBFV_ERR_ARGUMENT, "null argument");
    candidates(s->var, s->eq, s->fl, s->rc, s->G.dim, count);
    return GBFV_OK;
}

int gbfv_candidate_info(gbfv_solver* s, int idx, int tile[3], int* threads, int* tma) {
    if (!s) return fail(GBFV_ERR_ARGUMENT, "null solver");
    int n = 0;
    const StageCandidate* c = candidates(s->var, s->eq, s->fl, s->rc, s->G.dim, &n);
    if (idx < 0 || idx >= n) return fail(GBFV_ERR_ARGUMENT, "no such stage kernel candidate");
    if (tile)
        for (int k = 0; k < 3; ++k) tile[k] = c[idx].tile[k];
    if (threads) *threads = c[idx].threads;
    if (tma) *tma = c[idx].tma;
    return GBFV_OK;
}

int gbfv_select_candidate(gbfv_solver* s, int idx) {
    if (!s) return fail(GBFV_ERR_ARGUMENT, "null solver");
    if (idx < 0) {
        s->cand = -1;
        s->pinned = false;
        return GBFV_OK;
    }
    const int r = use_candidate(s, idx);
    if (r == GBFV_OK) s->pinned = true;
    return r;
}

int gbfv_current_candidate(gbfv_solver* s, int* idx) {
    if (!s || !idx) return fail(GBFV_ERR_ARGUMENT, "null argument");
    *idx = s->cand;
    return GBFV_OK;
}

int gbfv_autotune(gbfv_solver* s, int* chosen, double* ms, int capacity) {
    if (!s) return fail(GBFV_ERR_ARGUMENT, "null solver");
    const int r = tune(s, true);
    if (r) return r;
    s->pinned = false;
    if (chosen) *chosen = s->cand;
    if (ms)
        for (int i = 0; i < capacity; ++i) ms[i] = i < (int)s->tune_ms.size() ? s->tune_ms[i] : -1.0;
    return GBFV_OK;
}

int gbfv_profile(gbfv_solver* s, int enable) {
    if (!s) return fail(GBFV_ERR_ARGUMENT, "null solver");
    s->profiling = enable != 0;
    return GBFV_OK;
}

int gbfv_profile_read(gbfv_solver* s, double* stage_ms, long long* stage_launches, long long* kernel_launches) {
    if (!s) return fail(GBFV_ERR_ARGUMENT, "null solver");
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    double total = 0;
    for (auto& e : s->events) {
        float ms = 0;
        CUDA_TRY(cudaEventElapsedTime(&ms, e.first, e.second));
        total += ms;
        s->event_pool.push_back(e.first);
        s->event_pool.push_back(e.second);
    }
    if (stage_ms) *stage_ms = total;
    if (stage_launches) *stage_launches = (long long)s->events.size();
    if (kernel_launches) *kernel_launches = s->launches;
    s->events.clear();
    return GBFV_OK;
}

int gbfv_time(gbfv_solver* s, double* t, long long* steps, double* last_dt) {
    if (!s) return fail(GBFV_ERR_ARGUMENT, "null solver");
    CUDA_TRY(cudaMemcpyAsync(s->st_host, s->st, sizeof(StepState), cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    if (t) *t = s->st_host->t;
    if (steps) *steps = s->st_host->steps;
    if (last_dt) *last_dt = s->st_host->dt;
    return GBFV_OK;
}

// The device address of a host buffer the GPU reads and writes in place
// (pinned memory mapped into the device's address space; on a GB300 node
// the accesses travel over NVLink-C2C), or null.
static void* mapped_host(const void* host) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type != cudaMemoryTypeHost || !a.devicePointer) return nullptr;
    return a.devicePointer;
}

// One time step on a state in mapped host memory, without the two state
// copies: the first stage reads the host state itself (the default
// candidate's per-thread loads) and writes the device copy the later stages
// read, and the last stage writes its result to the host state as well as
// to the device state. The copies' link time overlaps the FP64-bound stage
// arithmetic. The same kernels compute every cell, so the result is the
// copying path's bit for bit. Returns 1 (nothing done) when the step does not
// apply and the copying path must run.
static int advance_host_mapped(gbfv_solver* s, void* hdev, double end_time, int number_of_saves) {
    if (s->cand < 0 && !s->pinned) {
        const int r = tune(s, false);
        if (r) return r;
    }
    {
        const int r = sync_step_state(s);
        if (r) return r;
    }
    if (!(s->st_host->t < end_time) || s->st_host->status != 0) return 1;
    if (number_of_saves > 0) s->time_interval = end_time / number_of_saves;
    StepParams P = step_params(s, end_time);
    P.time_interval = number_of_saves > 0 ? s->time_interval : 0.0;
    s->st_host_valid = false;
    begin_kernel<<<1, 1, 0, s->stream>>>(s->st, P.end_time, s->st_host->steps + 1);
    CUDA_TRY(cudaGetLastError());
    s->launches += 1;
    int ncand = 0;
    const StageCandidate* c = candidates(s->var, s->eq, s->fl, s->rc, s->G.dim, &ncand);
    const StageCandidate& stage = c[s->cand < 0 ? 0 : s->cand];
    cudaStream_t q = s->stream;
    // the first stage reads host memory with per-thread loads: the chosen
    // candidate if it loads that way, else the fastest such candidate the
    // autotuner timed (candidate 0 untuned)
    int first = 0;
    if (s->cand >= 0 && !c[s->cand].tma) {
        first = s->cand;
    } else {
        for (int i = 1; i < ncand && i < (int)s->tune_ms.size(); ++i)
            if (!c[i].tma && s->tune_ms[i] >= 0 && (s->tune_ms[first] < 0 || s->tune_ms[i] < s->tune_ms[first]))
                first = i;
    }
    StageArgs a = stage_args(s, s->st, hdev, hdev, nullptr, s->L, MODE_L, 0);
    a.copy_in = s->U;
    STAGE_TRY(launch_stage(s, c[first], a));
    dt_kernel<<<1, 1, 0, q>>>(s->st, P);
    CUDA_TRY(cudaGetLastError());
    s->launches += 2;  // dt + finish
    if (s->in == IN_RK3) {
        STAGE_TRY(launch_stage(s, stage, stage_args(s, s->st, s->U, s->U, s->L, s->V, MODE_RK3_S1, 0)));
        StageArgs b = stage_args(s, s->st, s->V, s->U, nullptr, s->U, MODE_RK3_S2, 1);
        b.out2 = hdev;
        STAGE_TRY(launch_stage(s, stage, b));
    } else {
        StageArgs b = stage_args(s, s->st, s->U, s->U, s->L, s->V, MODE_RK2_S1, 1);
        b.out2 = hdev;
        STAGE_TRY(launch_stage(s, stage, b));
        s->launches += 1;
        const long long n = (long long)s->nvar * s->G.total;
        copy_state_kernel<double><<<1184, 256, 0, q>>>(s->st, (const double*)s->V, (double*)s->U, n);
        CUDA_TRY(cudaGetLastError());
    }
    finish_kernel<<<1, 1, 0, q>>>(s->st, P);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpyAsync(s->st_host, s->st, sizeof(StepState), cudaMemcpyDeviceToHost, q));
    CUDA_TRY(cudaStreamSynchronize(q));
    s->st_host_valid = true;
    if (s->st_host->status == kStatusTmaTimeout) {
        char msg[256];
        snprintf(msg, sizeof msg, "a TMA halo copy did not complete within the time limit (step %d)",
                 s->st_host->failed_step);
        return fail(GBFV_ERR_CUDA, msg);
    }
    if (s->st_host->status != 0) {
        char msg[256];
        snprintf(msg, sizeof msg,
                 "Simulation state does not obey constraints! At time %.17g, number of timesteps performed %d",
                 s->st_host->t, s->st_host->failed_step);
        return fail(GBFV_ERR_CONSTRAINT, msg);
    }
    return GBFV_OK;
}

int gbfv_advance_host(gbfv_solver* s, double* host, double end_time, int number_of_saves, int max_steps) {
    if (!s || !host) return fail(GBFV_ERR_ARGUMENT, "null argument");
    // one step of an FP64 state in mapped (pinned) host memory: in place
    if (max_steps == 1 && !s->profiling && (s->var == VAR_F64 || s->var == VAR_F64_EXACT) &&
        (s->in == IN_RK3 || s->in == IN_RK2)) {
        void* hdev = mapped_host(host);
        if (hdev) {
            const int r = advance_host_mapped(s, hdev, end_time, number_of_saves);
            if (r <= 0) return r;
        }
    }
    int r = upload(s, host);
    if (r) return r;
    r = gbfv_advance(s, end_time, number_of_saves, max_steps);
    const int r2 = download(s, host);
    return r ? r : r2;
}

// ------------------------------------------------------ operator level

int gbfv_compute_flux(gbfv_solver* s, const void* U, void* out, double ws[3]) {
    if (!s || !U || !out) return fail(GBFV_ERR_ARGUMENT, "null argument");
    StepState z;
    std::memset(&z, 0, sizeof z);
    CUDA_TRY(cudaMemcpyAsync(s->st_op, &z, sizeof z, cudaMemcpyHostToDevice, s->stream));
    int ncand = 0;
    const StageCandidate* c = candidates(s->var, s->eq, s->fl, s->rc, s->G.dim, &ncand);
    LAUNCH_TRY(c[0].stage(stage_args(s, s->st_op, U, U, nullptr, out, MODE_L, 0), nullptr, s->stream));
    CUDA_TRY(cudaMemcpyAsync(s->st_host, s->st_op, sizeof(StepState), cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    if (ws)
        for (int d = 0; d < 3; ++d) {
            unsigned long long b = s->st_host->ws_bits[d];
            double v;
            std::memcpy(&v, &b, sizeof v);
            ws[d] = d < s->G.dim ? v : 0.0;
        }
    return GBFV_OK;
}

int gbfv_reconstruct(gbfv_solver* s, int direction, const void* U, void* left, void* right) {
    if (!s || !U || !left || !right) return fail(GBFV_ERR_ARGUMENT, "null argument");
    if (direction < 0 || direction >= s->G.dim) return fail(GBFV_ERR_ARGUMENT, "bad direction");
    ReconArgs a;
    std::memset(&a, 0, sizeof a);
    a.in = U;
    a.left = left;
    a.right = right;
    a.G = s->G;
    a.dir = direction;
    a.gamma = s->gamma;
    LAUNCH_TRY(registry().recon[s->var][s->eq][s->rc](a, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    return GBFV_OK;
}

int gbfv_apply_boundary(gbfv_solver* s, void* U) {
    if (!s || !U) return fail(GBFV_ERR_ARGUMENT, "null argument");
    int r = launch_boundary(s, U);
    if (r) return r;
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    return GBFV_OK;
}

int gbfv_obeys_constraints(gbfv_solver* s, const void* U, int* ok) {
    if (!s || !U || !ok) return fail(GBFV_ERR_ARGUMENT, "null argument");
    *s->flag_host = 1;
    CUDA_TRY(cudaMemcpyAsync(s->flag, s->flag_host, sizeof(int), cudaMemcpyHostToDevice, s->stream));
    CheckArgs a;
    a.in = U;
    a.flag = s->flag;
    a.G = s->G;
    a.gamma = s->gamma;
    LAUNCH_TRY(registry().check[s->var][s->eq](a, s->stream));
    CUDA_TRY(cudaMemcpyAsync(s->flag_host, s->flag, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    *ok = *s->flag_host;
    return GBFV_OK;
}

// ------------------------------------- operator level, one array per variable

// The arrays of one volume are a padded block (variable k at base + k * total
// elements) or nvar separate allocations, as the reference's Volume holds
// them (one Memory per variable).
static bool contiguous(const gbfv_solver* s, const void* const* vars) {
    const char* b = (const char*)vars[0];
    for (int k = 1; k < s->nvar; ++k)
        if ((const char*)vars[k] != b + (size_t)k * s->G.total * s->elem) return false;
    return true;
}

static bool all_set(const gbfv_solver* s, const void* const* vars) {
    if (!vars) return false;
    for (int k = 0; k < s->nvar; ++k)
        if (!vars[k]) return false;
    return true;
}

// Scratch block of the solver for the gather / scatter of separate arrays
// (allocated at its first use; the step buffers V and L serve as the others).
static int op_scratch(gbfv_solver* s, void** p) {
    if (!s->op_block) {
        cudaError_t e = cudaMalloc(&s->op_block, state_bytes(s));
        if (e != cudaSuccess) {
            s->op_block = nullptr;
            return fail(e == cudaErrorMemoryAllocation ? GBFV_ERR_MEMORY : GBFV_ERR_CUDA,
                        std::string("operator scratch: ") + cudaGetErrorString(e));
        }
    }
    *p = s->op_block;
    return GBFV_OK;
}

static int gather(gbfv_solver* s, const void* const* vars, void* block, cudaStream_t q) {
    const size_t bytes = (size_t)s->G.total * s->elem;
    for (int k = 0; k < s->nvar; ++k)
        CUDA_TRY(cudaMemcpyAsync((char*)block + k * bytes, vars[k], bytes, cudaMemcpyDeviceToDevice, q));
    return GBFV_OK;
}

static int scatter(gbfv_solver* s, const void* block, void* const* vars, cudaStream_t q) {
    const size_t bytes = (size_t)s->G.total * s->elem;
    for (int k = 0; k < s->nvar; ++k)
        CUDA_TRY(cudaMemcpyAsync(vars[k], (const char*)block + k * bytes, bytes, cudaMemcpyDeviceToDevice, q));
    return GBFV_OK;
}

int gbfv_compute_flux_region(gbfv_solver* s, const void* const* state_vars, void* const* out_vars, double ws[3],
                             const int start[3], const int end[3], void* stream) {
    if (!s || !all_set(s, state_vars) || !all_set(s, (const void* const*)out_vars))
        return fail(GBFV_ERR_ARGUMENT, "gbfv_compute_flux_region: null argument");
    int lo[3], hi[3];
    bool empty = false;
    for (int d = 0; d < 3; ++d) {
        const int a = start ? start[d] : 0, b = end ? end[d] : 0;
        if (d >= s->G.dim) {
            if (a != 0 || b != 0) return fail(GBFV_ERR_ARGUMENT, "start / end of an inactive dimension must be 0");
            lo[d] = 0;
            hi[d] = 1;
            continue;
        }
        lo[d] = a;
        hi[d] = s->G.n[d] + b;
        if (lo[d] < 0 || hi[d] > s->G.n[d])
            return fail(GBFV_ERR_ARGUMENT, "gbfv_compute_flux_region: the region leaves the interior");
        if (hi[d] <= lo[d]) empty = true;
    }
    if (ws)
        for (int d = 0; d < 3; ++d) ws[d] = 0.0;
    if (empty) return GBFV_OK;
    const RegionLauncher launch = registry().region[s->var][s->eq][s->fl][s->rc][s->G.dim - 1];
    if (!launch) return fail(GBFV_ERR_UNSUPPORTED, "no region kernel for this scheme");
    cudaStream_t q = stream ? (cudaStream_t)stream : s->stream;
    CUDA_TRY(cudaMemsetAsync(s->st_op, 0, sizeof(StepState), q));
    StageArgs a = stage_args(s, s->st_op, state_vars[0], nullptr, nullptr, out_vars[0], MODE_L, 0);
    for (int d = 0; d < 3; ++d) {
        a.rlo[d] = lo[d];
        a.rhi[d] = hi[d];
    }
    for (int k = 0; k < s->nvar; ++k) {
        a.vin[k] = state_vars[k];
        a.vout[k] = out_vars[k];
    }
    LAUNCH_TRY(launch(a, q));
    s->launches += 1;
    CUDA_TRY(cudaMemcpyAsync(s->st_host, s->st_op, sizeof(StepState), cudaMemcpyDeviceToHost, q));
    CUDA_TRY(cudaStreamSynchronize(q));
    if (ws)
        for (int d = 0; d < s->G.dim; ++d) {
            unsigned long long b = s->st_host->ws_bits[d];
            std::memcpy(&ws[d], &b, sizeof(double));
        }
    return GBFV_OK;
}

int gbfv_reconstruct_vars(gbfv_solver* s, int direction, const void* const* state_vars, void* const* left_vars,
                          void* const* right_vars, const int start[3], const int end[3], void* stream) {
    if (!s || !all_set(s, state_vars) || !all_set(s, (const void* const*)left_vars) ||
        !all_set(s, (const void* const*)right_vars))
        return fail(GBFV_ERR_ARGUMENT, "gbfv_reconstruct_vars: null argument");
    if (direction < 0 || direction >= s->G.dim) return fail(GBFV_ERR_ARGUMENT, "bad direction");
    cudaStream_t q = stream ? (cudaStream_t)stream : s->stream;
    ReconArgs a;
    std::memset(&a, 0, sizeof a);
    a.G = s->G;
    a.dir = direction;
    a.gamma = s->gamma;
    for (int d = 0; d < 3; ++d) {
        a.start[d] = d < s->G.dim && start ? start[d] : 0;
        a.end[d] = d < s->G.dim && end ? end[d] : 0;
    }
    const bool c = contiguous(s, state_vars) && contiguous(s, (const void* const*)left_vars) &&
                   contiguous(s, (const void* const*)right_vars);
    void* blk = nullptr;
    if (c) {
        a.in = state_vars[0];
        a.left = left_vars[0];
        a.right = right_vars[0];
    } else {
        // separate arrays: through the solver's step buffers and scratch (the
        // outputs are gathered too, so cells outside the range keep their values)
        int r = op_scratch(s, &blk);
        if (!r) r = gather(s, state_vars, blk, q);
        if (!r) r = gather(s, (const void* const*)left_vars, s->V, q);
        if (!r) r = gather(s, (const void* const*)right_vars, s->L, q);
        if (r) return r;
        a.in = blk;
        a.left = s->V;
        a.right = s->L;
    }
    LAUNCH_TRY(registry().recon[s->var][s->eq][s->rc](a, q));
    s->launches += 1;
    if (!c) {
        int r = scatter(s, s->V, left_vars, q);
        if (!r) r = scatter(s, s->L, right_vars, q);
        if (r) return r;
    }
    CUDA_TRY(cudaStreamSynchronize(q));
    return GBFV_OK;
}

int gbfv_apply_boundary_vars(gbfv_solver* s, void* const* vars, void* stream) {
    if (!s || !all_set(s, (const void* const*)vars)) return fail(GBFV_ERR_ARGUMENT, "null argument");
    cudaStream_t q = stream ? (cudaStream_t)stream : s->stream;
    const bool c = contiguous(s, (const void* const*)vars);
    void* blk = vars[0];
    if (!c) {
        int r = op_scratch(s, &blk);
        if (!r) r = gather(s, (const void* const*)vars, blk, q);
        if (r) return r;
    }
    cudaStream_t own = s->stream;
    s->stream = q;
    int r = launch_boundary(s, blk);
    s->stream = own;
    if (r) return r;
    s->launches += 1;
    if (!c) {
        r = scatter(s, blk, vars, q);
        if (r) return r;
    }
    CUDA_TRY(cudaStreamSynchronize(q));
    return GBFV_OK;
}

int gbfv_obeys_constraints_vars(gbfv_solver* s, const void* const* vars, int* ok, void* stream) {
    if (!s || !ok || !all_set(s, vars)) return fail(GBFV_ERR_ARGUMENT, "null argument");
    cudaStream_t q = stream ? (cudaStream_t)stream : s->stream;
    const void* blk = vars[0];
    if (!contiguous(s, vars)) {
        void* b = nullptr;
        int r = op_scratch(s, &b);
        if (!r) r = gather(s, vars, b, q);
        if (r) return r;
        blk = b;
    }
    *s->flag_host = 1;
    CUDA_TRY(cudaMemcpyAsync(s->flag, s->flag_host, sizeof(int), cudaMemcpyHostToDevice, q));
    CheckArgs a;
    a.in = blk;
    a.flag = s->flag;
    a.G = s->G;
    a.gamma = s->gamma;
    LAUNCH_TRY(registry().check[s->var][s->eq](a, q));
    s->launches += 1;
    CUDA_TRY(cudaMemcpyAsync(s->flag_host, s->flag, sizeof(int), cudaMemcpyDeviceToHost, q));
    CUDA_TRY(cudaStreamSynchronize(q));
    *ok = *s->flag_host;
    return GBFV_OK;
}

}  // extern "C"

// Per-cell maps of CellComputer over every cell of a volume (ghosts
// included), one array per variable, in the element type R of the solver.
struct VarPtrs {
    const void* in[5];
    void* out[5];
};

// computeFromPrimitive: Euler::computeConserved (alsfvm/include/alsfvm/
// equation/euler/Euler.hpp:236-245) in its operand order; Burgers copies u.
template <class R>
__global__ void cells_prim_to_cons_kernel(VarPtrs v, long long total, int eq, R gamma) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    if (eq == EQ_BURGERS) {
        ((R*)v.out[0])[i] = ((const R*)v.in[0])[i];
        return;
    }
    const int nsd = eq;
    const R rho = ((const R*)v.in[0])[i];
    R u[3];
    for (int k = 0; k < nsd; ++k) u[k] = ((const R*)v.in[1 + k])[i];
    const R p = ((const R*)v.in[1 + nsd])[i];
    R dot = u[0] * u[0];
    for (int k = 1; k < nsd; ++k) dot = dot + u[k] * u[k];
    ((R*)v.out[0])[i] = rho;
    for (int k = 0; k < nsd; ++k) ((R*)v.out[1 + k])[i] = u[k] * rho;
    ((R*)v.out[1 + nsd])[i] = p / (gamma - R(1)) + R(0.5) * rho * dot;
}

// computeExtraVariables: Euler::computeExtra (Euler.hpp:204-211): p, then u.
template <class R>
__global__ void cells_extra_kernel(VarPtrs v, long long total, int nsd, R gamma) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    const R rho = ((const R*)v.in[0])[i];
    R m[3];
    for (int k = 0; k < nsd; ++k) m[k] = ((const R*)v.in[1 + k])[i];
    const R E = ((const R*)v.in[1 + nsd])[i];
    R dot = m[0] * m[0];
    for (int k = 1; k < nsd; ++k) dot = dot + m[k] * m[k];
    const R ie = E - R(0.5) * dot / rho;
    ((R*)v.out[0])[i] = (gamma - R(1)) * ie;
    for (int k = 0; k < nsd; ++k) ((R*)v.out[1 + k])[i] = m[k] / rho;
}

// computeMaxWaveSpeed in direction d: the maximum over cells of
// |u_d| + sqrt(gamma p / rho) (Euler.hpp:251-258) or |u| (Burgers); cells
// whose value is not a number are passed over, as std::max passes them.
template <class R>
__global__ void cells_wave_speed_kernel(VarPtrs v, long long total, int eq, int d, R gamma,
                                        unsigned long long* bits) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double w = 0.0;
    if (i < total) {
        if (eq == EQ_BURGERS) {
            w = (double)fabs(((const R*)v.in[0])[i]);
        } else {
            const int nsd = eq;
            const R rho = ((const R*)v.in[0])[i];
            R m[3];
            for (int k = 0; k < nsd; ++k) m[k] = ((const R*)v.in[1 + k])[i];
            const R E = ((const R*)v.in[1 + nsd])[i];
            R dot = m[0] * m[0];
            for (int k = 1; k < nsd; ++k) dot = dot + m[k] * m[k];
            const R p = (gamma - R(1)) * (E - R(0.5) * dot / rho);
            const R ud = d < nsd ? m[d] / rho : R(0);
            w = (double)(fabs(ud) + sqrt(gamma * p / rho));
        }
        if (!(w >= 0.0)) w = 0.0;  // NaN
    }
    for (int off = 16; off > 0; off >>= 1) w = fmax(w, __shfl_xor_sync(0xffffffffu, w, off));
    if ((threadIdx.x & 31) == 0 && w > 0.0) atomicMax(bits, (unsigned long long)__double_as_longlong(w));
}

static int cells_launch(gbfv_solver* s, int which, const void* const* in, void* const* out, int d, double* result,
                        void* stream) {
    cudaStream_t q = stream ? (cudaStream_t)stream : s->stream;
    VarPtrs v;
    std::memset(&v, 0, sizeof v);
    const int nsd = s->eq == EQ_BURGERS ? 1 : s->eq;
    const int nin = which == 0 ? s->nvar : s->nvar;
    const int nout = which == 0 ? s->nvar : (which == 1 ? (s->eq == EQ_BURGERS ? 0 : nsd + 1) : 0);
    for (int k = 0; k < nin; ++k) {
        if (!in[k]) return fail(GBFV_ERR_ARGUMENT, "null variable array");
        v.in[k] = in[k];
    }
    for (int k = 0; k < nout; ++k) {
        if (!out || !out[k]) return fail(GBFV_ERR_ARGUMENT, "null variable array");
        v.out[k] = out[k];
    }
    const long long total = s->G.total;
    const int bs = 256;
    const unsigned nb = (unsigned)((total + bs - 1) / bs);
    if (which == 0) {
        if (s->elem == 8) cells_prim_to_cons_kernel<double><<<nb, bs, 0, q>>>(v, total, s->eq, s->gamma);
        else cells_prim_to_cons_kernel<float><<<nb, bs, 0, q>>>(v, total, s->eq, (float)s->gamma);
    } else if (which == 1) {
        if (nout == 0) return GBFV_OK;  // Burgers has no extra variables
        if (s->elem == 8) cells_extra_kernel<double><<<nb, bs, 0, q>>>(v, total, nsd, s->gamma);
        else cells_extra_kernel<float><<<nb, bs, 0, q>>>(v, total, nsd, (float)s->gamma);
    } else {
        CUDA_TRY(cudaMemsetAsync(s->st_op, 0, sizeof(StepState), q));
        unsigned long long* bits = &s->st_op->ws_bits[0];
        if (s->elem == 8) cells_wave_speed_kernel<double><<<nb, bs, 0, q>>>(v, total, s->eq, d, s->gamma, bits);
        else cells_wave_speed_kernel<float><<<nb, bs, 0, q>>>(v, total, s->eq, d, (float)s->gamma, bits);
        CUDA_TRY(cudaGetLastError());
        CUDA_TRY(cudaMemcpyAsync(s->st_host, s->st_op, sizeof(StepState), cudaMemcpyDeviceToHost, q));
    }
    CUDA_TRY(cudaGetLastError());
    s->launches += 1;
    CUDA_TRY(cudaStreamSynchronize(q));
    if (which == 2 && result) {
        unsigned long long b = s->st_host->ws_bits[0];
        std::memcpy(result, &b, sizeof(double));
    }
    return GBFV_OK;
}

extern "C" {

int gbfv_prim_to_cons_vars(gbfv_solver* s, const void* const* prim_vars, void* const* cons_vars, void* stream) {
    if (!s || !prim_vars || !cons_vars) return fail(GBFV_ERR_ARGUMENT, "null argument");
    return cells_launch(s, 0, prim_vars, cons_vars, 0, nullptr, stream);
}

int gbfv_extra_variables_vars(gbfv_solver* s, const void* const* cons_vars, void* const* extra_vars, void* stream) {
    if (!s || !cons_vars) return fail(GBFV_ERR_ARGUMENT, "null argument");
    return cells_launch(s, 1, cons_vars, extra_vars, 0, nullptr, stream);
}

int gbfv_max_wave_speed_vars(gbfv_solver* s, const void* const* cons_vars, int direction, double* speed,
                             void* stream) {
    if (!s || !cons_vars || !speed || direction < 0 || direction > 2)
        return fail(GBFV_ERR_ARGUMENT, "gbfv_max_wave_speed_vars: bad arguments");
    return cells_launch(s, 2, cons_vars, nullptr, direction, speed, stream);
}

int gbfv_test_tma_wait_limit(gbfv_solver* s, unsigned extra_bytes) {
    if (!s) return fail(GBFV_ERR_ARGUMENT, "null solver");
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    s->tma_extra_tx = extra_bytes;
    // captured step graphs hold the old launch parameters
    if (s->step_graph) {
        cudaGraphExecDestroy(s->step_graph);
        s->step_graph = nullptr;
        s->graph_cand = -2;
    }
    return GBFV_OK;
}

// ------------------------------------------------------- generator

// The process-wide engine of STLMersenne as an object: one mt19937_64 with
// the default seed and the count of numbers it has produced
// (alsuq/src/generator/STLMersenne.cpp:24-29).
struct gbfv_generator {
    std::mt19937_64 engine;
    long long drawn = 0;
};

int gbfv_uniform(int dimension, int sample, double lower, double upper, double* out) {
    if (dimension <= 0 || sample < 0 || !out) return fail(GBFV_ERR_ARGUMENT, "bad arguments");
    std::mt19937_64 gen;  // default seed, as the reference's process-wide engine
    gen.discard((unsigned long long)sample * (unsigned long long)dimension);
    std::uniform_real_distribution<double> dist{0.0, 1.0};
    for (int c = 0; c < dimension; ++c) out[c] = dist(gen) * (upper - lower) + lower;
    return GBFV_OK;
}

int gbfv_generator_create(gbfv_generator** out) {
    if (!out) return fail(GBFV_ERR_ARGUMENT, "null argument");
    *out = new gbfv_generator();
    return GBFV_OK;
}

int gbfv_generator_destroy(gbfv_generator* g) {
    delete g;
    return GBFV_OK;
}

int gbfv_generator_uniform(gbfv_generator* g, int dimension, int component, long long sample, double lower,
                           double upper, double* out) {
    if (!g || !out || dimension <= 0 || component < 0 || sample < 0)
        return fail(GBFV_ERR_ARGUMENT, "bad arguments");
    if (component >= dimension) return fail(GBFV_ERR_ARGUMENT, "Component given higher than dimension");
    const long long dim = dimension;
    // skip forward to the sample's block, then to the component within it;
    // a generator never moves backwards (a repeated or earlier request draws
    // the next number, as the reference's engine does)
    if (g->drawn / dim < sample) {
        const long long skip = sample * dim - g->drawn;
        g->engine.discard((unsigned long long)skip);
        g->drawn += skip;
    }
    if (g->drawn % dim < component) {
        const long long skip = component - g->drawn % dim;
        g->engine.discard((unsigned long long)skip);
        g->drawn += skip;
    }
    g->drawn += 1;
    std::uniform_real_distribution<double> dist{0.0, 1.0};
    *out = dist(g->engine) * (upper - lower) + lower;
    return GBFV_OK;
}

}  // extern "C"

// ------------------------------------------------------------------------
// Helpers for the allocation-free entry point (gbfv_noalloc.cu): the same
// validation as gbfv_create and the same kernel sequence as one gbfv_advance
// step, on buffers the caller provides.

#include "gbfv_internal.h"

int gbfv_internal_plan(const gbfv_desc* d, GbfvPlan* p) {
    if (!d || !p) return fail(GBFV_ERR_ARGUMENT, "null argument");
    const int eq = parse_eq(d->equation), fl = parse_flux(d->flux), rc = parse_recon(d->reconstruction);
    const int in = parse_integrator(d->integrator), bc = parse_bc(d->boundary);
    if (eq < 0 || fl < 0 || rc < 0 || in < 0 || bc < 0) return fail(GBFV_ERR_ARGUMENT, "unknown name in descriptor");
    if (!flux_applies(eq, fl)) return fail(GBFV_ERR_UNSUPPORTED, "flux does not apply to this equation");
    if (d->precision < 0 || d->precision >= NUM_VARIANTS) return fail(GBFV_ERR_ARGUMENT, "bad precision");
    for (int k = 0; k < 3; ++k)
        if (d->n[k] < 1) return fail(GBFV_ERR_ARGUMENT, "grid dimensions must be >= 1");
    const int dim = d->n[2] > 1 ? 3 : (d->n[1] > 1 ? 2 : 1);
    if (eq != EQ_BURGERS && eq != dim) return fail(GBFV_ERR_UNSUPPORTED, "euler<d> needs a d-dimensional grid");
    const int g = kReconGhosts[rc];
    for (int k = 0; k < dim; ++k)
        if (d->n[k] < g) return fail(GBFV_ERR_UNSUPPORTED, "every active dimension needs at least as many cells as ghost cells");
    p->eq = eq; p->fl = fl; p->rc = rc; p->in = in; p->periodic = bc; p->var = d->precision;
    p->nvar = eq == EQ_BURGERS ? 1 : eq + 2;
    p->elem = d->precision == VAR_F32 ? 4 : 8;
    p->gamma = d->gamma;
    p->cfl = d->cfl;
    p->G.dim = dim;
    long long total = 1;
    for (int k = 0; k < 3; ++k) {
        p->G.n[k] = d->n[k];
        p->G.g[k] = k < dim ? g : 0;
        p->G.t[k] = d->n[k] + 2 * p->G.g[k];
        total *= p->G.t[k];
    }
    p->G.total = total;
    for (int k = 0; k < 3; ++k) p->cell_lengths[k] = (d->upper[k] - d->lower[k]) / d->n[k];
    if (d->n[1] == 1) p->cell_lengths[1] = 1;
    if (d->n[2] == 1) p->cell_lengths[2] = 1;
    return GBFV_OK;
}

int gbfv_internal_begin(StepState* st, double end_time, long long step_limit, cudaStream_t q) {
    begin_kernel<<<1, 1, 0, q>>>(st, end_time, step_limit);
    CUDA_TRY(cudaGetLastError());
    return GBFV_OK;
}

int gbfv_internal_step(const GbfvPlan& p, void* U, void* V, void* L, StepState* st, const StepParams& P,
                       cudaStream_t q) {
    Registry& R = registry();
    int ncand = 0;
    // caller buffers: the default candidate (plain halo loads, no tensor maps)
    const StageLauncher launch0 = candidates(p.var, p.eq, p.fl, p.rc, p.G.dim, &ncand)[0].stage;
    auto stage = [&](const StageArgs& a, cudaStream_t qq) { return launch0(a, nullptr, qq); };
    auto args = [&](const void* in, const void* u0, const void* l0, void* out, int mode, int check) {
        StageArgs a;
        std::memset(&a, 0, sizeof a);
        a.in = in; a.u0 = u0; a.l0 = l0; a.out = out; a.st = st; a.G = p.G; a.gamma = p.gamma;
        a.gamma_f = (float)p.gamma;
        a.tm_in = nullptr; a.tm_l0 = nullptr;
        a.mode = mode; a.periodic = p.periodic; a.check = check;
        return a;
    };
    LAUNCH_TRY(stage(args(U, U, nullptr, L, MODE_L, 0), q));
    dt_kernel<<<1, 1, 0, q>>>(st, P);
    CUDA_TRY(cudaGetLastError());
    if (p.in == IN_RK3) {
        LAUNCH_TRY(stage(args(U, U, L, V, MODE_RK3_S1, 0), q));
        LAUNCH_TRY(stage(args(V, U, nullptr, U, MODE_RK3_S2, 1), q));
    } else if (p.in == IN_RK2) {
        LAUNCH_TRY(stage(args(U, U, L, V, MODE_RK2_S1, 1), q));
        const long long n = (long long)p.nvar * p.G.total;
        if (p.elem == 8)
            copy_state_kernel<double><<<1184, 256, 0, q>>>(st, (const double*)V, (double*)U, n);
        else
            copy_state_kernel<float><<<1184, 256, 0, q>>>(st, (const float*)V, (float*)U, n);
        CUDA_TRY(cudaGetLastError());
    } else {
        LAUNCH_TRY(R.apply[p.var][p.eq](args(U, U, L, U, MODE_L, 1), q));
    }
    finish_kernel<<<1, 1, 0, q>>>(st, P);
    CUDA_TRY(cudaGetLastError());
    return GBFV_OK;
}

// Host primitive -> conserved conversion into a padded array (interior cells;
// ghosts left at zero), as gbfv_set_primitive does.
int gbfv_internal_prim_to_cons(const GbfvPlan& p, const double* prim, double* cons) {
    prim_to_cons(p.eq, p.gamma, p.G, prim, cons);
    return GBFV_OK;
}

// Uploads a padded double state into a device state of the plan's precision
// and fills its ghost cells.
int gbfv_internal_load_state(const GbfvPlan& p, const double* host, void* dev, cudaStream_t q) {
    const size_t n = (size_t)p.nvar * p.G.total;
    if (p.elem == 8) {
        CUDA_TRY(cudaMemcpyAsync(dev, host, n * 8, cudaMemcpyHostToDevice, q));
        CUDA_TRY(cudaStreamSynchronize(q));
    } else {
        std::vector<float> f(n);
        for (size_t i = 0; i < n; ++i) f[i] = (float)host[i];
        CUDA_TRY(cudaMemcpyAsync(dev, f.data(), n * 4, cudaMemcpyHostToDevice, q));
        CUDA_TRY(cudaStreamSynchronize(q));
    }
    const int bs = 256;
    const unsigned nb = (unsigned)((p.G.total + bs - 1) / bs);
    if (p.elem == 8)
        boundary_kernel<double><<<nb, bs, 0, q>>>((double*)dev, p.G, p.nvar, p.periodic);
    else
        boundary_kernel<float><<<nb, bs, 0, q>>>((float*)dev, p.G, p.nvar, p.periodic);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaStreamSynchronize(q));
    return GBFV_OK;
}
