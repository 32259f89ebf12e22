// Ensemble engine: many grids (members) of one scheme advanced together.
//
// alsuq runs its samples one after another, rebuilding a Simulator per sample
// (alsuq/src/run/Runner.cpp:39-90). Here every member lives in one device pool
// and each RK stage of the whole ensemble is one persistent launch over a tile
// list that spans all members (batch_stage_kernel). Each member keeps its own
// step state, so its dt comes from its own wave-speed maximum (a segmented
// CFL reduction) and its own save-time clamp; members that reach end_time stop
// while the rest continue. One time step of the ensemble is captured once as
// a CUDA graph and replayed. Final states are folded into FP64 Welford mean /
// variance accumulators per statistics group (MeanVariance with
// FixedIntervalStatistics at the end time, alsuq/src/stats/MeanVariance.cpp:
// 30-67, FixedIntervalStatistics.cpp:33-86), in member order, so the result
// does not depend on which members finish in the same step.
//
// Members join and leave between advance calls (the serving loop's slots);
// memory for them comes from one pool allocated at creation, so admission is
// bounded by that pool (the HBM budget).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <limits>
#include <map>
#include <string>
#include <vector>

#include "fv_registry.h"
#include "fv_tma.cuh"
#include "gbfv_internal.h"

using namespace gbfv;

namespace {

struct MemberParam {
    double cell_lengths[3];
    double time_interval;  // save-time clamp interval (0: none): the statistics' (FixedIntervalStatistics)
    double time_interval2; // second clamp (0: none): the fvm writer's (FixedIntervalWriter)
    double end_time;       // the member's own end time (+inf: the advance's)
    int dim;
    int active;
};

struct GroupAcc {
    double* mean;
    double* m2;
    long long cells;  // nvar * padded total of the group's grid
    long long count;  // members folded in
};

// per-member dt (Integrator::computeTimestep + the save-time clamp)
__global__ void batch_dt_kernel(StepState* st, const MemberParam* mp, int M, double cfl) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= M || !mp[s].active || st[s].done) return;
    set_step_dt(st[s], mp[s].dim, mp[s].cell_lengths, cfl, mp[s].time_interval, mp[s].time_interval2);
}

__global__ void batch_finish_kernel(StepState* st, const MemberParam* mp, int M, int alternate) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= M || !mp[s].active || st[s].done) return;
    StepState& S = st[s];
    const MemberParam& P = mp[s];
    S.t = S.t + S.dt;
    S.steps += 1;
    S.just_saved = -1;
    if (P.time_interval > 0 && S.t >= (double)S.number_saved * P.time_interval + 0.0) {
        S.just_saved = (int)(S.number_saved - 1);  // save index k reached: t >= (k + 1) * interval
        S.number_saved += 1;
    }
    if (P.time_interval2 > 0 && S.t >= (double)S.number_saved2 * P.time_interval2) S.number_saved2 += 1;
    S.ws_bits[0] = S.ws_bits[1] = S.ws_bits[2] = 0ull;
    if (alternate) S.parity ^= 1;
    const bool reached = !(S.t < S.end_time);
    if (reached || (S.step_limit >= 0 && S.steps >= S.step_limit) || S.status != 0) {
        S.done = 1;
        S.just_done = (reached && S.status == 0) ? 1 : 0;
    }
}

__global__ void batch_begin_kernel(StepState* st, const MemberParam* mp, int M, double end_time, long long max_steps) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= M) return;
    StepState& S = st[s];
    if (!mp[s].active) {
        S.done = 1;
        return;
    }
    const double end = mp[s].end_time < end_time ? mp[s].end_time : end_time;
    S.end_time = end;
    S.step_limit = max_steps > 0 ? S.steps + max_steps : -1;
    S.ws_bits[0] = S.ws_bits[1] = S.ws_bits[2] = 0ull;
    S.just_done = 0;
    S.done = (!(S.t < end) || S.status != 0) ? 1 : 0;
}

// Welford order: members to fold in this step, in member order. With one
// statistics save a member is folded when it reaches end_time; with nsaves
// saves (FixedIntervalStatistics at (k + 1) end_time / nsaves) it is folded
// into accumulator (group, k) at each save k its clamp stopped it at.
// list[i] = (member, accumulator, count after the fold). All threads read the
// members' flags in parallel; one warp then numbers the (few) folds in order.
constexpr int kAssignThreads = 1024;
constexpr int kAssignChunk = 4096;
__global__ void __launch_bounds__(kAssignThreads) batch_assign_kernel(StepState* st, const MemberParam* mp, int M,
                                                                      GroupAcc* accs, int nacc, int nsaves,
                                                                      int4* list, int* nlist) {
    // every thread: the accumulator index of members of the chunk (and their
    // flags cleared); then warp 0 compacts the list in member order, so the
    // counts each group's members receive follow the member order
    __shared__ int acc_of[kAssignChunk];
    __shared__ int m_shared;
    if (threadIdx.x == 0) m_shared = 0;
    for (int base0 = 0; base0 < M; base0 += kAssignChunk) {
        const int len = min(kAssignChunk, M - base0);
        for (int i = threadIdx.x; i < len; i += blockDim.x) {
            const int s = base0 + i;
            int a = -1;
            const int done = st[s].just_done;
            const int saved = st[s].just_saved;
            if (done || saved >= 0) {
                st[s].just_done = 0;
                st[s].just_saved = -1;
                // one save: at the statistics clamp's save when the member has
                // one (its advance may stop earlier, at a writer's save), else
                // at the end of the advance
                const bool clamp = mp[s].time_interval > 0;
                const int k = nsaves <= 1 ? ((clamp ? (saved == 0 && st[s].status == 0) : done) ? 0 : -1)
                                          : (st[s].status == 0 ? saved : -1);
                const int g = st[s].group;
                if (k >= 0 && k < nsaves && g >= 0 && g * nsaves + k < nacc) a = g * nsaves + k;
            }
            acc_of[i] = a;
        }
        __syncthreads();
        if (threadIdx.x < 32) {
            const int lane = threadIdx.x;
            int m = m_shared;
            for (int b = 0; b < len; b += 32) {
                const int a = b + lane < len ? acc_of[b + lane] : -1;
                unsigned mask = __ballot_sync(0xffffffffu, a >= 0);
                while (mask) {
                    const int l = __ffs(mask) - 1;
                    mask &= mask - 1;
                    const int al = __shfl_sync(0xffffffffu, a, l);
                    if (lane == 0 && accs[al].mean) {
                        accs[al].count += 1;
                        list[m++] = make_int4(base0 + b + l, al, (int)accs[al].count, 0);
                    }
                }
            }
            if (lane == 0) m_shared = m;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) *nlist = m_shared;
}

template <class R>
__global__ void batch_stats_kernel(const BatchMember* members, const StepState* st, const GroupAcc* groups,
                                   int ngroups, long long total_cells, const int4* list, const int* nlist) {
    const int m = *nlist;
    if (m == 0) return;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total_cells;
         i += (long long)gridDim.x * blockDim.x) {
        int g = 0;
        long long c = i;
        while (g < ngroups && c >= groups[g].cells) {
            c -= groups[g].cells;
            ++g;
        }
        if (g >= ngroups) return;
        double mean = groups[g].mean[c], m2 = groups[g].m2[c];
        bool touched = false;
        for (int k = 0; k < m; ++k) {
            if (list[k].y != g) continue;
            const int s = list[k].x;
            const R* u = reinterpret_cast<const R*>(st[s].parity ? members[s].v : members[s].u);
            const double x = (double)u[c];
            const double n = (double)list[k].z;
            const double delta = x - mean;
            mean = mean + delta / n;
            m2 = m2 + delta * (x - mean);
            touched = true;
        }
        if (touched) {
            groups[g].mean[c] = mean;
            groups[g].m2[c] = m2;
        }
    }
}

__global__ void batch_count_kernel(const StepState* st, const MemberParam* mp, int M, int* running) {
    __shared__ int c;
    if (threadIdx.x == 0) c = 0;
    __syncthreads();
    for (int s = threadIdx.x; s < M; s += blockDim.x)
        if (mp[s].active && !st[s].done) atomicAdd(&c, 1);
    __syncthreads();
    if (threadIdx.x == 0) *running = c;
}

size_t round256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace

struct gbfv_batch {
    GbfvPlan scheme;  // names, variant, dim of the members (grid fields unused)
    gbfv_desc desc;
    std::string names[5];
    int max_members = 0;
    int dim = 0;
    // pool
    char* pool = nullptr;
    size_t capacity = 0;
    std::map<size_t, size_t> free_blocks;  // offset -> size
    // members
    struct Host {
        bool active = false;
        size_t off = 0, bytes = 0;
        BatchMember m;
        MemberParam p;
        int group = -1;
        bool own_end = false;  // end time and save clamp set by gbfv_batch_set_member_end
    };
    std::vector<Host> members;
    BatchMember* d_members = nullptr;
    MemberParam* d_params = nullptr;
    StepState* d_states = nullptr;
    StepState* h_states = nullptr;  // pinned
    // tiles
    int4* d_tiles = nullptr;
    int* d_ntiles = nullptr;
    size_t tile_cap = 0;
    bool tiles_dirty = true;
    // statistics
    // accumulators: index group * stats_saves + save
    std::vector<GroupAcc> groups;
    std::vector<int> group_dims;  // nvar*total per accumulator
    GroupAcc* d_groups = nullptr;
    int stats_saves = 1;
    int4* d_list = nullptr;
    int* d_nlist = nullptr;
    long long stats_cells = 0;
    // running count
    int* d_running = nullptr;
    int* h_running = nullptr;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t step_graph = nullptr;
    int graph_chunk = 0;
    long long launches = 0;
    // stage kernel configuration: the candidate in use, whether the
    // autotuner has settled it (or the caller pinned it), and the members'
    // tensor maps for its halo box (3 per slot: u, v, l)
    int cand = 0;
    bool tuned = false;
    bool pinned = false;
    std::vector<CUtensorMap> h_maps;
    CUtensorMap* d_maps = nullptr;
    StepState* d_tune_states = nullptr;
    std::vector<double> tune_ms;
};

namespace {

int bfail(int code, const std::string& m) { return gbfv_internal_fail(code, m.c_str()); }

#define BCUDA(x)                                                                          \
    do {                                                                                  \
        cudaError_t e_ = (x);                                                             \
        if (e_ != cudaSuccess) return bfail(GBFV_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
    } while (0)

const StageCandidate& current(const gbfv_batch* b) {
    int n = 0;
    const GbfvPlan& p = b->scheme;
    return candidates(p.var, p.eq, p.fl, p.rc, b->dim, &n)[b->cand];
}

int tile_shape(const gbfv_batch* b, int k) { return current(b).tile[k]; }

// Host side: the tensor maps of member `slot` for the current candidate's
// halo box; the member keeps plain loads when they cannot be encoded.
void encode_member_maps(gbfv_batch* b, int slot) {
    auto& h = b->members[slot];
    const StageCandidate& c = current(b);
    h.m.tma = 0;
    if (!h.active || !c.tma) return;
    void* bufs[3] = {h.m.u, h.m.v, h.m.l};
    for (int k = 0; k < 3; ++k)
        if (!gbfv_encode_state_map(&b->h_maps[3 * slot + k], bufs[k], h.m.G, b->scheme.nvar, b->scheme.elem,
                                   c.halo[0], c.halo[1], c.halo[2]))
            return;
    h.m.tma = 1;
}

int upload_maps(gbfv_batch* b, int first, int count) {
    BCUDA(cudaMemcpyAsync(b->d_maps + 3 * first, &b->h_maps[3 * first], (size_t)3 * count * sizeof(CUtensorMap),
                          cudaMemcpyHostToDevice, b->stream));
    return GBFV_OK;
}

int rebuild_tiles(gbfv_batch* b) {
    std::vector<int4> tiles;
    const int tx = tile_shape(b, 0), ty = tile_shape(b, 1), tz = tile_shape(b, 2);
    for (size_t s = 0; s < b->members.size(); ++s) {
        const auto& h = b->members[s];
        if (!h.active) continue;
        const StepState& S = b->h_states[s];
        if (S.done && (S.t >= S.end_time || S.status != 0)) continue;  // finished or stopped by a failure
        for (int z = 0; z < h.m.G.n[2]; z += tz)
            for (int y = 0; y < h.m.G.n[1]; y += ty)
                for (int x = 0; x < h.m.G.n[0]; x += tx) tiles.push_back(make_int4((int)s, x, y, z));
    }
    if (tiles.size() > b->tile_cap) {
        if (b->d_tiles) cudaFree(b->d_tiles);
        b->d_tiles = nullptr;
        const size_t cap = std::max<size_t>(tiles.size() * 3 / 2, 1024);
        BCUDA(cudaMalloc(&b->d_tiles, cap * sizeof(int4)));
        b->tile_cap = cap;
        if (b->step_graph) {
            cudaGraphExecDestroy(b->step_graph);
            b->step_graph = nullptr;
        }
    }
    const int n = (int)tiles.size();
    if (n) BCUDA(cudaMemcpyAsync(b->d_tiles, tiles.data(), tiles.size() * sizeof(int4), cudaMemcpyHostToDevice, b->stream));
    BCUDA(cudaMemcpyAsync(b->d_ntiles, &n, sizeof(int), cudaMemcpyHostToDevice, b->stream));
    BCUDA(cudaStreamSynchronize(b->stream));
    b->tiles_dirty = false;
    return GBFV_OK;
}

int upload_members(gbfv_batch* b) {
    const int M = b->max_members;
    std::vector<BatchMember> m(M);
    std::vector<MemberParam> p(M);
    for (int s = 0; s < M; ++s) {
        m[s] = b->members[s].m;
        p[s] = b->members[s].p;
    }
    BCUDA(cudaMemcpyAsync(b->d_members, m.data(), M * sizeof(BatchMember), cudaMemcpyHostToDevice, b->stream));
    BCUDA(cudaMemcpyAsync(b->d_params, p.data(), M * sizeof(MemberParam), cudaMemcpyHostToDevice, b->stream));
    BCUDA(cudaStreamSynchronize(b->stream));
    return GBFV_OK;
}

// One ensemble time step (the body of the captured graph).
int enqueue_batch_step(gbfv_batch* b) {
    const GbfvPlan& p = b->scheme;
    const BatchLauncher launch = current(b).batch;
    if (!launch) return bfail(GBFV_ERR_UNSUPPORTED, "no ensemble kernel for this scheme and precision");
    BatchArgs a;
    a.members = b->d_members;
    a.states = b->d_states;
    a.tiles = b->d_tiles;
    a.ntiles = b->d_ntiles;
    a.maps = b->d_maps;
    a.gamma = p.gamma;
    a.gamma_f = (float)p.gamma;
    a.periodic = p.periodic;
    const int M = b->max_members;
    const unsigned mb = (unsigned)((M + 127) / 128);
    cudaStream_t q = b->stream;
    a.mode = MODE_L;
    int r = launch(a, 0, q);
    if (r) return bfail(GBFV_ERR_CUDA, std::string("batch stage: ") + cudaGetErrorString((cudaError_t)r));
    batch_dt_kernel<<<mb, 128, 0, q>>>(b->d_states, b->d_params, M, p.cfl);
    if (p.in == 2) {
        a.mode = MODE_RK3_S1;
        r = launch(a, 0, q);
        if (!r) {
            a.mode = MODE_RK3_S2;
            r = launch(a, 0, q);
        }
    } else {
        a.mode = MODE_RK2_S1;
        r = launch(a, 0, q);
    }
    if (r) return bfail(GBFV_ERR_CUDA, std::string("batch stage: ") + cudaGetErrorString((cudaError_t)r));
    batch_finish_kernel<<<mb, 128, 0, q>>>(b->d_states, b->d_params, M, p.in == 1 ? 1 : 0);
    if (!b->groups.empty()) {
        batch_assign_kernel<<<1, kAssignThreads, 0, q>>>(b->d_states, b->d_params, M, b->d_groups,
                                                          (int)b->groups.size(), b->stats_saves, b->d_list,
                                                          b->d_nlist);
        const long long cells = b->stats_cells;
        unsigned nb = (unsigned)std::min<long long>((cells + 255) / 256, 152 * 8);
        if (b->scheme.elem == 8)
            batch_stats_kernel<double><<<nb, 256, 0, q>>>(b->d_members, b->d_states, b->d_groups,
                                                          (int)b->groups.size(), cells, b->d_list, b->d_nlist);
        else
            batch_stats_kernel<float><<<nb, 256, 0, q>>>(b->d_members, b->d_states, b->d_groups,
                                                         (int)b->groups.size(), cells, b->d_list, b->d_nlist);
    }
    BCUDA(cudaGetLastError());
    b->launches += (p.in == 2 ? 3 : 2) + 2 + (b->groups.empty() ? 0 : 2);
    return GBFV_OK;
}

// Makes candidate idx current: members' tensor maps re-encoded for its halo
// box, tile list rebuilt for its tile shape, the step graph dropped.
int set_candidate(gbfv_batch* b, int idx) {
    int n = 0;
    const GbfvPlan& p = b->scheme;
    candidates(p.var, p.eq, p.fl, p.rc, b->dim, &n);
    if (idx < 0 || idx >= n) return bfail(GBFV_ERR_ARGUMENT, "no such stage kernel candidate");
    if (idx == b->cand) return GBFV_OK;
    BCUDA(cudaStreamSynchronize(b->stream));
    b->cand = idx;
    for (int s = 0; s < b->max_members; ++s) encode_member_maps(b, s);
    int r = upload_maps(b, 0, b->max_members);
    if (!r) r = upload_members(b);
    if (r) return r;
    b->tiles_dirty = true;
    if (b->step_graph) {
        cudaGraphExecDestroy(b->step_graph);
        b->step_graph = nullptr;
    }
    return GBFV_OK;
}

// Interior cells of the members that still run (the tuning workload).
long long running_cells(const gbfv_batch* b) {
    long long c = 0;
    for (int s = 0; s < b->max_members; ++s) {
        const auto& h = b->members[s];
        if (!h.active || b->h_states[s].done) continue;
        c += (long long)h.m.G.n[0] * h.m.G.n[1] * h.m.G.n[2];
    }
    return c;
}

// The ensemble autotuner: with the step states of the current advance on the
// device (after the begin kernel), times the stage launches of every
// candidate over the running members and keeps the fastest: MODE_L (out =
// each member's L buffer) and, for SSP-RK3, the first combination stage
// (out = each member's V buffer, which every step rewrites before reading),
// scored as one step's L + 2 x stage-1 launches; wave speeds and step
// updates go into a copy of the step states, so the run is unaffected. The
// choice is cached per scheme for the process; ensembles below 2^22 running
// cells keep their current candidate and are tuned at a later advance (small
// ensembles are launch-latency bound and time every candidate alike).
int tune_batch(gbfv_batch* b, bool force) {
    const GbfvPlan& p = b->scheme;
    int n = 0;
    candidates(p.var, p.eq, p.fl, p.rc, b->dim, &n);
    b->tune_ms.assign(n, -1.0);
    if (n <= 1 || !gbfv_autotune_enabled()) {
        b->tuned = true;
        return set_candidate(b, 0);
    }
    char key[128];
    snprintf(key, sizeof key, "batch:%d:%d:%d:%d:%d:%d", p.var, p.eq, p.fl, p.rc, p.in, b->dim);
    int best = 0;
    if (!force && gbfv_tune_cache_get(key, &best)) {
        b->tuned = true;
        return set_candidate(b, best);
    }
    if (!force && running_cells(b) < (1LL << 22)) return GBFV_OK;
    const int M = b->max_members;
    if (!b->d_tune_states) BCUDA(cudaMalloc(&b->d_tune_states, M * sizeof(StepState)));
    cudaEvent_t e0, e1;
    BCUDA(cudaEventCreate(&e0));
    BCUDA(cudaEventCreate(&e1));
    double best_ms = 0;
    int err = GBFV_OK;
    const int kTimed = 2;
    for (int i = 0; i < n && !err; ++i) {
        err = set_candidate(b, i);
        if (!err) err = rebuild_tiles(b);
        if (err) break;
        BatchArgs a;
        a.members = b->d_members;
        a.states = b->d_tune_states;
        a.tiles = b->d_tiles;
        a.ntiles = b->d_ntiles;
        a.maps = b->d_maps;
        a.gamma = p.gamma;
        a.gamma_f = (float)p.gamma;
        a.periodic = p.periodic;
        a.mode = MODE_L;
        const BatchLauncher launch = current(b).batch;
        cudaError_t e = cudaMemcpyAsync(b->d_tune_states, b->d_states, M * sizeof(StepState),
                                        cudaMemcpyDeviceToDevice, b->stream);
        int r = e == cudaSuccess ? 0 : (int)e;
        const int nmodes = p.in == 2 ? 2 : 1;
        double step_ms = 0;
        for (int m = 0; m < nmodes && !r; ++m) {
            a.mode = m == 0 ? MODE_L : MODE_RK3_S1;
            r = launch(a, 0, b->stream);  // warm-up
            if (!r) r = (int)cudaEventRecord(e0, b->stream);
            for (int k = 0; k < kTimed && !r; ++k) r = launch(a, 0, b->stream);
            if (!r) r = (int)cudaEventRecord(e1, b->stream);
            if (!r) r = (int)cudaEventSynchronize(e1);
            float ms = 0;
            if (!r) r = (int)cudaEventElapsedTime(&ms, e0, e1);
            step_ms += (m == 0 ? 1.0 : 2.0) * ms / kTimed;
            b->launches += 1 + kTimed;
        }
        if (r) {
            err = bfail(GBFV_ERR_CUDA, std::string("ensemble autotuning launch: ") + cudaGetErrorString((cudaError_t)r));
            break;
        }
        // per stage launch of one step
        b->tune_ms[i] = step_ms / (nmodes == 2 ? 3.0 : 1.0);
        if (i == 0 || b->tune_ms[i] < best_ms) {
            best_ms = b->tune_ms[i];
            best = i;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (err) return err;
    gbfv_tune_cache_put(key, best);
    b->tuned = true;
    err = set_candidate(b, best);
    if (!err) err = rebuild_tiles(b);
    return err;
}

}  // namespace

extern "C" {

int gbfv_batch_create(const gbfv_desc* scheme, long long pool_bytes, int max_members, gbfv_batch** out) {
    if (!scheme || !out || pool_bytes <= 0 || max_members <= 0)
        return bfail(GBFV_ERR_ARGUMENT, "gbfv_batch_create: bad arguments");
    *out = nullptr;
    gbfv_batch* b = new gbfv_batch();
    b->desc = *scheme;
    const char* src[5] = {scheme->equation, scheme->flux, scheme->reconstruction, scheme->integrator, scheme->boundary};
    for (int k = 0; k < 5; ++k) b->names[k] = src[k] ? src[k] : "";
    b->desc.equation = b->names[0].c_str();
    b->desc.flux = b->names[1].c_str();
    b->desc.reconstruction = b->names[2].c_str();
    b->desc.integrator = b->names[3].c_str();
    b->desc.boundary = b->names[4].c_str();
    int r = gbfv_internal_plan(&b->desc, &b->scheme);
    if (r) {
        delete b;
        return r;
    }
    if (b->scheme.in == 0) {
        delete b;
        return bfail(GBFV_ERR_UNSUPPORTED, "gbfv_batch_create: the ensemble engine runs rungekutta2 and rungekutta3");
    }
    b->dim = b->scheme.G.dim;
    b->max_members = max_members;
    b->members.resize(max_members);
    for (auto& h : b->members) {
        std::memset(&h.m, 0, sizeof h.m);
        std::memset(&h.p, 0, sizeof h.p);
    }
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&b->pool, (size_t)pool_bytes);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_members, max_members * sizeof(BatchMember));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_params, max_members * sizeof(MemberParam));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_states, max_members * sizeof(StepState));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_maps, (size_t)3 * max_members * sizeof(CUtensorMap));
    if (e == cudaSuccess) e = cudaMallocHost(&b->h_states, max_members * sizeof(StepState));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_ntiles, sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_list, max_members * sizeof(int4));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_nlist, sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_running, sizeof(int));
    if (e == cudaSuccess) e = cudaMallocHost(&b->h_running, sizeof(int));
    if (e == cudaSuccess) e = cudaMemsetAsync(b->d_nlist, 0, sizeof(int), b->stream);
    if (e == cudaSuccess) {
        std::memset(b->h_states, 0, max_members * sizeof(StepState));
        for (int s = 0; s < max_members; ++s) {
            b->h_states[s].done = 1;
            b->h_states[s].group = -1;
            b->h_states[s].number_saved = 1;
        }
        e = cudaMemcpyAsync(b->d_states, b->h_states, max_members * sizeof(StepState), cudaMemcpyHostToDevice, b->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) {
        const int code = e == cudaErrorMemoryAllocation ? GBFV_ERR_MEMORY : GBFV_ERR_CUDA;
        gbfv_batch_destroy(b);
        return bfail(code, std::string("gbfv_batch_create: ") + cudaGetErrorString(e));
    }
    b->capacity = (size_t)pool_bytes;
    b->free_blocks[0] = b->capacity;
    b->h_maps.resize((size_t)3 * max_members);
    std::memset(b->h_maps.data(), 0, b->h_maps.size() * sizeof(CUtensorMap));
    int rr = upload_maps(b, 0, max_members);
    if (!rr) rr = upload_members(b);
    if (rr) {
        gbfv_batch_destroy(b);
        return rr;
    }
    *out = b;
    return GBFV_OK;
}

int gbfv_batch_destroy(gbfv_batch* b) {
    if (!b) return GBFV_OK;
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->step_graph) cudaGraphExecDestroy(b->step_graph);
    for (auto& g : b->groups) {
        cudaFree(g.mean);
        cudaFree(g.m2);
    }
    cudaFree(b->d_groups);
    cudaFree(b->pool);
    cudaFree(b->d_members);
    cudaFree(b->d_params);
    cudaFree(b->d_states);
    cudaFree(b->d_maps);
    cudaFree(b->d_tune_states);
    cudaFree(b->d_tiles);
    cudaFree(b->d_ntiles);
    cudaFree(b->d_list);
    cudaFree(b->d_nlist);
    cudaFree(b->d_running);
    if (b->h_states) cudaFreeHost(b->h_states);
    if (b->h_running) cudaFreeHost(b->h_running);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return GBFV_OK;
}

// Bytes a member of this grid occupies in the pool (three padded state arrays).
long long gbfv_batch_member_bytes(const gbfv_batch* b, const int n[3]) {
    if (!b || !n) return bfail(GBFV_ERR_ARGUMENT, "null argument");
    gbfv_desc d = b->desc;
    for (int k = 0; k < 3; ++k) d.n[k] = n[k];
    GbfvPlan p;
    int r = gbfv_internal_plan(&d, &p);
    if (r) return r;
    return (long long)(3 * round256((size_t)p.nvar * p.G.total * p.elem));
}

int gbfv_batch_add(gbfv_batch* b, const int n[3], const double lower[3], const double upper[3],
                   const double* prim_host, int group, int* slot_out) {
    if (!b || !n || !lower || !upper || !prim_host || !slot_out) return bfail(GBFV_ERR_ARGUMENT, "null argument");
    gbfv_desc d = b->desc;
    for (int k = 0; k < 3; ++k) {
        d.n[k] = n[k];
        d.lower[k] = lower[k];
        d.upper[k] = upper[k];
    }
    GbfvPlan p;
    int r = gbfv_internal_plan(&d, &p);
    if (r) return r;
    if (p.G.dim != b->dim) return bfail(GBFV_ERR_UNSUPPORTED, "all members of an ensemble share one dimension");
    int slot = -1;
    for (int s = 0; s < b->max_members; ++s)
        if (!b->members[s].active) {
            slot = s;
            break;
        }
    if (slot < 0) return bfail(GBFV_ERR_MEMORY, "gbfv_batch_add: every member slot is in use");
    const size_t arr = round256((size_t)p.nvar * p.G.total * p.elem);
    const size_t need = 3 * arr;
    size_t off = (size_t)-1;
    for (auto it = b->free_blocks.begin(); it != b->free_blocks.end(); ++it)
        if (it->second >= need) {
            off = it->first;
            const size_t rest = it->second - need;
            b->free_blocks.erase(it);
            if (rest) b->free_blocks[off + need] = rest;
            break;
        }
    if (off == (size_t)-1) return bfail(GBFV_ERR_MEMORY, "gbfv_batch_add: the ensemble pool has no room for this member");
    if (group >= 0) {
        // the accumulators of this group, one per statistics save
        const int S = b->stats_saves;
        while ((int)b->groups.size() < (group + 1) * S) {
            GroupAcc g;
            std::memset(&g, 0, sizeof g);
            b->groups.push_back(g);
            b->group_dims.push_back(0);
        }
        const long long cells = (long long)p.nvar * p.G.total;
        if (b->groups[group * S].mean && b->groups[group * S].cells != cells) {
            b->free_blocks[off] = need;
            return bfail(GBFV_ERR_ARGUMENT, "members of one statistics group must share their grid");
        }
        if (!b->groups[group * S].mean) {
            for (int k = 0; k < S; ++k) {
                GroupAcc& g = b->groups[group * S + k];
                BCUDA(cudaMalloc(&g.mean, cells * sizeof(double)));
                BCUDA(cudaMalloc(&g.m2, cells * sizeof(double)));
                BCUDA(cudaMemsetAsync(g.mean, 0, cells * sizeof(double), b->stream));
                BCUDA(cudaMemsetAsync(g.m2, 0, cells * sizeof(double), b->stream));
                g.cells = cells;
                g.count = 0;
            }
            if (b->d_groups) cudaFree(b->d_groups);
            b->d_groups = nullptr;
            BCUDA(cudaMalloc(&b->d_groups, b->groups.size() * sizeof(GroupAcc)));
            b->stats_cells = 0;
            for (auto& x : b->groups) b->stats_cells += x.cells;
            if (b->step_graph) {
                cudaGraphExecDestroy(b->step_graph);
                b->step_graph = nullptr;
            }
        }
        BCUDA(cudaMemcpyAsync(b->d_groups, b->groups.data(), b->groups.size() * sizeof(GroupAcc),
                              cudaMemcpyHostToDevice, b->stream));
    }
    auto& h = b->members[slot];
    h.active = true;
    h.off = off;
    h.bytes = need;
    h.group = group;
    h.m.u = b->pool + off;
    h.m.v = b->pool + off + arr;
    h.m.l = b->pool + off + 2 * arr;
    h.m.G = p.G;
    for (int k = 0; k < 3; ++k) h.p.cell_lengths[k] = p.cell_lengths[k];
    h.p.time_interval = 0;
    h.p.time_interval2 = 0;
    h.p.end_time = std::numeric_limits<double>::infinity();
    h.own_end = false;
    h.p.dim = p.G.dim;
    h.p.active = 1;

    // initial data: primitive -> conserved on the host (gbfv_set_primitive's
    // conversion), upload, ghost fill on the device
    {
        std::vector<double> cons((size_t)p.nvar * p.G.total, 0.0);
        gbfv_internal_prim_to_cons(p, prim_host, cons.data());
        r = gbfv_internal_load_state(p, cons.data(), h.m.u, b->stream);
        if (r) {
            h.active = false;
            b->free_blocks[off] = need;
            return r;
        }
    }
    StepState z;
    std::memset(&z, 0, sizeof z);
    z.number_saved = 1;
    z.number_saved2 = 1;
    z.done = 1;
    z.group = group;
    b->h_states[slot] = z;
    BCUDA(cudaMemcpyAsync(b->d_states + slot, &b->h_states[slot], sizeof(StepState), cudaMemcpyHostToDevice, b->stream));
    encode_member_maps(b, slot);
    r = upload_maps(b, slot, 1);
    if (!r) r = upload_members(b);
    if (r) return r;
    b->tiles_dirty = true;
    *slot_out = slot;
    return GBFV_OK;
}

int gbfv_batch_remove(gbfv_batch* b, int slot) {
    if (!b || slot < 0 || slot >= b->max_members || !b->members[slot].active)
        return bfail(GBFV_ERR_ARGUMENT, "gbfv_batch_remove: bad slot");
    BCUDA(cudaStreamSynchronize(b->stream));
    auto& h = b->members[slot];
    // return the block and merge neighbours
    size_t off = h.off, size = h.bytes;
    auto next = b->free_blocks.lower_bound(off);
    if (next != b->free_blocks.end() && next->first == off + size) {
        size += next->second;
        b->free_blocks.erase(next);
    }
    auto prev = b->free_blocks.lower_bound(off);
    if (prev != b->free_blocks.begin()) {
        --prev;
        if (prev->first + prev->second == off) {
            off = prev->first;
            size += prev->second;
            b->free_blocks.erase(prev);
        }
    }
    b->free_blocks[off] = size;
    h.active = false;
    std::memset(&h.m, 0, sizeof h.m);
    std::memset(&h.p, 0, sizeof h.p);
    int r = upload_members(b);
    if (r) return r;
    b->tiles_dirty = true;
    return GBFV_OK;
}

int gbfv_batch_free_bytes(const gbfv_batch* b, long long* free_total, long long* largest) {
    if (!b) return bfail(GBFV_ERR_ARGUMENT, "null batch");
    long long t = 0, l = 0;
    for (auto& kv : b->free_blocks) {
        t += (long long)kv.second;
        l = std::max(l, (long long)kv.second);
    }
    if (free_total) *free_total = t;
    if (largest) *largest = l;
    return GBFV_OK;
}

int gbfv_batch_advance(gbfv_batch* b, double end_time, int number_of_saves, int max_steps) {
    if (!b) return bfail(GBFV_ERR_ARGUMENT, "null batch");
    const int M = b->max_members;
    // save-time clamp per member (FixedIntervalStatistics / FixedIntervalWriter)
    for (int s = 0; s < M; ++s)
        if (b->members[s].active && !b->members[s].own_end)
            b->members[s].p.time_interval = number_of_saves > 0 ? end_time / number_of_saves : 0;
    int r = upload_members(b);
    if (r) return r;
    const unsigned mb = (unsigned)((M + 127) / 128);
    batch_begin_kernel<<<mb, 128, 0, b->stream>>>(b->d_states, b->d_params, M, end_time, max_steps);
    BCUDA(cudaGetLastError());
    BCUDA(cudaMemcpyAsync(b->h_states, b->d_states, M * sizeof(StepState), cudaMemcpyDeviceToHost, b->stream));
    BCUDA(cudaStreamSynchronize(b->stream));
    if (!b->tuned && !b->pinned) {
        r = tune_batch(b, false);
        if (r) return r;
    }
    b->tiles_dirty = true;
    r = rebuild_tiles(b);
    if (r) return r;
    // first step launched directly (initialises the launchers), the rest from a graph
    r = enqueue_batch_step(b);
    if (r) return r;
    if (!b->step_graph) {
        cudaGraph_t g = nullptr;
        BCUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        const long long before = b->launches;
        r = enqueue_batch_step(b);
        cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
        b->launches = before;
        if (r) return r;
        if (ce != cudaSuccess) return bfail(GBFV_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
        ce = cudaGraphInstantiate(&b->step_graph, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) return bfail(GBFV_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ce));
    }
    const long long per_step = (b->scheme.in == 2 ? 3 : 2) + 2 + (b->groups.empty() ? 0 : 2);
    int chunk = 4;
    int last_running = -1;
    for (;;) {
        batch_count_kernel<<<1, 256, 0, b->stream>>>(b->d_states, b->d_params, M, b->d_running);
        BCUDA(cudaMemcpyAsync(b->h_running, b->d_running, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
        BCUDA(cudaStreamSynchronize(b->stream));
        const int running = *b->h_running;
        if (running == 0) break;
        if (last_running >= 0 && running < last_running) {
            // members finished: drop their tiles from the work list
            BCUDA(cudaMemcpyAsync(b->h_states, b->d_states, M * sizeof(StepState), cudaMemcpyDeviceToHost, b->stream));
            BCUDA(cudaStreamSynchronize(b->stream));
            r = rebuild_tiles(b);
            if (r) return r;
        }
        last_running = running;
        for (int i = 0; i < chunk; ++i) {
            BCUDA(cudaGraphLaunch(b->step_graph, b->stream));
            b->launches += per_step;
        }
        if (chunk < 64) chunk *= 2;
    }
    BCUDA(cudaMemcpyAsync(b->h_states, b->d_states, M * sizeof(StepState), cudaMemcpyDeviceToHost, b->stream));
    BCUDA(cudaMemcpyAsync(b->groups.data(), b->d_groups, b->groups.size() * sizeof(GroupAcc), cudaMemcpyDeviceToHost,
                          b->stream));
    BCUDA(cudaStreamSynchronize(b->stream));
    for (int s = 0; s < M; ++s)
        if (b->members[s].active && b->h_states[s].status == kStatusTmaTimeout) {
            char msg[256];
            snprintf(msg, sizeof msg, "member %d: a TMA halo copy did not complete within the time limit (step %d)",
                     s, b->h_states[s].failed_step);
            return bfail(GBFV_ERR_CUDA, msg);
        }
    for (int s = 0; s < M; ++s)
        if (b->members[s].active && b->h_states[s].status != 0) {
            char msg[256];
            snprintf(msg, sizeof msg, "member %d does not obey constraints at time %.17g (step %d)", s,
                     b->h_states[s].t, b->h_states[s].failed_step);
            return bfail(GBFV_ERR_CONSTRAINT, msg);
        }
    return GBFV_OK;
}

int gbfv_batch_set_member_end(gbfv_batch* b, int slot, double end_time, int number_of_saves) {
    if (!b || slot < 0 || slot >= b->max_members || !b->members[slot].active)
        return bfail(GBFV_ERR_ARGUMENT, "gbfv_batch_set_member_end: bad slot");
    if (!(end_time > 0) || number_of_saves < 0)
        return bfail(GBFV_ERR_ARGUMENT, "gbfv_batch_set_member_end: bad end time or number of saves");
    auto& h = b->members[slot];
    h.own_end = true;
    h.p.end_time = end_time;
    h.p.time_interval = number_of_saves > 0 ? end_time / number_of_saves : 0;
    return upload_members(b);
}

int gbfv_batch_set_member_write_interval(gbfv_batch* b, int slot, double interval) {
    if (!b || slot < 0 || slot >= b->max_members || !b->members[slot].active)
        return bfail(GBFV_ERR_ARGUMENT, "gbfv_batch_set_member_write_interval: bad slot");
    if (!(interval >= 0)) return bfail(GBFV_ERR_ARGUMENT, "gbfv_batch_set_member_write_interval: bad interval");
    b->members[slot].p.time_interval2 = interval;
    return upload_members(b);
}

int gbfv_batch_member_status(gbfv_batch* b, int slot, int* status, int* failed_step) {
    if (!b || slot < 0 || slot >= b->max_members || !b->members[slot].active)
        return bfail(GBFV_ERR_ARGUMENT, "bad slot");
    BCUDA(cudaMemcpyAsync(&b->h_states[slot], b->d_states + slot, sizeof(StepState), cudaMemcpyDeviceToHost, b->stream));
    BCUDA(cudaStreamSynchronize(b->stream));
    if (status) *status = b->h_states[slot].status;
    if (failed_step) *failed_step = b->h_states[slot].failed_step;
    return GBFV_OK;
}

int gbfv_batch_member_time(gbfv_batch* b, int slot, double* t, long long* steps) {
    if (!b || slot < 0 || slot >= b->max_members || !b->members[slot].active)
        return bfail(GBFV_ERR_ARGUMENT, "bad slot");
    BCUDA(cudaMemcpyAsync(&b->h_states[slot], b->d_states + slot, sizeof(StepState), cudaMemcpyDeviceToHost, b->stream));
    BCUDA(cudaStreamSynchronize(b->stream));
    if (t) *t = b->h_states[slot].t;
    if (steps) *steps = b->h_states[slot].steps;
    return GBFV_OK;
}

int gbfv_batch_member_state(gbfv_batch* b, int slot, double* host) {
    if (!b || !host || slot < 0 || slot >= b->max_members || !b->members[slot].active)
        return bfail(GBFV_ERR_ARGUMENT, "bad slot");
    BCUDA(cudaMemcpyAsync(&b->h_states[slot], b->d_states + slot, sizeof(StepState), cudaMemcpyDeviceToHost, b->stream));
    BCUDA(cudaStreamSynchronize(b->stream));
    const auto& h = b->members[slot];
    const void* src = b->h_states[slot].parity ? h.m.v : h.m.u;
    const size_t n = (size_t)b->scheme.nvar * h.m.G.total;
    if (b->scheme.elem == 8) {
        BCUDA(cudaMemcpy(host, src, n * 8, cudaMemcpyDeviceToHost));
    } else {
        std::vector<float> f(n);
        BCUDA(cudaMemcpy(f.data(), src, n * 4, cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < n; ++i) host[i] = (double)f[i];
    }
    return GBFV_OK;
}

static int stats_index(const gbfv_batch* b, int group, int save) {
    if (save < 0) save = b->stats_saves - 1;  // the last save (the end time)
    const int a = group * b->stats_saves + save;
    if (group < 0 || save >= b->stats_saves || a >= (int)b->groups.size() || !b->groups[a].mean) return -1;
    return a;
}

int gbfv_batch_stats_result(gbfv_batch* b, int group, double* mean_host, double* var_host, long long* count) {
    const int a = b ? stats_index(b, group, -1) : -1;
    if (a < 0) return bfail(GBFV_ERR_ARGUMENT, "unknown statistics group");
    BCUDA(cudaStreamSynchronize(b->stream));
    BCUDA(cudaMemcpy(b->groups.data(), b->d_groups, b->groups.size() * sizeof(GroupAcc), cudaMemcpyDeviceToHost));
    const GroupAcc& g = b->groups[a];
    if (count) *count = g.count;
    if (g.count == 0) return bfail(GBFV_ERR_ARGUMENT, "no member of this group has reached the end time");
    std::vector<double> m2(g.cells);
    if (mean_host) BCUDA(cudaMemcpy(mean_host, g.mean, g.cells * sizeof(double), cudaMemcpyDeviceToHost));
    if (var_host) {
        BCUDA(cudaMemcpy(m2.data(), g.m2, g.cells * sizeof(double), cudaMemcpyDeviceToHost));
        for (long long i = 0; i < g.cells; ++i) var_host[i] = m2[i] / (double)g.count;
    }
    return GBFV_OK;
}

int gbfv_batch_stats_export(gbfv_batch* b, int group, double* mean_host, double* m2_host, long long* count) {
    return gbfv_batch_stats_export_save(b, group, -1, mean_host, m2_host, count);
}

int gbfv_batch_stats_export_save(gbfv_batch* b, int group, int save, double* mean_host, double* m2_host,
                                 long long* count) {
    const int a = b ? stats_index(b, group, save) : -1;
    if (a < 0) return bfail(GBFV_ERR_ARGUMENT, "unknown statistics group or save");
    BCUDA(cudaStreamSynchronize(b->stream));
    BCUDA(cudaMemcpy(b->groups.data(), b->d_groups, b->groups.size() * sizeof(GroupAcc), cudaMemcpyDeviceToHost));
    const GroupAcc& g = b->groups[a];
    if (count) *count = g.count;
    if (mean_host) BCUDA(cudaMemcpy(mean_host, g.mean, g.cells * sizeof(double), cudaMemcpyDeviceToHost));
    if (m2_host) BCUDA(cudaMemcpy(m2_host, g.m2, g.cells * sizeof(double), cudaMemcpyDeviceToHost));
    return GBFV_OK;
}

int gbfv_batch_stats_reset(gbfv_batch* b) {
    if (!b) return bfail(GBFV_ERR_ARGUMENT, "null batch");
    BCUDA(cudaStreamSynchronize(b->stream));
    for (auto& g : b->groups) {
        if (!g.mean) continue;
        BCUDA(cudaMemset(g.mean, 0, g.cells * sizeof(double)));
        BCUDA(cudaMemset(g.m2, 0, g.cells * sizeof(double)));
        g.count = 0;
    }
    if (b->d_groups)
        BCUDA(cudaMemcpy(b->d_groups, b->groups.data(), b->groups.size() * sizeof(GroupAcc), cudaMemcpyHostToDevice));
    return GBFV_OK;
}

int gbfv_batch_finished(gbfv_batch* b, int* slots, int capacity, int* count) {
    if (!b || !count || (capacity > 0 && !slots)) return bfail(GBFV_ERR_ARGUMENT, "null argument");
    int c = 0;
    for (int s = 0; s < b->max_members; ++s) {
        if (!b->members[s].active) continue;
        const StepState& S = b->h_states[s];
        if (S.done && S.status == 0 && !(S.t < S.end_time)) {
            if (c < capacity) slots[c] = s;
            ++c;
        }
    }
    *count = c;
    return GBFV_OK;
}

int gbfv_batch_active(const gbfv_batch* b, int* count) {
    if (!b || !count) return bfail(GBFV_ERR_ARGUMENT, "null argument");
    int c = 0;
    for (int s = 0; s < b->max_members; ++s) c += b->members[s].active ? 1 : 0;
    *count = c;
    return GBFV_OK;
}

int gbfv_batch_launches(gbfv_batch* b, long long* launches) {
    if (!b || !launches) return bfail(GBFV_ERR_ARGUMENT, "null argument");
    *launches = b->launches;
    return GBFV_OK;
}

int gbfv_batch_set_statistics_saves(gbfv_batch* b, int saves) {
    if (!b || saves < 1) return bfail(GBFV_ERR_ARGUMENT, "statistics saves must be >= 1");
    if (!b->groups.empty()) return bfail(GBFV_ERR_UNSUPPORTED, "set the statistics saves before adding members");
    b->stats_saves = saves;
    return GBFV_OK;
}

int gbfv_batch_select_candidate(gbfv_batch* b, int idx) {
    if (!b) return bfail(GBFV_ERR_ARGUMENT, "null batch");
    if (idx < 0) {
        b->pinned = false;
        b->tuned = false;
        return GBFV_OK;
    }
    const int r = set_candidate(b, idx);
    if (r == GBFV_OK) b->pinned = true;
    return r;
}

int gbfv_batch_current_candidate(gbfv_batch* b, int* idx, int* member_tma) {
    if (!b || !idx) return bfail(GBFV_ERR_ARGUMENT, "null argument");
    *idx = b->cand;
    if (member_tma) {
        int c = 0;
        for (int s = 0; s < b->max_members; ++s) c += (b->members[s].active && b->members[s].m.tma) ? 1 : 0;
        *member_tma = c;
    }
    return GBFV_OK;
}

int gbfv_batch_autotune_result(gbfv_batch* b, double* ms, int capacity) {
    if (!b || (capacity > 0 && !ms)) return bfail(GBFV_ERR_ARGUMENT, "null argument");
    for (int i = 0; i < capacity; ++i) ms[i] = i < (int)b->tune_ms.size() ? b->tune_ms[i] : -1.0;
    return GBFV_OK;
}

int gbfv_batch_stream(gbfv_batch* b, void** stream) {
    if (!b || !stream) return bfail(GBFV_ERR_ARGUMENT, "null argument");
    *stream = (void*)b->stream;
    return GBFV_OK;
}

}  // extern "C"
