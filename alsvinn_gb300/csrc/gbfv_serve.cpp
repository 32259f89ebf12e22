// Continuous-batching request loop over two ensembles.
//
// Requests are solves of one of two kinds: 1D Burgers (godunov flux, WENO2,
// SSP-RK2, periodic on [0,1], u0 = sin(2 pi x) + 0.5 phase) or 2D
// Kelvin-Helmholtz (euler2, HLL3, WENO2, SSP-RK3, periodic on [0,1]^2, the
// seeded interface perturbation of generator sample `sample`). Each kind is an
// ensemble (gbfv_batch) driven by its own host thread on its own stream, so the
// two kinds' work overlaps on the GPU. A request is admitted once it has
// arrived and its grid fits into its ensemble's free memory (first fit in
// arrival order: a later, smaller request may pass one that does not fit
// yet); it then runs inside the ensemble's persistent stage launches next to
// whatever is already in flight, with its own dt, until its end time. Its
// final state is folded into the FP64 Welford statistics of its (kind, grid)
// group and it leaves the ensemble, freeing its slot and memory. Every request
// has its own end time (the ensemble stops each member at its own end). A
// request whose state breaks the constraint check stops alone: it is marked
// failed and leaves, while the others run on. The reference has no
// counterpart (alsuq runs a fixed sample list, alsuq/src/run/Runner.cpp:39-90).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "gbfv.h"

int gbfv_internal_fail(int code, const char* msg);

namespace {

using Clock = std::chrono::steady_clock;

struct Req {
    gbfv_request r;
    int id = -1;
    int state = 0;  // 0 queued, 1 running, 2 done, 3 failed
    int slot = -1;
    double admit_s = 0, finish_s = 0;
    long long steps = 0;
    std::vector<double> final_state;
    std::vector<double> initial;  // caller's primitive initial data (empty: the kind's family)
};

struct Kind {
    gbfv_batch* batch = nullptr;
    int dim = 1;
    std::map<std::pair<int, double>, int> group_of;  // (grid size, end time) -> statistics group
};

}  // namespace

struct gbfv_server {
    Kind kinds[2];
    std::vector<Req> reqs;
    std::mutex mu;
    Clock::time_point start;
    int precision = GBFV_FP32;
    int max_slots = 0;
    std::string error;
    int error_code = 0;
    long long completed = 0;
    long long failed = 0;
};

namespace {

double since(const Clock::time_point& t0) {
    return std::chrono::duration<double>(Clock::now() - t0).count();
}

int grid_of(const gbfv_request& r, int n3[3], double lo[3], double hi[3]) {
    lo[0] = lo[1] = lo[2] = 0.0;
    hi[0] = hi[1] = 1.0;
    hi[2] = r.kind == GBFV_REQUEST_BURGERS ? 1.0 : 0.0;
    n3[0] = r.n;
    n3[1] = r.kind == GBFV_REQUEST_BURGERS ? 1 : r.n;
    n3[2] = 1;
    return 0;
}

int initial_data(const Req& q, std::vector<double>& prim) {
    const gbfv_request& r = q.r;
    if (!q.initial.empty()) {
        prim = q.initial;
        return GBFV_OK;
    }
    int n3[3];
    double lo[3], hi[3];
    grid_of(r, n3, lo, hi);
    if (r.kind == GBFV_REQUEST_BURGERS) {
        prim.assign((size_t)r.n, 0.0);
        return gbfv_init_burgers_sine(n3, lo, hi, r.phase, prim.data());
    }
    double X[40];
    int rc = gbfv_uniform(40, r.sample, 0.0, 1.0, X);
    if (rc) return rc;
    prim.assign((size_t)4 * r.n * r.n, 0.0);
    return gbfv_init_kelvin_helmholtz(n3, lo, hi, X, prim.data());
}

// One ensemble's loop: admit, advance a chunk, retire; until every request of
// this kind is done.
void drive(gbfv_server* S, int kind, int steps_per_chunk) {
    Kind& K = S->kinds[kind];
    std::vector<int> finished(S->max_slots);
    std::vector<double> prim;
    for (;;) {
        // admission: arrived requests of this kind, in arrival order, first fit
        bool any_pending = false;
        double next_arrival = 1e300;
        {
            std::vector<int> order;
            {
                std::lock_guard<std::mutex> g(S->mu);
                for (auto& q : S->reqs) {
                    if (q.r.kind != kind) continue;
                    if (q.state == 0) order.push_back(q.id);
                }
            }
            std::sort(order.begin(), order.end(), [&](int a, int b) {
                return S->reqs[a].r.arrival < S->reqs[b].r.arrival || (S->reqs[a].r.arrival == S->reqs[b].r.arrival && a < b);
            });
            const double now = since(S->start);
            for (int id : order) {
                Req& q = S->reqs[id];
                if (q.r.arrival > now) {
                    any_pending = true;
                    next_arrival = std::min(next_arrival, q.r.arrival);
                    continue;
                }
                int n3[3];
                double lo[3], hi[3];
                grid_of(q.r, n3, lo, hi);
                const long long need = gbfv_batch_member_bytes(K.batch, n3);
                long long free_total = 0, largest = 0;
                gbfv_batch_free_bytes(K.batch, &free_total, &largest);
                int active = 0;
                gbfv_batch_active(K.batch, &active);
                if (need < 0 || need > largest || active >= S->max_slots) {
                    any_pending = true;  // waits for memory / a slot
                    continue;
                }
                if (initial_data(q, prim)) {
                    std::lock_guard<std::mutex> g(S->mu);
                    q.state = 3;
                    continue;
                }
                int group;
                {
                    std::lock_guard<std::mutex> g(S->mu);
                    const auto key = std::make_pair(q.r.n, q.r.end_time);
                    auto it = K.group_of.find(key);
                    if (it == K.group_of.end()) it = K.group_of.emplace(key, (int)K.group_of.size()).first;
                    group = it->second;
                }
                int slot = -1;
                int rc = gbfv_batch_add(K.batch, n3, lo, hi, prim.data(), group, &slot);
                // the request's own end time; one save clamp lands it exactly there
                if (rc == GBFV_OK) {
                    rc = gbfv_batch_set_member_end(K.batch, slot, q.r.end_time, 1);
                    if (rc) gbfv_batch_remove(K.batch, slot);
                }
                std::lock_guard<std::mutex> g(S->mu);
                if (rc == GBFV_ERR_MEMORY) {
                    any_pending = true;
                    continue;
                }
                if (rc) {
                    q.state = 3;
                    S->error = gbfv_last_error();
                    S->error_code = rc;
                    continue;
                }
                q.state = 1;
                q.slot = slot;
                q.admit_s = since(S->start);
            }
        }
        int active = 0;
        gbfv_batch_active(K.batch, &active);
        if (active == 0) {
            if (!any_pending) return;  // nothing queued, nothing running
            const double wait = next_arrival - since(S->start);
            if (wait > 0) std::this_thread::sleep_for(std::chrono::duration<double>(std::min(wait, 0.05)));
            continue;
        }
        // one chunk of steps for everything in flight
        double end_time = 0;
        {
            std::lock_guard<std::mutex> g(S->mu);
            for (auto& q : S->reqs)
                if (q.r.kind == kind && q.state == 1) end_time = std::max(end_time, q.r.end_time);
        }
        int rc = gbfv_batch_advance(K.batch, end_time, 0, steps_per_chunk);
        if (rc == GBFV_ERR_CONSTRAINT) {
            // members whose state broke the constraints stopped alone: those
            // requests fail and leave; the rest of the chunk ran as usual
            std::vector<Req*> running;
            {
                std::lock_guard<std::mutex> g(S->mu);
                for (auto& q : S->reqs)
                    if (q.r.kind == kind && q.state == 1) running.push_back(&q);
            }
            const double t_fail = since(S->start);
            for (Req* q : running) {
                int status = 0, failed_step = 0;
                if (gbfv_batch_member_status(K.batch, q->slot, &status, &failed_step) || status == 0) continue;
                long long steps = 0;
                gbfv_batch_member_time(K.batch, q->slot, nullptr, &steps);
                gbfv_batch_remove(K.batch, q->slot);
                std::lock_guard<std::mutex> g(S->mu);
                q->state = 3;
                q->finish_s = t_fail;
                q->steps = steps;
                S->failed += 1;
            }
            rc = GBFV_OK;
        }
        if (rc) {
            std::lock_guard<std::mutex> g(S->mu);
            S->error = gbfv_last_error();
            S->error_code = rc;
            for (auto& q : S->reqs)
                if (q.r.kind == kind && q.state == 1) q.state = 3;
            return;
        }
        int nf = 0;
        gbfv_batch_finished(K.batch, finished.data(), (int)finished.size(), &nf);
        const double t_done = since(S->start);
        for (int k = 0; k < nf; ++k) {
            const int slot = finished[k];
            Req* q = nullptr;
            {
                std::lock_guard<std::mutex> g(S->mu);
                for (auto& x : S->reqs)
                    if (x.r.kind == kind && x.state == 1 && x.slot == slot) q = &x;
            }
            if (!q) continue;
            double t = 0;
            long long steps = 0;
            gbfv_batch_member_time(K.batch, slot, &t, &steps);
            if (q->r.keep) {
                int n3[3];
                double lo[3], hi[3];
                grid_of(q->r, n3, lo, hi);
                const int nvar = kind == GBFV_REQUEST_BURGERS ? 1 : 4;
                const long long total = kind == GBFV_REQUEST_BURGERS ? (long long)(q->r.n + 4)
                                                                     : (long long)(q->r.n + 4) * (q->r.n + 4);
                q->final_state.assign((size_t)nvar * total, 0.0);
                gbfv_batch_member_state(K.batch, slot, q->final_state.data());
            }
            gbfv_batch_remove(K.batch, slot);
            std::lock_guard<std::mutex> g(S->mu);
            q->state = 2;
            q->finish_s = t_done;
            q->steps = steps;
            S->completed += 1;
        }
    }
}

}  // namespace

extern "C" {

int gbfv_server_create(long long budget_bytes, int precision, int max_slots, gbfv_server** out) {
    if (budget_bytes <= 0 || max_slots <= 0 || !out) return gbfv_internal_fail(GBFV_ERR_ARGUMENT, "bad arguments");
    *out = nullptr;
    gbfv_server* S = new gbfv_server();
    S->precision = precision;
    S->max_slots = max_slots;
    // Burgers members are small (<= 8196 cells): a 1/64 share of the budget
    // holds thousands of them; the rest goes to the 2D ensemble.
    const long long burgers_bytes = std::max<long long>(budget_bytes / 64, 16ll << 20);
    const long long kh_bytes = budget_bytes - burgers_bytes;
    gbfv_desc d;
    std::memset(&d, 0, sizeof d);
    d.equation = "burgers";
    d.flux = "godunov";
    d.reconstruction = "weno2";
    d.integrator = "rungekutta2";
    d.boundary = "periodic";
    d.n[0] = 8; d.n[1] = 1; d.n[2] = 1;
    d.upper[0] = d.upper[1] = d.upper[2] = 1.0;
    d.gamma = 1.4;
    d.cfl = 0.475;
    d.precision = precision;
    int rc = gbfv_batch_create(&d, burgers_bytes, max_slots, &S->kinds[0].batch);
    if (rc) {
        delete S;
        return rc;
    }
    d.equation = "euler2";
    d.flux = "hll3";
    d.integrator = "rungekutta3";
    d.n[1] = 8;
    d.cfl = 0.4;
    rc = gbfv_batch_create(&d, kh_bytes, max_slots, &S->kinds[1].batch);
    if (rc) {
        gbfv_batch_destroy(S->kinds[0].batch);
        delete S;
        return rc;
    }
    S->kinds[0].dim = 1;
    S->kinds[1].dim = 2;
    *out = S;
    return GBFV_OK;
}

int gbfv_server_destroy(gbfv_server* S) {
    if (!S) return GBFV_OK;
    for (auto& k : S->kinds)
        if (k.batch) gbfv_batch_destroy(k.batch);
    delete S;
    return GBFV_OK;
}

int gbfv_server_submit(gbfv_server* S, const gbfv_request* r, int* id) {
    if (!S || !r || !id) return gbfv_internal_fail(GBFV_ERR_ARGUMENT, "null argument");
    if (r->kind != GBFV_REQUEST_BURGERS && r->kind != GBFV_REQUEST_KELVIN_HELMHOLTZ)
        return gbfv_internal_fail(GBFV_ERR_ARGUMENT, "unknown request kind");
    if (r->n < 8 || !(r->end_time > 0)) return gbfv_internal_fail(GBFV_ERR_ARGUMENT, "bad request grid or end time");
    std::lock_guard<std::mutex> g(S->mu);
    Req q;
    q.r = *r;
    if (r->initial_primitive) {
        const size_t cells = r->kind == GBFV_REQUEST_BURGERS ? (size_t)r->n : (size_t)4 * r->n * r->n;
        q.initial.assign(r->initial_primitive, r->initial_primitive + cells);
    }
    q.r.initial_primitive = nullptr;
    q.id = (int)S->reqs.size();
    S->reqs.push_back(q);
    *id = q.id;
    return GBFV_OK;
}

int gbfv_server_run(gbfv_server* S, int steps_per_chunk) {
    if (!S) return gbfv_internal_fail(GBFV_ERR_ARGUMENT, "null server");
    if (steps_per_chunk <= 0) steps_per_chunk = 16;
    S->start = Clock::now();
    S->error.clear();
    S->error_code = 0;
    std::thread t0(drive, S, 0, steps_per_chunk);
    std::thread t1(drive, S, 1, steps_per_chunk);
    t0.join();
    t1.join();
    if (S->error_code) return gbfv_internal_fail(S->error_code, S->error.c_str());
    return GBFV_OK;
}

int gbfv_server_result(gbfv_server* S, int id, double* arrival_s, double* admit_s, double* finish_s,
                       long long* steps, int* status) {
    if (!S || id < 0 || id >= (int)S->reqs.size()) return gbfv_internal_fail(GBFV_ERR_ARGUMENT, "bad request id");
    const Req& q = S->reqs[id];
    if (arrival_s) *arrival_s = q.r.arrival;
    if (admit_s) *admit_s = q.admit_s;
    if (finish_s) *finish_s = q.finish_s;
    if (steps) *steps = q.steps;
    if (status) *status = q.state;
    return GBFV_OK;
}

int gbfv_server_final_state(gbfv_server* S, int id, double* state_host, long long capacity) {
    if (!S || id < 0 || id >= (int)S->reqs.size() || !state_host)
        return gbfv_internal_fail(GBFV_ERR_ARGUMENT, "bad request id");
    const Req& q = S->reqs[id];
    if (q.state != 2 || q.final_state.empty())
        return gbfv_internal_fail(GBFV_ERR_ARGUMENT, "request not done or its state was not kept");
    if ((long long)q.final_state.size() > capacity) return gbfv_internal_fail(GBFV_ERR_ARGUMENT, "buffer too small");
    std::memcpy(state_host, q.final_state.data(), q.final_state.size() * sizeof(double));
    return GBFV_OK;
}

int gbfv_server_stats_at(gbfv_server* S, int kind, int n, double end_time, double* mean_host, double* var_host,
                        long long* count) {
    if (!S || (kind != 0 && kind != 1)) return gbfv_internal_fail(GBFV_ERR_ARGUMENT, "bad kind");
    auto it = S->kinds[kind].group_of.find(std::make_pair(n, end_time));
    if (it == S->kinds[kind].group_of.end())
        return gbfv_internal_fail(GBFV_ERR_ARGUMENT, "no request of this grid and end time");
    return gbfv_batch_stats_result(S->kinds[kind].batch, it->second, mean_host, var_host, count);
}

int gbfv_server_stats(gbfv_server* S, int kind, int n, double* mean_host, double* var_host, long long* count) {
    if (!S || (kind != 0 && kind != 1)) return gbfv_internal_fail(GBFV_ERR_ARGUMENT, "bad kind");
    const std::pair<int, double>* key = nullptr;
    for (const auto& kv : S->kinds[kind].group_of) {
        if (kv.first.first != n) continue;
        if (key) return gbfv_internal_fail(GBFV_ERR_ARGUMENT, "requests of this grid have several end times: "
                                                              "use gbfv_server_stats_at");
        key = &kv.first;
    }
    if (!key) return gbfv_internal_fail(GBFV_ERR_ARGUMENT, "no request of this grid");
    return gbfv_server_stats_at(S, kind, n, key->second, mean_host, var_host, count);
}

int gbfv_server_launches(gbfv_server* S, long long* launches) {
    if (!S || !launches) return gbfv_internal_fail(GBFV_ERR_ARGUMENT, "null argument");
    long long a = 0, b = 0;
    gbfv_batch_launches(S->kinds[0].batch, &a);
    gbfv_batch_launches(S->kinds[1].batch, &b);
    *launches = a + b;
    return GBFV_OK;
}

}  // extern "C"
