// gbfv_advance_noalloc: time stepping on a caller-owned device state without
// allocating any memory.
//
// Some callers cannot call cudaMalloc: code that runs inside a host
// application whose device memory is owned by a pool or arena it does not
// expose, plug-ins loaded into a process that forbids allocation after start-up,
// and hosts that record work into a pre-sized memory budget. gbfv_advance needs
// two state-sized scratch arrays and a step-state block that gbfv_create
// allocates; this entry point takes them from one file-scope device array of
// GBFV_NOALLOC_SCRATCH_BYTES instead. Every GPU that loads the library holds
// that array until the process exits.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>

#include "fv_registry.h"
#include "gbfv_internal.h"

using namespace gbfv;

// The scratch array: step state, then the stage-0 flux difference L, then the
// second state buffer V, each at a 256-byte boundary.
static __device__ __align__(256) unsigned char g_noalloc_scratch[GBFV_NOALLOC_SCRATCH_BYTES];

// Device address of g_noalloc_scratch per device, looked up at the first call
// on the device (host code may not take the address of a __device__ array
// directly: in host code the name is a host-side stand-in). The address
// belongs to the device's context: it is kept with that context's unique id
// and looked up again when the current context is another one (after a
// cudaDeviceReset, for instance). Calls from several host threads share the
// table under a mutex.
struct ScratchAddress {
    unsigned long long context_id = 0;
    void* ptr = nullptr;
};
static ScratchAddress g_scratch_address[256];
static std::mutex g_scratch_mutex;

typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);

// The unique id of the calling thread's current context (0: unknown).
static unsigned long long current_context_id() {
    static CtxGetCurrentFn get_current = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            return (CtxGetCurrentFn) nullptr;
        return reinterpret_cast<CtxGetCurrentFn>(p);
    }();
    static CtxGetIdFn get_id = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            return (CtxGetIdFn) nullptr;
        return reinterpret_cast<CtxGetIdFn>(p);
    }();
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS)
        return 0;
    return id;
}

static size_t round256(size_t b) { return (b + 255) & ~(size_t)255; }

extern "C" int gbfv_advance_noalloc(const gbfv_desc* desc, void* state_dev, double* t_inout,
                                    long long* steps_inout, double end_time, int number_of_saves,
                                    int max_steps, void* stream) {
    if (!desc || !state_dev || !t_inout || !steps_inout)
        return gbfv_internal_fail(GBFV_ERR_ARGUMENT, "gbfv_advance_noalloc: null argument");
    GbfvPlan p;
    int r = gbfv_internal_plan(desc, &p);
    if (r) return r;
    const size_t state_bytes = (size_t)p.nvar * (size_t)p.G.total * (size_t)p.elem;
    const size_t need = round256(sizeof(StepState)) + 2 * round256(state_bytes);
    if (need > (size_t)GBFV_NOALLOC_SCRATCH_BYTES) {
        char msg[256];
        snprintf(msg, sizeof msg,
                 "gbfv_advance_noalloc: grid needs %zu bytes of scratch, more than the built-in %u bytes "
                 "(two state arrays of %zu bytes plus the step state); use gbfv_create/gbfv_advance",
                 need, (unsigned)GBFV_NOALLOC_SCRATCH_BYTES, state_bytes);
        return gbfv_internal_fail(GBFV_ERR_UNSUPPORTED, msg);
    }
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess || device < 0 || device >= 256)
        return gbfv_internal_fail(GBFV_ERR_CUDA, "gbfv_advance_noalloc: no current CUDA device");
    // set-up, at the first call on a device (and again in a new context of
    // it), with that device current
    unsigned char* base = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_scratch_mutex);
        ScratchAddress& a = g_scratch_address[device];
        const unsigned long long id = current_context_id();
        if (!a.ptr || id == 0 || id != a.context_id) {
            void* ptr = nullptr;
            e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
            if (e != cudaSuccess || !ptr)
                return gbfv_internal_fail(GBFV_ERR_CUDA,
                                          (std::string("gbfv_advance_noalloc: cudaGetSymbolAddress: ") +
                                           cudaGetErrorString(e)).c_str());
            a.ptr = ptr;
            a.context_id = id;
        }
        base = static_cast<unsigned char*>(a.ptr);
    }
    StepState* st = reinterpret_cast<StepState*>(base);
    void* L = base + round256(sizeof(StepState));
    void* V = base + round256(sizeof(StepState)) + round256(state_bytes);
    cudaStream_t q = static_cast<cudaStream_t>(stream);

    // The array keeps the previous call's contents: the step state must start
    // from the caller's time. L and V are written in full before they are read.
    StepState h;
    std::memset(&h, 0, sizeof h);
    h.t = *t_inout;
    h.steps = *steps_inout;
    h.number_saved = 1;
    h.number_saved2 = 1;
    const double interval = number_of_saves > 0 ? end_time / number_of_saves : 0.0;
    if (number_of_saves > 0)
        for (int k = 0; k < (1 << 20) && h.t >= (double)h.number_saved * interval + 0.0; ++k) h.number_saved += 1;
    h.done = 1;
    e = cudaMemcpyAsync(st, &h, sizeof h, cudaMemcpyHostToDevice, q);
    if (e != cudaSuccess) return gbfv_internal_fail(GBFV_ERR_CUDA, cudaGetErrorString(e));

    StepParams P;
    P.cfl = p.cfl;
    for (int k = 0; k < 3; ++k) P.cell_lengths[k] = p.cell_lengths[k];
    P.end_time = end_time;
    P.time_interval = interval;
    P.dim = p.G.dim;
    const long long limit = max_steps > 0 ? h.steps + max_steps : -1;
    r = gbfv_internal_begin(st, end_time, limit, q);
    if (r) return r;
    int chunk = 1;
    for (;;) {
        for (int i = 0; i < chunk; ++i) {
            r = gbfv_internal_step(p, state_dev, V, L, st, P, q);
            if (r) return r;
        }
        e = cudaMemcpyAsync(&h, st, sizeof h, cudaMemcpyDeviceToHost, q);
        if (e == cudaSuccess) e = cudaStreamSynchronize(q);
        if (e != cudaSuccess) return gbfv_internal_fail(GBFV_ERR_CUDA, cudaGetErrorString(e));
        if (h.done) break;
        if (chunk < 64) chunk *= 2;
    }
    *t_inout = h.t;
    *steps_inout = h.steps;
    if (h.status != 0) {
        char msg[256];
        snprintf(msg, sizeof msg,
                 "Simulation state does not obey constraints! At time %.17g, number of timesteps performed %d",
                 h.t, h.failed_step);
        return gbfv_internal_fail(GBFV_ERR_CONSTRAINT, msg);
    }
    return GBFV_OK;
}
