// Streaming FP64 mean / variance on the device (Welford's update, Chan et al.'s
// pairwise merge). Stands in for alsuq's MeanVariance, which accumulates
// sum u and sum u^2 and forms sum/N and sum2/N - mean^2
// (alsuq/src/stats/MeanVariance.cpp:30-67, StatisticsHelper.cpp:35-79); the
// Welford form gives the same population variance without the cancellation.
#include <cuda_runtime.h>

#include <cstring>
#include <string>

#include "gbfv.h"

namespace {

}  // namespace

// Records the message for gbfv_last_error (defined with the solver API).
int gbfv_internal_fail(int code, const char* msg);

namespace {

int sfail(int code, const std::string& m) { return gbfv_internal_fail(code, m.c_str()); }

template <class T>
__global__ void welford_add(double* __restrict__ mean, double* __restrict__ m2, const T* __restrict__ x,
                            long long count, double n) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < count;
         i += (long long)gridDim.x * blockDim.x) {
        const double v = (double)x[i];
        const double mu = mean[i];
        const double delta = v - mu;
        const double mu2 = mu + delta / n;
        mean[i] = mu2;
        m2[i] = m2[i] + delta * (v - mu2);
    }
}

__global__ void welford_merge(double* __restrict__ mean, double* __restrict__ m2, const double* __restrict__ mb,
                              const double* __restrict__ m2b, long long count, double na, double nb) {
    const double n = na + nb;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < count;
         i += (long long)gridDim.x * blockDim.x) {
        const double delta = mb[i] - mean[i];
        mean[i] = mean[i] + delta * (nb / n);
        m2[i] = m2[i] + m2b[i] + delta * delta * (na * nb / n);
    }
}

__global__ void welford_finish(const double* __restrict__ m2, double* __restrict__ var, long long count, double n) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < count;
         i += (long long)gridDim.x * blockDim.x)
        var[i] = m2[i] / n;
}

unsigned grid_for(long long count) {
    long long b = (count + 255) / 256;
    if (b > 152 * 16) b = 152 * 16;
    return (unsigned)(b < 1 ? 1 : b);
}

}  // namespace

struct gbfv_stats {
    long long count = 0;
    long long n = 0;
    double* mean = nullptr;
    double* m2 = nullptr;
    double* scratch = nullptr;  // host-sample upload / variance output
    cudaStream_t stream = nullptr;
};

extern "C" {

int gbfv_stats_create(long long count, gbfv_stats** out) {
    if (count <= 0 || !out) return sfail(GBFV_ERR_ARGUMENT, "bad count");
    gbfv_stats* st = new gbfv_stats();
    st->count = count;
    cudaError_t e = cudaStreamCreateWithFlags(&st->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&st->mean, count * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&st->m2, count * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&st->scratch, count * sizeof(double));
    if (e == cudaSuccess) e = cudaMemsetAsync(st->mean, 0, count * sizeof(double), st->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(st->m2, 0, count * sizeof(double), st->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st->stream);
    if (e != cudaSuccess) {
        gbfv_stats_destroy(st);
        return sfail(GBFV_ERR_MEMORY, std::string("gbfv_stats_create: ") + cudaGetErrorString(e));
    }
    *out = st;
    return GBFV_OK;
}

int gbfv_stats_destroy(gbfv_stats* st) {
    if (!st) return GBFV_OK;
    if (st->stream) cudaStreamSynchronize(st->stream);
    if (st->mean) cudaFree(st->mean);
    if (st->m2) cudaFree(st->m2);
    if (st->scratch) cudaFree(st->scratch);
    if (st->stream) cudaStreamDestroy(st->stream);
    delete st;
    return GBFV_OK;
}

int gbfv_stats_reset(gbfv_stats* st) {
    if (!st) return sfail(GBFV_ERR_ARGUMENT, "null stats");
    st->n = 0;
    cudaMemsetAsync(st->mean, 0, st->count * sizeof(double), st->stream);
    cudaMemsetAsync(st->m2, 0, st->count * sizeof(double), st->stream);
    const cudaError_t e = cudaStreamSynchronize(st->stream);
    return e == cudaSuccess ? GBFV_OK : sfail(GBFV_ERR_CUDA, cudaGetErrorString(e));
}

int gbfv_stats_add_device(gbfv_stats* st, const void* x, int precision) {
    if (!st || !x) return sfail(GBFV_ERR_ARGUMENT, "null argument");
    st->n += 1;
    if (precision == GBFV_FP32)
        welford_add<float><<<grid_for(st->count), 256, 0, st->stream>>>(st->mean, st->m2, (const float*)x, st->count,
                                                                        (double)st->n);
    else
        welford_add<double><<<grid_for(st->count), 256, 0, st->stream>>>(st->mean, st->m2, (const double*)x,
                                                                         st->count, (double)st->n);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(st->stream);
    return e == cudaSuccess ? GBFV_OK : sfail(GBFV_ERR_CUDA, cudaGetErrorString(e));
}

int gbfv_stats_add_host(gbfv_stats* st, const double* x) {
    if (!st || !x) return sfail(GBFV_ERR_ARGUMENT, "null argument");
    cudaError_t e = cudaMemcpyAsync(st->scratch, x, st->count * sizeof(double), cudaMemcpyHostToDevice, st->stream);
    if (e != cudaSuccess) return sfail(GBFV_ERR_CUDA, cudaGetErrorString(e));
    return gbfv_stats_add_device(st, st->scratch, GBFV_FP64);
}

int gbfv_stats_merge(gbfv_stats* st, const gbfv_stats* o) {
    if (!st || !o || o->count != st->count) return sfail(GBFV_ERR_ARGUMENT, "mismatched statistics");
    if (o->n == 0) return GBFV_OK;
    cudaStreamSynchronize(o->stream);
    welford_merge<<<grid_for(st->count), 256, 0, st->stream>>>(st->mean, st->m2, o->mean, o->m2, st->count,
                                                                (double)st->n, (double)o->n);
    st->n += o->n;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(st->stream);
    return e == cudaSuccess ? GBFV_OK : sfail(GBFV_ERR_CUDA, cudaGetErrorString(e));
}

int gbfv_stats_result(gbfv_stats* st, double* mean, double* var, long long* samples) {
    if (!st) return sfail(GBFV_ERR_ARGUMENT, "null stats");
    if (samples) *samples = st->n;
    if (st->n == 0) return sfail(GBFV_ERR_ARGUMENT, "no samples");
    cudaError_t e = cudaSuccess;
    if (mean) e = cudaMemcpyAsync(mean, st->mean, st->count * sizeof(double), cudaMemcpyDeviceToHost, st->stream);
    if (var && e == cudaSuccess) {
        welford_finish<<<grid_for(st->count), 256, 0, st->stream>>>(st->m2, st->scratch, st->count, (double)st->n);
        e = cudaMemcpyAsync(var, st->scratch, st->count * sizeof(double), cudaMemcpyDeviceToHost, st->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st->stream);
    return e == cudaSuccess ? GBFV_OK : sfail(GBFV_ERR_CUDA, cudaGetErrorString(e));
}

int gbfv_stats_export(gbfv_stats* st, double* mean, double* m2, long long* samples) {
    if (!st) return sfail(GBFV_ERR_ARGUMENT, "null stats");
    if (samples) *samples = st->n;
    cudaError_t e = cudaSuccess;
    if (mean) e = cudaMemcpyAsync(mean, st->mean, st->count * sizeof(double), cudaMemcpyDeviceToHost, st->stream);
    if (m2 && e == cudaSuccess)
        e = cudaMemcpyAsync(m2, st->m2, st->count * sizeof(double), cudaMemcpyDeviceToHost, st->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st->stream);
    return e == cudaSuccess ? GBFV_OK : sfail(GBFV_ERR_CUDA, cudaGetErrorString(e));
}

}  // extern "C"
