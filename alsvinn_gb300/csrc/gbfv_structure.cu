// Cube structure functions of ensemble states on the device: alsuq's
// StructureCube statistic (alsuq/src/stats/StructureCube.cpp:36-76) with the
// kernel of alsfvm/include/alsfvm/functional/structure_common.hpp:37-154.
// For every variable and h in 1 .. H-1 one sample contributes
//     S(h) = sum over cells x, over the points y of the cube surface at
//            distance h around x, of |u(x) - u(y)|^p / (nx ny nz),
// with the surface visited per direction and side in the reference's loop
// bounds and points outside the grid wrapped (periodic) or clamped (Neumann)
// to the interior (ValueAtBoundary.hpp). The statistic is the mean of S over
// the samples (StatisticsHelper::combineStatistics divides the rank sums by
// the sample count).
//
// One thread per cell; per h a block reduction writes one partial sum per
// block, and a second kernel adds the partials in block order, so a sample's
// contribution does not depend on scheduling.
#include <cuda_runtime.h>

#include <cmath>
#include <string>

#include "gbfv.h"

int gbfv_internal_fail(int code, const char* msg);

namespace {

struct StructGrid {
    int n[3];
    int g[3];
    int t[3];
    int dim;
    int periodic;
    long long total;
};

__device__ __forceinline__ int wrap_or_clamp(int q, int n, int periodic) {
    if (periodic) {
        while (q < 0) q += n;
        return q % n;
    }
    q = q < n - 1 ? q : n - 1;
    return q > 0 ? q : 0;
}

__device__ __forceinline__ long long struct_index(const StructGrid& G, int x, int y, int z) {
    x = wrap_or_clamp(x, G.n[0], G.periodic) + G.g[0];
    y = wrap_or_clamp(y, G.n[1], G.periodic) + G.g[1];
    z = wrap_or_clamp(z, G.n[2], G.periodic) + G.g[2];
    return ((long long)z * G.t[1] + y) * G.t[0] + x;
}

// |x|^p: the reference's FastPower<p> products for p = 1..5, pow otherwise
template <int IP> __device__ __forceinline__ double struct_power(double x, double p) {
    if constexpr (IP == 1) return x;
    else if constexpr (IP == 2) return x * x;
    else if constexpr (IP == 3) return x * (x * x);
    else if constexpr (IP == 4) return x * (x * (x * x));
    else if constexpr (IP == 5) return x * (x * (x * (x * x)));
    else return pow(x, p);
}

constexpr int kThreads = 256;

// grid: (blocks over cells, nvar); partial[(v * H + h) * nblocks + block]
template <class T, int IP>
__global__ void __launch_bounds__(kThreads) structure_kernel(const T* __restrict__ U, StructGrid G, int H, double p,
                                                            double inv_cells, double* __restrict__ partial) {
    __shared__ double red[kThreads / 32];
    const int v = blockIdx.y;
    const long long cells = (long long)G.n[0] * G.n[1] * G.n[2];
    const long long c = (long long)blockIdx.x * kThreads + threadIdx.x;
    const bool active = c < cells;
    int i = 0, j = 0, k = 0;
    double uc = 0.0;
    const T* u = U + (long long)v * G.total;
    if (active) {
        i = (int)(c % G.n[0]);
        j = (int)((c / G.n[0]) % G.n[1]);
        k = (int)(c / ((long long)G.n[0] * G.n[1]));
        uc = (double)u[((long long)(k + G.g[2]) * G.t[1] + (j + G.g[1])) * G.t[0] + (i + G.g[0])];
    }
    const int dims = G.dim;
    for (int h = 1; h < H; ++h) {
        double s = 0.0;
        if (active) {
            for (int d = 0; d < dims; d++)
                for (int side = 0; side < 2; side++) {
                    const bool zDir = d == 2, yDir = d == 1, xDir = d == 0;
                    const int zStart = zDir ? (side == 0 ? k - h : k + h) : (dims > 2 ? k - h : 0);
                    const int zEnd = zDir ? (zStart + 1) : (dims > 2 ? k + h + 1 : 1);
                    const int yStart = yDir ? (side == 0 ? j - h : j + h) : (dims >= 2 ? j - h + 1 : 0);
                    const int yEnd = yDir ? (yStart + 1) : (dims >= 2 ? j + h : 1);
                    int xStart = xDir ? (side == 0 ? i - h : i + h) : i - h;
                    int xEnd = xDir ? (xStart + 1) : i + h + 1;
                    if (zDir) {
                        xStart += 1;
                        xEnd -= 1;
                    }
                    for (int z = zStart; z < zEnd; z++)
                        for (int y = yStart; y < yEnd; y++)
                            for (int x = xStart; x < xEnd; x++) {
                                const double uh = (double)u[struct_index(G, x, y, z)];
                                s += struct_power<IP>(fabs(uc - uh), p);
                            }
                }
            s *= inv_cells;
        }
        for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0.0;
            for (int w = 0; w < kThreads / 32; ++w) t += red[w];
            partial[((long long)v * H + h) * gridDim.x + blockIdx.x] = t;
        }
        __syncthreads();
    }
}

// Structure function along one axis (alsuq's StructureBasic,
// alsuq/src/stats/StructureBasic.cpp:50-92): for h in 0 .. H-1,
//     S(h) = sum over cells x of |u(x) - u(x + h e_dir)|^p / (nx ny nz),
// the shifted point wrapped (periodic) or clamped (Neumann) to the interior
// (ValueAtBoundary.hpp); pow as the reference's std::pow, one division per
// term.
template <class T>
__global__ void __launch_bounds__(kThreads) structure_basic_kernel(const T* __restrict__ U, StructGrid G, int H,
                                                                  double p, int dir, double* __restrict__ partial) {
    __shared__ double red[kThreads / 32];
    const int v = blockIdx.y;
    const long long cells = (long long)G.n[0] * G.n[1] * G.n[2];
    const long long c = (long long)blockIdx.x * kThreads + threadIdx.x;
    const bool active = c < cells;
    int i = 0, j = 0, k = 0;
    double uc = 0.0;
    const T* u = U + (long long)v * G.total;
    if (active) {
        i = (int)(c % G.n[0]);
        j = (int)((c / G.n[0]) % G.n[1]);
        k = (int)(c / ((long long)G.n[0] * G.n[1]));
        uc = (double)u[((long long)(k + G.g[2]) * G.t[1] + (j + G.g[1])) * G.t[0] + (i + G.g[0])];
    }
    const double ncells = (double)(G.n[0] * G.n[1] * G.n[2]);
    for (int h = 0; h < H; ++h) {
        double s = 0.0;
        if (active) {
            const double uh = (double)u[struct_index(G, i + (dir == 0) * h, j + (dir == 1) * h, k + (dir == 2) * h)];
            s = pow(fabs(uc - uh), p) / ncells;
        }
        for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0.0;
            for (int w = 0; w < kThreads / 32; ++w) t += red[w];
            partial[((long long)v * H + h) * gridDim.x + blockIdx.x] = t;
        }
        __syncthreads();
    }
}

// sums[v * H + h] += the partials of (v, h) in block order
__global__ void structure_finish(const double* __restrict__ partial, int nblocks, int count, double* sums) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= count) return;
    double t = 0.0;
    for (int b = 0; b < nblocks; ++b) t += partial[(long long)e * nblocks + b];
    sums[e] += t;
}

int sfail(int code, const std::string& m) { return gbfv_internal_fail(code, m.c_str()); }

}  // namespace

struct gbfv_structure {
    StructGrid G;
    int nvar = 0;
    int H = 0;
    double p = 2.0;
    int ip = 0;
    int nblocks = 0;
    long long samples = 0;
    int basic_dir = -1;  // >= 0: the axis structure function (structure_basic) along this axis
    double* d_partial = nullptr;
    double* d_sums = nullptr;
    cudaStream_t stream = nullptr;
};

template <class T>
static void launch_structure(gbfv_structure* s, const T* U) {
    const dim3 grid((unsigned)s->nblocks, (unsigned)s->nvar);
    if (s->basic_dir >= 0) {
        structure_basic_kernel<T><<<grid, kThreads, 0, s->stream>>>(U, s->G, s->H, s->p, s->basic_dir, s->d_partial);
        return;
    }
    const double inv = 1.0 / ((double)s->G.n[0] * s->G.n[1] * s->G.n[2]);
    switch (s->ip) {
        case 1: structure_kernel<T, 1><<<grid, kThreads, 0, s->stream>>>(U, s->G, s->H, s->p, inv, s->d_partial); break;
        case 2: structure_kernel<T, 2><<<grid, kThreads, 0, s->stream>>>(U, s->G, s->H, s->p, inv, s->d_partial); break;
        case 3: structure_kernel<T, 3><<<grid, kThreads, 0, s->stream>>>(U, s->G, s->H, s->p, inv, s->d_partial); break;
        case 4: structure_kernel<T, 4><<<grid, kThreads, 0, s->stream>>>(U, s->G, s->H, s->p, inv, s->d_partial); break;
        case 5: structure_kernel<T, 5><<<grid, kThreads, 0, s->stream>>>(U, s->G, s->H, s->p, inv, s->d_partial); break;
        default: structure_kernel<T, 0><<<grid, kThreads, 0, s->stream>>>(U, s->G, s->H, s->p, inv, s->d_partial); break;
    }
}

extern "C" {

int gbfv_structure_create(const char* boundary, const int n[3], int ghosts, int nvar, int number_of_h, double p,
                          gbfv_structure** out) {
    if (!boundary || !n || !out || nvar < 1 || number_of_h < 1 || ghosts < 0 || !(p > 0.0))
        return sfail(GBFV_ERR_ARGUMENT, "bad structure function arguments");
    const std::string bc(boundary);
    if (bc != "periodic" && bc != "neumann") return sfail(GBFV_ERR_ARGUMENT, "unknown boundary");
    for (int d = 0; d < 3; ++d)
        if (n[d] < 1) return sfail(GBFV_ERR_ARGUMENT, "grid dimensions must be >= 1");
    gbfv_structure* s = new gbfv_structure();
    StructGrid& G = s->G;
    G.dim = n[2] > 1 ? 3 : (n[1] > 1 ? 2 : 1);
    G.periodic = bc == "periodic";
    G.total = 1;
    for (int d = 0; d < 3; ++d) {
        G.n[d] = n[d];
        G.g[d] = d < G.dim ? ghosts : 0;
        G.t[d] = n[d] + 2 * G.g[d];
        G.total *= G.t[d];
    }
    s->nvar = nvar;
    s->H = number_of_h;
    s->p = p;
    s->ip = p == 1.0 ? 1 : p == 2.0 ? 2 : p == 3.0 ? 3 : p == 4.0 ? 4 : p == 5.0 ? 5 : 0;
    const long long cells = (long long)n[0] * n[1] * n[2];
    s->nblocks = (int)((cells + kThreads - 1) / kThreads);
    cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess)
        e = cudaMalloc(&s->d_partial, (size_t)nvar * number_of_h * s->nblocks * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&s->d_sums, (size_t)nvar * number_of_h * sizeof(double));
    if (e == cudaSuccess) e = cudaMemsetAsync(s->d_partial, 0, (size_t)nvar * number_of_h * s->nblocks * sizeof(double), s->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->d_sums, 0, (size_t)nvar * number_of_h * sizeof(double), s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) {
        gbfv_structure_destroy(s);
        return sfail(GBFV_ERR_MEMORY, std::string("gbfv_structure_create: ") + cudaGetErrorString(e));
    }
    *out = s;
    return GBFV_OK;
}

int gbfv_structure_create_basic(const char* boundary, const int n[3], int ghosts, int nvar, int number_of_h,
                                double p, int direction, gbfv_structure** out) {
    if (!n || !out) return sfail(GBFV_ERR_ARGUMENT, "null argument");
    const int dim = n[2] > 1 ? 3 : (n[1] > 1 ? 2 : 1);
    if (direction < 0 || direction >= dim) return sfail(GBFV_ERR_ARGUMENT, "direction outside the grid's dimension");
    const int r = gbfv_structure_create(boundary, n, ghosts, nvar, number_of_h, p, out);
    if (r) return r;
    (*out)->basic_dir = direction;
    return GBFV_OK;
}

int gbfv_structure_destroy(gbfv_structure* s) {
    if (!s) return GBFV_OK;
    if (s->stream) cudaStreamSynchronize(s->stream);
    if (s->d_partial) cudaFree(s->d_partial);
    if (s->d_sums) cudaFree(s->d_sums);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return GBFV_OK;
}

int gbfv_structure_add_device(gbfv_structure* s, const void* state_dev, int precision) {
    if (!s || !state_dev) return sfail(GBFV_ERR_ARGUMENT, "null argument");
    if (precision == GBFV_FP32)
        launch_structure<float>(s, (const float*)state_dev);
    else
        launch_structure<double>(s, (const double*)state_dev);
    const int count = s->nvar * s->H;
    structure_finish<<<(count + 127) / 128, 128, 0, s->stream>>>(s->d_partial, s->nblocks, count, s->d_sums);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return sfail(GBFV_ERR_CUDA, cudaGetErrorString(e));
    s->samples += 1;
    return GBFV_OK;
}

int gbfv_structure_reset(gbfv_structure* s) {
    if (!s) return sfail(GBFV_ERR_ARGUMENT, "null structure function");
    cudaError_t e = cudaMemsetAsync(s->d_sums, 0, (size_t)s->nvar * s->H * sizeof(double), s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return sfail(GBFV_ERR_CUDA, cudaGetErrorString(e));
    s->samples = 0;
    return GBFV_OK;
}

int gbfv_structure_export(gbfv_structure* s, double* sums_host, long long* samples) {
    if (!s) return sfail(GBFV_ERR_ARGUMENT, "null structure function");
    if (samples) *samples = s->samples;
    if (sums_host) {
        const cudaError_t e = cudaMemcpy(sums_host, s->d_sums, (size_t)s->nvar * s->H * sizeof(double),
                                         cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return sfail(GBFV_ERR_CUDA, cudaGetErrorString(e));
    }
    return GBFV_OK;
}

int gbfv_structure_result(gbfv_structure* s, double* mean_host, long long* samples) {
    if (!s || !mean_host) return sfail(GBFV_ERR_ARGUMENT, "null argument");
    const int r = gbfv_structure_export(s, mean_host, samples);
    if (r) return r;
    if (s->samples == 0) return sfail(GBFV_ERR_ARGUMENT, "no samples");
    for (int e = 0; e < s->nvar * s->H; ++e) mean_host[e] /= (double)s->samples;
    return GBFV_OK;
}

}  // extern "C"

// The device sums (nvar x number_of_h) of the structure function, for the
// structure_cube functional.
double* gbfv_internal_structure_sums(gbfv_structure* s) { return s ? s->d_sums : nullptr; }
