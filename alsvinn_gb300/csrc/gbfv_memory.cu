// Elementwise arithmetic of device arrays: what a device Memory<real> of the
// "gb300" platform needs to run the reference's own integrators and
// statistics on device state (memory::Memory<real>, alsfvm/include/alsfvm/
// memory/Memory.hpp:166-302; the reference's cuda platform implements it in
// alsfvm/src/cuda/CudaMemory.cpp over alsfvm/src/cuda/vector_operations.cu).
//
// Every operation runs in the element type of the array, in the order the
// reference's HostMemory loops write it (alsfvm/src/memory/HostMemory.cpp:
// 97-311), and this unit is compiled without multiply-add contraction, so
// FP64 results equal the reference CPU path's bit for bit (pow with a power
// other than 1 or 2 is CUDA's, within its documented error bound).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>

#include "gbfv_internal.h"

namespace {

int mfail(int code, const char* msg) { return gbfv_internal_fail(code, msg); }

unsigned blocks_for(long long n) {
    const long long b = (n + 255) / 256;
    return (unsigned)(b < 152 * 16 ? (b > 0 ? b : 1) : 152 * 16);
}

template <class T>
__global__ void memory_op_kernel(T* a, const T* b, long long n, int op) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const T x = a[i], y = b[i];
        a[i] = op == GBFV_MEMORY_ADD ? x + y : (op == GBFV_MEMORY_SUBTRACT ? x - y : (op == GBFV_MEMORY_MULTIPLY ? x * y : x / y));
    }
}

// data[i] op= scalar with a double scalar: a float element is widened, the
// operation runs in double and the result is rounded back, as `float +=
// double` does in C++.
template <class T>
__global__ void memory_scalar_kernel(T* a, double s, long long n, int op) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double x = (double)a[i];
        a[i] = (T)(op == GBFV_MEMORY_ADD ? x + s : (op == GBFV_MEMORY_SUBTRACT ? x - s : (op == GBFV_MEMORY_MULTIPLY ? x * s : x / s)));
    }
}

// v1 = a1 v1 + a2 v2 + a3 v3 + a4 v4 + a5 v5, summed left to right with
// coefficients of the element type (Memory<T>::addLinearCombination).
template <class T>
__global__ void memory_lincomb_kernel(T* v1, T a1, T a2, const T* v2, T a3, const T* v3, T a4, const T* v4, T a5,
                                      const T* v5, long long n) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        v1[i] = a1 * v1[i] + a2 * v2[i] + a3 * v3[i] + a4 * v4[i] + a5 * v5[i];
}

__device__ __forceinline__ double power_of(double x, double p) {
    if (p == 1.0) return x;
    if (p == 2.0) return x * x;
    return pow(x, p);
}

// a += factor * pow(b, power) (sign = 1) or a -= pow(b, power) (sign = -1,
// factor 1), the power and the product in double.
template <class T>
__global__ void memory_power_kernel(T* a, const T* b, double power, double factor, int sign, long long n) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double pw = power_of((double)b[i], power);
        const double x = (double)a[i];
        a[i] = (T)(sign > 0 ? x + factor * pw : x - pw);
    }
}

// Total variation over a box of a padded array with extents t (x fastest):
// direction < 0: sum over x in [lo0, hi0), y in [lo1, hi1), z in [lo2, hi2)
// of pow(sqrt(pow(u - u(y-1), 2) + pow(u - u(x-1), 2)), p); direction d:
// sum of pow(|u - u(-e_d)|, p). Per-block partial sums in FP64, combined in
// block order by a second launch, so the result does not depend on timing.
template <class T>
__global__ void memory_tv_kernel(const T* a, int t0, int t1, int lo0, int lo1, int lo2, int e0, int e1, int e2,
                                 int direction, double p, double* partial) {
    __shared__ double red[256];
    const long long n = (long long)e0 * e1 * e2;
    double s = 0.0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int x = lo0 + (int)(i % e0), y = lo1 + (int)((i / e0) % e1), z = lo2 + (int)(i / ((long long)e0 * e1));
        const long long idx = ((long long)z * t1 + y) * t0 + x;
        const double u = (double)a[idx];
        if (direction < 0) {
            const long long ix = idx - 1;
            const long long iy = t1 > 1 ? idx - t0 : (long long)z * t1 * t0 + x;
            const double dy = u - (double)a[iy], dx = u - (double)a[ix];
            s += power_of(sqrt(dy * dy + dx * dx), p);
        } else {
            const long long step = direction == 0 ? 1 : (direction == 1 ? t0 : (long long)t0 * t1);
            s += power_of(fabs(u - (double)a[idx - step]), p);
        }
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

__global__ void sum_partials_kernel(const double* partial, int n, double* out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += partial[i];
    *out = s;
}

int elem_of(int precision) { return precision == GBFV_FP32 ? 4 : 8; }

bool valid_precision(int precision) { return precision >= GBFV_FP64 && precision <= GBFV_FP64_DF; }

#define MCUDA(x)                                                                                  \
    do {                                                                                          \
        cudaError_t e_ = (x);                                                                     \
        if (e_ != cudaSuccess) {                                                                  \
            char m_[256];                                                                         \
            snprintf(m_, sizeof m_, "%s: %s", #x, cudaGetErrorString(e_));                        \
            return mfail(GBFV_ERR_CUDA, m_);                                                      \
        }                                                                                         \
    } while (0)

}  // namespace

extern "C" {

int gbfv_memory_op(int op, void* a_dev, const void* b_dev, long long count, int precision, void* stream) {
    if (!a_dev || !b_dev || count < 0 || op < GBFV_MEMORY_ADD || op > GBFV_MEMORY_DIVIDE || !valid_precision(precision))
        return mfail(GBFV_ERR_ARGUMENT, "gbfv_memory_op: bad arguments");
    if (count == 0) return GBFV_OK;
    cudaStream_t q = (cudaStream_t)stream;
    if (elem_of(precision) == 8)
        memory_op_kernel<double><<<blocks_for(count), 256, 0, q>>>((double*)a_dev, (const double*)b_dev, count, op);
    else
        memory_op_kernel<float><<<blocks_for(count), 256, 0, q>>>((float*)a_dev, (const float*)b_dev, count, op);
    MCUDA(cudaGetLastError());
    return GBFV_OK;
}

int gbfv_memory_op_scalar(int op, void* a_dev, double scalar, long long count, int precision, void* stream) {
    if (!a_dev || count < 0 || op < GBFV_MEMORY_ADD || op > GBFV_MEMORY_DIVIDE || !valid_precision(precision))
        return mfail(GBFV_ERR_ARGUMENT, "gbfv_memory_op_scalar: bad arguments");
    if (count == 0) return GBFV_OK;
    cudaStream_t q = (cudaStream_t)stream;
    if (elem_of(precision) == 8)
        memory_scalar_kernel<double><<<blocks_for(count), 256, 0, q>>>((double*)a_dev, scalar, count, op);
    else
        memory_scalar_kernel<float><<<blocks_for(count), 256, 0, q>>>((float*)a_dev, scalar, count, op);
    MCUDA(cudaGetLastError());
    return GBFV_OK;
}

int gbfv_memory_make_zero(void* a_dev, long long count, int precision, void* stream) {
    if (!a_dev || count < 0 || !valid_precision(precision))
        return mfail(GBFV_ERR_ARGUMENT, "gbfv_memory_make_zero: bad arguments");
    MCUDA(cudaMemsetAsync(a_dev, 0, (size_t)count * elem_of(precision), (cudaStream_t)stream));
    return GBFV_OK;
}

int gbfv_memory_add_linear_combination(void* v1_dev, double a1, double a2, const void* v2_dev, double a3,
                                       const void* v3_dev, double a4, const void* v4_dev, double a5,
                                       const void* v5_dev, long long count, int precision, void* stream) {
    if (!v1_dev || !v2_dev || !v3_dev || !v4_dev || !v5_dev || count < 0 || !valid_precision(precision))
        return mfail(GBFV_ERR_ARGUMENT, "gbfv_memory_add_linear_combination: bad arguments");
    if (count == 0) return GBFV_OK;
    cudaStream_t q = (cudaStream_t)stream;
    if (elem_of(precision) == 8)
        memory_lincomb_kernel<double><<<blocks_for(count), 256, 0, q>>>(
            (double*)v1_dev, a1, a2, (const double*)v2_dev, a3, (const double*)v3_dev, a4, (const double*)v4_dev, a5,
            (const double*)v5_dev, count);
    else
        memory_lincomb_kernel<float><<<blocks_for(count), 256, 0, q>>>(
            (float*)v1_dev, (float)a1, (float)a2, (const float*)v2_dev, (float)a3, (const float*)v3_dev, (float)a4,
            (const float*)v4_dev, (float)a5, (const float*)v5_dev, count);
    MCUDA(cudaGetLastError());
    return GBFV_OK;
}

static int power_op(void* a_dev, const void* b_dev, double power, double factor, int sign, long long count,
                    int precision, void* stream) {
    if (!a_dev || !b_dev || count < 0 || !valid_precision(precision))
        return mfail(GBFV_ERR_ARGUMENT, "gbfv_memory power operation: bad arguments");
    if (count == 0) return GBFV_OK;
    cudaStream_t q = (cudaStream_t)stream;
    if (elem_of(precision) == 8)
        memory_power_kernel<double><<<blocks_for(count), 256, 0, q>>>((double*)a_dev, (const double*)b_dev, power,
                                                                      factor, sign, count);
    else
        memory_power_kernel<float><<<blocks_for(count), 256, 0, q>>>((float*)a_dev, (const float*)b_dev, power,
                                                                     factor, sign, count);
    MCUDA(cudaGetLastError());
    return GBFV_OK;
}

int gbfv_memory_add_power(void* a_dev, const void* b_dev, double power, double factor, long long count, int precision,
                          void* stream) {
    return power_op(a_dev, b_dev, power, factor, 1, count, precision, stream);
}

int gbfv_memory_subtract_power(void* a_dev, const void* b_dev, double power, long long count, int precision,
                               void* stream) {
    return power_op(a_dev, b_dev, power, 1.0, -1, count, precision, stream);
}

int gbfv_memory_total_variation(const void* a_dev, const int extents[3], int p, int direction, const int start[3],
                                const int end[3], int precision, double* result, void* stream) {
    if (!a_dev || !extents || !start || !end || !result || !valid_precision(precision) || direction < -1 ||
        direction > 2)
        return mfail(GBFV_ERR_ARGUMENT, "gbfv_memory_total_variation: bad arguments");
    const int t0 = extents[0], t1 = extents[1], t2 = extents[2];
    if (t0 < 1 || t1 < 1 || t2 < 1) return mfail(GBFV_ERR_ARGUMENT, "gbfv_memory_total_variation: bad extents");
    int lo[3], hi[3];
    if (direction < 0) {
        // the reference's isotropic total variation is 1D / 2D only
        if (t2 > 1) return mfail(GBFV_ERR_UNSUPPORTED, "the total variation over all directions is 1D / 2D only");
        lo[0] = start[0] + 1;
        lo[1] = start[1] + (t1 > 1 ? 1 : 0);
        lo[2] = 0;
        hi[0] = end[0];
        hi[1] = end[1];
        hi[2] = end[2];
    } else {
        const int active = 1 + (t1 > 1) + (t2 > 1);
        if (direction > active) return mfail(GBFV_ERR_ARGUMENT, "direction is bigger than the grid's dimension");
        for (int k = 0; k < 3; ++k) {
            lo[k] = start[k] + (k == direction ? 1 : 0);
            hi[k] = end[k];
        }
    }
    const int ext[3] = {t0, t1, t2};
    for (int k = 0; k < 3; ++k) {
        if (hi[k] > ext[k] || lo[k] < 0)
            return mfail(GBFV_ERR_ARGUMENT, "gbfv_memory_total_variation: the range leaves the array");
        if (hi[k] <= lo[k]) {
            *result = 0.0;
            return GBFV_OK;
        }
    }
    const int e0 = hi[0] - lo[0], e1 = hi[1] - lo[1], e2 = hi[2] - lo[2];
    cudaStream_t q = (cudaStream_t)stream;
    const unsigned nb = blocks_for((long long)e0 * e1 * e2);
    double* buf = nullptr;
    MCUDA(cudaMallocAsync(&buf, (nb + 1) * sizeof(double), q));
    if (elem_of(precision) == 8)
        memory_tv_kernel<double><<<nb, 256, 0, q>>>((const double*)a_dev, t0, t1, lo[0], lo[1], lo[2], e0, e1, e2,
                                                    direction, (double)p, buf);
    else
        memory_tv_kernel<float><<<nb, 256, 0, q>>>((const float*)a_dev, t0, t1, lo[0], lo[1], lo[2], e0, e1, e2,
                                                   direction, (double)p, buf);
    sum_partials_kernel<<<1, 32, 0, q>>>(buf, (int)nb, buf + nb);
    cudaError_t e = cudaGetLastError();
    double h = 0.0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, buf + nb, sizeof(double), cudaMemcpyDeviceToHost, q);
    cudaError_t f = cudaFreeAsync(buf, q);
    if (e == cudaSuccess) e = cudaStreamSynchronize(q);
    if (e == cudaSuccess) e = f;
    MCUDA(e);
    *result = h;
    return GBFV_OK;
}

}  // extern "C"
