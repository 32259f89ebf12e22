// Accuracy of the fast FP64 special functions and the bit-pattern compare
// helpers of fv_math.cuh against CUDA's IEEE operations:
//   rcp_<double>      vs __drcp_rn(x)                    <= 1 ulp
//   rsqrt_nr          vs 1 / __dsqrt_rn(x)               <= 2 ulp
//   sqrt_<double>     vs __dsqrt_rn(x)                   <= 2 ulp
//   inv_sqrt_pair     (the FP64 state's: 1/rho by rcp_, sqrt(rho) as a
//                     double-float) 1/rho <= 1 ulp; sqrt(rho) within 2^-46
//                     relative wherever the kernels use it (df_root_range)
//   df_coef_to_double vs the IEEE sum hi + lo            <= 1 ulp, exact when
//                     lo's bits all fit under hi's (exponent gap <= 29)
//   gt0 / lt0 / ge0 / is0 / abs_less / fmin_ / fmax_: identical to the IEEE
//   comparisons and fmin / fmax on every pair of special and random values
// Prints the worst errors and "ALL PASSED" when every bound holds.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include "fv_math.cuh"

using namespace gbfv::common;

__global__ void functions_kernel(const double* x, int n, double* out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double v = x[i];
        double rinv;
        gbfv::dfloat wd;
        inv_sqrt_pair(v, rinv, wd);
        const double w = df_root_range(v) ? (double)wd : __dsqrt_rn(v);
        out[8 * i + 0] = rcp_<double>(v);
        out[8 * i + 1] = __drcp_rn(v);
        out[8 * i + 2] = rsqrt_nr(v);
        out[8 * i + 3] = __drcp_rn(__dsqrt_rn(v));
        out[8 * i + 4] = sqrt_<double>(v);
        out[8 * i + 5] = __dsqrt_rn(v);
        out[8 * i + 6] = rinv;
        out[8 * i + 7] = w;
    }
}

// double-float pairs from splits, products and differences of the inputs;
// out: the integer-pipe conversion, the IEEE sum, the exponent gap
__global__ void coef_kernel(const double* x, int n, double* out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const gbfv::dfloat a(x[i]), b(x[(i + 1) % n]);
        const gbfv::dfloat v[3] = {a, a * b, a - b};
        for (int k = 0; k < 3; ++k) {
            out[9 * i + 3 * k + 0] = df_coef_to_double(v[k]);
            out[9 * i + 3 * k + 1] = __dadd_rn((double)v[k].hi, (double)v[k].lo);
            const int eh = (__float_as_uint(v[k].hi) >> 23) & 0xff, el = (__float_as_uint(v[k].lo) >> 23) & 0xff;
            out[9 * i + 3 * k + 2] = (double)(eh - el);
        }
    }
}

// one pair (a, b) per thread: 7 boolean tests and 2 extrema from the helpers,
// the same from the IEEE operations
__global__ void compare_kernel(const double* a, const double* b, int n, int* flags, double* ext) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double x = a[i], y = b[i];
        int f = 0;
        f |= (gt0<double>(x) != (x > 0.0)) << 0;
        f |= (lt0<double>(x) != (x < 0.0)) << 1;
        f |= (ge0<double>(x) != (x >= 0.0)) << 2;
        f |= (is0<double>(x) != (x == 0.0)) << 3;
        f |= (abs_less<double>(x, y) != (fabs(x) < fabs(y))) << 4;
        flags[i] = f;
        ext[4 * i + 0] = fmin_<double>(x, y);
        ext[4 * i + 1] = fmin(x, y);
        ext[4 * i + 2] = fmax_<double>(x, y);
        ext[4 * i + 3] = fmax(x, y);
    }
}

static double ulps(double got, double want) {
    if (std::isnan(want)) return std::isnan(got) ? 0.0 : 1e300;
    if (std::isinf(want)) return got == want ? 0.0 : 1e300;
    if (got == want) return 0.0;
    const double u = std::nextafter(std::fabs(want), INFINITY) - std::fabs(want);
    return std::fabs(got - want) / u;
}

#define CUDA_OK(x)                                                         \
    do {                                                                   \
        cudaError_t e_ = (x);                                              \
        if (e_ != cudaSuccess) {                                           \
            std::printf("CUDA error %s at %d\n", cudaGetErrorString(e_), __LINE__); \
            return 2;                                                      \
        }                                                                  \
    } while (0)

int main() {
    // positive arguments over the whole range the kernels use them on
    std::mt19937_64 rng(12345);
    std::uniform_real_distribution<double> ex(-300.0, 300.0), mant(1.0, 10.0);
    std::vector<double> xs;
    for (int i = 0; i < 1 << 20; ++i) xs.push_back(mant(rng) * std::pow(10.0, ex(rng)));
    for (double v : {1.0, 2.0, 0.5, 4.0, 1.4, 2.5, 1e-300, 1e300, 9.99e299, 3.0, 7.0})
        xs.push_back(v);
    const int n = (int)xs.size();
    double *dx, *dout;
    CUDA_OK(cudaMalloc(&dx, n * sizeof(double)));
    CUDA_OK(cudaMalloc(&dout, 8 * (size_t)n * sizeof(double)));
    CUDA_OK(cudaMemcpy(dx, xs.data(), n * sizeof(double), cudaMemcpyHostToDevice));
    functions_kernel<<<152 * 4, 256>>>(dx, n, dout);
    CUDA_OK(cudaGetLastError());
    std::vector<double> out(8 * (size_t)n);
    CUDA_OK(cudaMemcpy(out.data(), dout, out.size() * sizeof(double), cudaMemcpyDeviceToHost));
    double worst[5] = {0, 0, 0, 0, 0};
    for (int i = 0; i < n; ++i) {
        const double* o = &out[8 * (size_t)i];
        worst[0] = std::fmax(worst[0], ulps(o[0], o[1]));
        worst[1] = std::fmax(worst[1], ulps(o[2], o[3]));
        worst[2] = std::fmax(worst[2], ulps(o[4], o[5]));
        worst[3] = std::fmax(worst[3], ulps(o[6], o[1]));
        worst[4] = std::fmax(worst[4], std::fabs(o[7] - o[5]) / o[5]);
    }
    std::printf("max ulp: rcp %.3g  rsqrt %.3g  sqrt %.3g  pair-rinv %.3g; pair-sqrt relative %.3g\n", worst[0],
                worst[1], worst[2], worst[3], worst[4]);
    bool ok = worst[0] <= 1.0 && worst[1] <= 2.0 && worst[2] <= 2.0 && worst[3] <= 1.0 && worst[4] <= 0x1p-46;

    // double-float coefficients back to double: values of the range the
    // coefficients take (weights, wave speeds), both signs
    {
        std::uniform_real_distribution<double> ce(-30.0, 30.0), cm(1.0, 2.0), sg(-1.0, 1.0);
        std::vector<double> cs;
        for (int i = 0; i < 1 << 18; ++i) cs.push_back((sg(rng) < 0 ? -1.0 : 1.0) * cm(rng) * std::pow(2.0, ce(rng)));
        for (double v : {1.0, -1.0, 0.5, 1.0 - 0x1p-30, 1.0 + 0x1p-40, -0.75, 0x1p-20 + 0x1p-60, 0.0, -0.0})
            cs.push_back(v);
        const int nc = (int)cs.size();
        double *dc, *dco;
        CUDA_OK(cudaMalloc(&dc, nc * sizeof(double)));
        CUDA_OK(cudaMalloc(&dco, 9 * (size_t)nc * sizeof(double)));
        CUDA_OK(cudaMemcpy(dc, cs.data(), nc * sizeof(double), cudaMemcpyHostToDevice));
        coef_kernel<<<152 * 4, 256>>>(dc, nc, dco);
        CUDA_OK(cudaGetLastError());
        std::vector<double> co(9 * (size_t)nc);
        CUDA_OK(cudaMemcpy(co.data(), dco, co.size() * sizeof(double), cudaMemcpyDeviceToHost));
        double worst_coef = 0;
        int inexact_small_gap = 0;
        for (size_t j = 0; j < co.size(); j += 3) {
            worst_coef = std::fmax(worst_coef, ulps(co[j], co[j + 1]));
            if (co[j + 2] <= 29 && co[j] != co[j + 1] && !(co[j] == 0 && co[j + 1] == 0)) ++inexact_small_gap;
        }
        std::printf("df_coef_to_double: max ulp %.3g, inexact with gap <= 29: %d\n", worst_coef, inexact_small_gap);
        ok = ok && worst_coef <= 1.0 && inexact_small_gap == 0;
        cudaFree(dc);
        cudaFree(dco);
    }

    // all pairs of special and a few ordinary values
    const double specials[] = {0.0, -0.0, 1.0, -1.0, 2.5, -2.5, 1e-310, -1e-310, 1e308, -1e308,
                               INFINITY, -INFINITY, NAN, -NAN, 3e-5, -7.25};
    std::vector<double> as, bs;
    for (double a : specials)
        for (double b : specials) {
            as.push_back(a);
            bs.push_back(b);
        }
    std::uniform_real_distribution<double> r(-5.0, 5.0);
    for (int i = 0; i < 4096; ++i) {
        as.push_back(r(rng));
        bs.push_back(r(rng));
    }
    const int m = (int)as.size();
    double *da, *db, *dext;
    int* dflags;
    CUDA_OK(cudaMalloc(&da, m * sizeof(double)));
    CUDA_OK(cudaMalloc(&db, m * sizeof(double)));
    CUDA_OK(cudaMalloc(&dext, 4 * (size_t)m * sizeof(double)));
    CUDA_OK(cudaMalloc(&dflags, m * sizeof(int)));
    CUDA_OK(cudaMemcpy(da, as.data(), m * sizeof(double), cudaMemcpyHostToDevice));
    CUDA_OK(cudaMemcpy(db, bs.data(), m * sizeof(double), cudaMemcpyHostToDevice));
    compare_kernel<<<64, 256>>>(da, db, m, dflags, dext);
    CUDA_OK(cudaGetLastError());
    std::vector<int> flags(m);
    std::vector<double> ext(4 * (size_t)m);
    CUDA_OK(cudaMemcpy(flags.data(), dflags, m * sizeof(int), cudaMemcpyDeviceToHost));
    CUDA_OK(cudaMemcpy(ext.data(), dext, ext.size() * sizeof(double), cudaMemcpyDeviceToHost));
    int bad = 0;
    for (int i = 0; i < m; ++i) {
        const double* e = &ext[4 * (size_t)i];
        // extrema: the same value (either zero of a +-0 pair; NaN only for two NaNs)
        const bool min_ok = (std::isnan(e[1]) && std::isnan(e[0])) || e[0] == e[1];
        const bool max_ok = (std::isnan(e[3]) && std::isnan(e[2])) || e[2] == e[3];
        if (flags[i] || !min_ok || !max_ok) {
            if (bad < 10)
                std::printf("  mismatch a=%g b=%g flags=%x min %g/%g max %g/%g\n", as[i], bs[i], flags[i], e[0], e[1],
                            e[2], e[3]);
            ++bad;
        }
    }
    std::printf("compare helpers: %d mismatches in %d pairs\n", bad, m);
    ok = ok && bad == 0;
    cudaFree(dx);
    cudaFree(dout);
    cudaFree(da);
    cudaFree(db);
    cudaFree(dext);
    cudaFree(dflags);
    if (ok) std::printf("ALL PASSED\n");
    return ok ? 0 : 1;
}
