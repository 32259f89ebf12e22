// Functionals of a state on the device: the reference's FunctionalFactory set
// that its CUDA platform registers (alsfvm/src/functional/: identity, moment,
// legendre_pointwise, log_entropy, bv, structure_cube) plus the per-direction
// total variation behind alsuq's bv_direction statistic. Each maps one padded
// state to a small volume (nvar x output cells) that is added, times a
// weight, into an FP64 accumulator on the device, as Functional::operator()
// adds into its output volume (alsfvm/include/alsfvm/functional/
// Functional.hpp:26-60).
//
//   identity            out(x) += w u(x)                       (Identity.cpp:25-49)
//   moment              out(x) += w pow(u(x), degree)          (Moment.cpp:27-41, HostMemory::addPower)
//   legendre_pointwise  out(x) += P_degree((u - min) / (max - min)) w, selected
//                       variables, 2D grids only                (LegendrePointWise.cpp:37-87)
//   log_entropy         out_E += w sum_x (-rho s / (gamma - 1)) dx dy dz,
//                       s = log p - gamma log rho              (LogEntropy.cpp:21-83)
//   bv                  out_v += w sum (sqrt((u - u_below)^2 + (u - u_left)^2))^degree,
//                       1D / 2D                                (BoundedVariation.cpp:21-40,
//                                                               HostMemory.cpp:325-362)
//   bv_direction        out_v += w sum |u - u(- e_d)|^degree     (HostMemory.cpp:365-400)
//   structure_cube      out = S(h) of this state, weight ignored (StructureCube.cpp:24-60:
//                       the reference zeroes its output first)
//
// Pointwise functionals run one thread per interior cell and round exactly as
// the reference (the unit is built with -fmad=false). The sums run as block
// reductions whose partials a second kernel adds in block order: the result
// does not depend on scheduling, and it differs from the reference's
// sequential sum only by rounding.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>

#include "gbfv.h"

int gbfv_internal_fail(int code, const char* msg);
double* gbfv_internal_structure_sums(gbfv_structure* s);

namespace {

enum { FN_IDENTITY, FN_MOMENT, FN_LEGENDRE, FN_LOG_ENTROPY, FN_BV, FN_BV_DIRECTION, FN_STRUCTURE_CUBE };

int parse_functional(const std::string& s) {
    if (s == "identity") return FN_IDENTITY;
    if (s == "moment") return FN_MOMENT;
    if (s == "legendre_pointwise") return FN_LEGENDRE;
    if (s == "log_entropy") return FN_LOG_ENTROPY;
    if (s == "bv") return FN_BV;
    if (s == "bv_direction") return FN_BV_DIRECTION;
    if (s == "structure_cube") return FN_STRUCTURE_CUBE;
    return -1;
}

int nvar_of(const std::string& eq) {
    if (eq == "burgers") return 1;
    if (eq == "euler1") return 3;
    if (eq == "euler2") return 4;
    if (eq == "euler3") return 5;
    return -1;
}

struct FnArgs {
    int n[3], g[3], t[3];
    long long total;
    int nvar, nsd;
    double weight;
    int degree;
    double min_value, max_value;
    unsigned mask;
    double gamma;
    double dxdydz;
    int direction;
    int lo[3], hi[3];  // padded cell range of the summed functionals
};

// Bonnet's recurrence in Boost.Math's legendre_p / legendre_next order
// (the reference's CPU LegendrePointWise calls boost::math::legendre_p):
// P_0 = 1, P_1 = x, P_{n+1} = ((2n+1) x P_n - n P_{n-1}) / (n+1), P_{-l-1} = P_l.
__device__ double legendre_p(int l, double x) {
    if (l < 0) l = -l - 1;
    double p0 = 1.0, p1 = x;
    if (l == 0) return p0;
    for (unsigned n = 1; n < (unsigned)l; ++n) {
        const double t = p0;
        p0 = p1;
        p1 = t;
        p1 = ((double)(2 * n + 1) * x * p0 - (double)n * p1) / (double)(n + 1);
    }
    return p1;
}

template <class T, int FN>
__global__ void pointwise_kernel(const T* __restrict__ U, FnArgs A, double* __restrict__ out, int* flag) {
    const long long cells = (long long)A.n[0] * A.n[1] * A.n[2];
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cells) return;
    const int i = (int)(c % A.n[0]);
    const int j = (int)((c / A.n[0]) % A.n[1]);
    const int k = (int)(c / ((long long)A.n[0] * A.n[1]));
    const long long p = ((long long)(k + A.g[2]) * A.t[1] + (j + A.g[1])) * A.t[0] + (i + A.g[0]);
    for (int v = 0; v < A.nvar; ++v) {
        if (FN == FN_LEGENDRE && A.mask && !((A.mask >> v) & 1u)) continue;
        const double x = (double)U[(long long)v * A.total + p];
        double* o = out + (long long)v * cells + c;
        if (FN == FN_IDENTITY) {
            *o += A.weight * x;
        } else if (FN == FN_MOMENT) {
            *o += A.weight * pow(x, (double)A.degree);
        } else {
            const double s = (x - A.min_value) / (A.max_value - A.min_value);
            if (!(s >= -1.0 && s <= 1.0)) {
                atomicExch(flag, 1);  // outside Boost's domain: the reference throws
                continue;
            }
            *o += legendre_p(A.degree, s) * A.weight;
        }
    }
}

constexpr int kSumThreads = 256;

template <class T, int FN>
__device__ double sum_term(const T* U, const FnArgs& A, int v, int x, int y, int z) {
    const T* u = U + (long long)v * A.total;
    const long long i = ((long long)z * A.t[1] + y) * A.t[0] + x;
    if (FN == FN_LOG_ENTROPY) {
        const double density = (double)U[i];
        const double energy = (double)U[(long long)(A.nvar - 1) * A.total + i];
        double momentumSquared = 0.0;
        for (int m = 0; m < A.nsd; ++m) {
            const double mm = (double)U[(long long)(1 + m) * A.total + i];
            momentumSquared += mm * mm;
        }
        const double pressure = (A.gamma - 1) * (energy - 1.0 / (2 * density) * momentumSquared);
        const double s = log(pressure) - A.gamma * log(density);
        const double e = (-density * s) / (A.gamma - 1);
        return e * A.dxdydz;
    } else if (FN == FN_BV) {
        const double d = (double)u[i];
        const double dl = (double)u[i - 1];
        const double db = A.t[1] > 1 ? (double)u[i - A.t[0]] : d;
        return pow(sqrt(pow(d - db, 2.0) + pow(d - dl, 2.0)), (double)A.degree);
    } else {  // FN_BV_DIRECTION
        const long long off = A.direction == 0 ? 1 : (A.direction == 1 ? A.t[0] : (long long)A.t[0] * A.t[1]);
        return pow(fabs((double)u[i] - (double)u[i - off]), (double)A.degree);
    }
}

// grid: (blocks over the range, variables); partial[v * nblocks + block]
template <class T, int FN>
__global__ void __launch_bounds__(kSumThreads) sum_kernel(const T* __restrict__ U, FnArgs A, double* partial) {
    __shared__ double red[kSumThreads / 32];
    const int v = blockIdx.y;
    const long long ex = A.hi[0] - A.lo[0], ey = A.hi[1] - A.lo[1], ez = A.hi[2] - A.lo[2];
    const long long c = (long long)blockIdx.x * kSumThreads + threadIdx.x;
    double s = 0.0;
    if (c < ex * ey * ez) {
        const int x = A.lo[0] + (int)(c % ex);
        const int y = A.lo[1] + (int)((c / ex) % ey);
        const int z = A.lo[2] + (int)(c / (ex * ey));
        s = sum_term<T, FN>(U, A, v, x, y, z);
    }
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < kSumThreads / 32; ++w) t += red[w];
        partial[(long long)v * gridDim.x + blockIdx.x] = t;
    }
}

// out[(v + first) * out_stride] += weight * (partials of sum v in block order)
__global__ void sum_finish(const double* __restrict__ partial, int nblocks, int nsums, int first, double weight,
                           double* out, long long out_stride) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nsums) return;
    double t = 0.0;
    for (int b = 0; b < nblocks; ++b) t += partial[(long long)v * nblocks + b];
    out[(long long)(v + first) * out_stride] += weight * t;
}

int ffail(int code, const std::string& m) { return gbfv_internal_fail(code, m.c_str()); }

}  // namespace

struct gbfv_functional {
    int fn = 0;
    FnArgs A;
    int out_n[3] = {1, 1, 1};
    long long out_cells = 1;
    int nblocks = 0;
    double* d_out = nullptr;
    double* d_partial = nullptr;
    int* d_flag = nullptr;
    gbfv_structure* sc = nullptr;
    cudaStream_t stream = nullptr;
};

template <class T>
static void launch_functional(gbfv_functional* f, const T* U) {
    FnArgs& A = f->A;
    cudaStream_t q = f->stream;
    const long long cells = (long long)A.n[0] * A.n[1] * A.n[2];
    const unsigned pb = (unsigned)((cells + 255) / 256);
    switch (f->fn) {
        case FN_IDENTITY: pointwise_kernel<T, FN_IDENTITY><<<pb, 256, 0, q>>>(U, A, f->d_out, f->d_flag); break;
        case FN_MOMENT: pointwise_kernel<T, FN_MOMENT><<<pb, 256, 0, q>>>(U, A, f->d_out, f->d_flag); break;
        case FN_LEGENDRE: pointwise_kernel<T, FN_LEGENDRE><<<pb, 256, 0, q>>>(U, A, f->d_out, f->d_flag); break;
        default: {
            // log_entropy is one sum, added to the energy variable's entry only
            const bool le = f->fn == FN_LOG_ENTROPY;
            const int nsums = le ? 1 : A.nvar;
            const dim3 grid((unsigned)f->nblocks, (unsigned)nsums);
            if (le)
                sum_kernel<T, FN_LOG_ENTROPY><<<grid, kSumThreads, 0, q>>>(U, A, f->d_partial);
            else if (f->fn == FN_BV)
                sum_kernel<T, FN_BV><<<grid, kSumThreads, 0, q>>>(U, A, f->d_partial);
            else
                sum_kernel<T, FN_BV_DIRECTION><<<grid, kSumThreads, 0, q>>>(U, A, f->d_partial);
            sum_finish<<<1, 32, 0, q>>>(f->d_partial, f->nblocks, nsums, le ? A.nvar - 1 : 0, A.weight, f->d_out,
                                        f->out_cells);
        }
    }
}

extern "C" {

int gbfv_functional_create(const char* name, const char* equation, const char* boundary, const int n[3], int ghosts,
                           const double lower[3], const double upper[3], const gbfv_functional_params* params,
                           gbfv_functional** out) {
    if (!name || !equation || !boundary || !n || !lower || !upper || !params || !out)
        return ffail(GBFV_ERR_ARGUMENT, "null argument");
    *out = nullptr;
    const int fn = parse_functional(name);
    if (fn < 0) return ffail(GBFV_ERR_ARGUMENT, std::string("Unknown functional: ") + name);
    const int nvar = nvar_of(equation);
    if (nvar < 0) return ffail(GBFV_ERR_ARGUMENT, "unknown equation");
    const std::string bc(boundary);
    if (bc != "periodic" && bc != "neumann") return ffail(GBFV_ERR_ARGUMENT, "unknown boundary");
    for (int d = 0; d < 3; ++d)
        if (n[d] < 1) return ffail(GBFV_ERR_ARGUMENT, "grid dimensions must be >= 1");
    if (ghosts < 0) return ffail(GBFV_ERR_ARGUMENT, "negative ghost width");
    FnArgs A;
    std::memset(&A, 0, sizeof A);
    const int dim = n[2] > 1 ? 3 : (n[1] > 1 ? 2 : 1);
    A.total = 1;
    for (int d = 0; d < 3; ++d) {
        A.n[d] = n[d];
        A.g[d] = d < dim ? ghosts : 0;
        A.t[d] = n[d] + 2 * A.g[d];
        A.total *= A.t[d];
    }
    A.nvar = nvar;
    A.nsd = nvar == 1 ? 1 : nvar - 2;
    A.degree = params->degree;
    A.min_value = params->min_value;
    A.max_value = params->max_value;
    A.mask = params->variable_mask;
    A.gamma = params->gamma;
    A.direction = params->direction;
    // Grid::computeCellLengths (alsfvm/src/grid/Grid.cpp:24-42)
    double len[3];
    for (int d = 0; d < 3; ++d) len[d] = (upper[d] - lower[d]) / n[d];
    if (n[1] == 1) len[1] = 1;
    if (n[2] == 1) len[2] = 1;
    A.dxdydz = len[0] * len[1] * len[2];
    gbfv_functional* f = new gbfv_functional();
    f->fn = fn;
    switch (fn) {
        case FN_LEGENDRE:
            if (len[2] > 1 || len[1] == 1) {
                delete f;
                return ffail(GBFV_ERR_UNSUPPORTED, "For now, Legendre polynomials only support 2d");
            }
            // fall through
        case FN_IDENTITY:
        case FN_MOMENT:
            for (int d = 0; d < 3; ++d) f->out_n[d] = n[d];
            break;
        case FN_LOG_ENTROPY:
            if (nvar == 1) {
                delete f;
                return ffail(GBFV_ERR_UNSUPPORTED, "log_entropy needs the Euler variables rho, m, E");
            }
            for (int d = 0; d < 3; ++d) {
                A.lo[d] = A.g[d];
                A.hi[d] = A.t[d] - A.g[d];
            }
            break;
        case FN_BV:
            if (len[2] > 1 || A.t[2] > 1) {
                delete f;
                return ffail(GBFV_ERR_UNSUPPORTED, "For now, BoundedVariation only supports 2d and 1d");
            }
            A.lo[0] = A.g[0] + 1;
            A.hi[0] = A.t[0] - A.g[0];
            A.lo[1] = A.g[1] + (A.t[1] > 1 ? 1 : 0);
            A.hi[1] = A.t[1] - A.g[1];
            A.lo[2] = 0;
            A.hi[2] = A.t[2] - A.g[2];
            break;
        case FN_BV_DIRECTION:
            if (A.direction < 0 || A.direction >= dim) {
                delete f;
                return ffail(GBFV_ERR_ARGUMENT, "direction is bigger than the current dimension");
            }
            for (int d = 0; d < 3; ++d) {
                A.lo[d] = A.g[d] + (d == A.direction ? 1 : 0);
                A.hi[d] = A.t[d] - A.g[d];
            }
            break;
        default:  // FN_STRUCTURE_CUBE
            if (params->number_of_h < 1) {
                delete f;
                return ffail(GBFV_ERR_ARGUMENT, "numberOfH must be >= 1");
            }
            f->out_n[0] = params->number_of_h;
            break;
    }
    f->out_cells = (long long)f->out_n[0] * f->out_n[1] * f->out_n[2];
    if (fn == FN_LOG_ENTROPY || fn == FN_BV || fn == FN_BV_DIRECTION) {
        const long long range = (long long)(A.hi[0] - A.lo[0]) * (A.hi[1] - A.lo[1]) * (A.hi[2] - A.lo[2]);
        f->nblocks = (int)((range > 0 ? range : 1) + kSumThreads - 1) / kSumThreads;
    }
    f->A = A;
    cudaError_t e = cudaStreamCreateWithFlags(&f->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&f->d_out, (size_t)nvar * f->out_cells * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&f->d_flag, sizeof(int));
    if (e == cudaSuccess && f->nblocks)
        e = cudaMalloc(&f->d_partial, (size_t)nvar * f->nblocks * sizeof(double));
    if (e == cudaSuccess) e = cudaMemsetAsync(f->d_out, 0, (size_t)nvar * f->out_cells * sizeof(double), f->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(f->d_flag, 0, sizeof(int), f->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(f->stream);
    if (e != cudaSuccess) {
        gbfv_functional_destroy(f);
        return ffail(GBFV_ERR_MEMORY, std::string("gbfv_functional_create: ") + cudaGetErrorString(e));
    }
    if (fn == FN_STRUCTURE_CUBE) {
        const int r = gbfv_structure_create(boundary, n, ghosts, nvar, params->number_of_h, params->p, &f->sc);
        if (r) {
            gbfv_functional_destroy(f);
            return r;
        }
    }
    *out = f;
    return GBFV_OK;
}

int gbfv_functional_destroy(gbfv_functional* f) {
    if (!f) return GBFV_OK;
    if (f->stream) cudaStreamSynchronize(f->stream);
    if (f->sc) gbfv_structure_destroy(f->sc);
    cudaFree(f->d_out);
    cudaFree(f->d_partial);
    cudaFree(f->d_flag);
    if (f->stream) cudaStreamDestroy(f->stream);
    delete f;
    return GBFV_OK;
}

int gbfv_functional_size(const gbfv_functional* f, int size[3], int* nvar) {
    if (!f) return ffail(GBFV_ERR_ARGUMENT, "null functional");
    if (size)
        for (int d = 0; d < 3; ++d) size[d] = f->out_n[d];
    if (nvar) *nvar = f->A.nvar;
    return GBFV_OK;
}

int gbfv_functional_reset(gbfv_functional* f) {
    if (!f) return ffail(GBFV_ERR_ARGUMENT, "null functional");
    cudaError_t e = cudaMemsetAsync(f->d_out, 0, (size_t)f->A.nvar * f->out_cells * sizeof(double), f->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(f->stream);
    if (e != cudaSuccess) return ffail(GBFV_ERR_CUDA, cudaGetErrorString(e));
    return GBFV_OK;
}

int gbfv_functional_apply(gbfv_functional* f, const void* state_dev, int precision, double weight) {
    if (!f || !state_dev) return ffail(GBFV_ERR_ARGUMENT, "null argument");
    if (f->fn == FN_STRUCTURE_CUBE) {
        // this state's structure function replaces the output (the weight is not used)
        double* sums = gbfv_internal_structure_sums(f->sc);
        int r = gbfv_structure_reset(f->sc);
        if (!r) r = gbfv_structure_add_device(f->sc, state_dev, precision);
        if (r) return r;
        const cudaError_t e = cudaMemcpy(f->d_out, sums, (size_t)f->A.nvar * f->out_cells * sizeof(double),
                                         cudaMemcpyDeviceToDevice);
        if (e != cudaSuccess) return ffail(GBFV_ERR_CUDA, cudaGetErrorString(e));
        return GBFV_OK;
    }
    f->A.weight = weight;
    if (precision == GBFV_FP32)
        launch_functional<float>(f, (const float*)state_dev);
    else
        launch_functional<double>(f, (const double*)state_dev);
    int flag = 0;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(&flag, f->d_flag, sizeof(int), cudaMemcpyDeviceToHost, f->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(f->stream);
    if (e != cudaSuccess) return ffail(GBFV_ERR_CUDA, cudaGetErrorString(e));
    if (flag) {
        cudaMemsetAsync(f->d_flag, 0, sizeof(int), f->stream);
        cudaStreamSynchronize(f->stream);
        return ffail(GBFV_ERR_ARGUMENT,
                     "legendre_pointwise: the Legendre polynomial is defined for -1 <= (u - minValue) / "
                     "(maxValue - minValue) <= 1");
    }
    return GBFV_OK;
}

int gbfv_functional_result(gbfv_functional* f, double* out_host) {
    if (!f || !out_host) return ffail(GBFV_ERR_ARGUMENT, "null argument");
    cudaError_t e = cudaStreamSynchronize(f->stream);
    if (e == cudaSuccess)
        e = cudaMemcpy(out_host, f->d_out, (size_t)f->A.nvar * f->out_cells * sizeof(double), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return ffail(GBFV_ERR_CUDA, cudaGetErrorString(e));
    return GBFV_OK;
}

}  // extern "C"
