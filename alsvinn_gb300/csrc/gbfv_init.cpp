// Initial data of the benchmark workloads, evaluated at cell midpoints
// origin + dx*i + dx/2 (alsfvm/src/grid/Grid.cpp:148-165) on the host, as the
// reference evaluates its initial data on the CPU (alsfvm/src/simulator/
// Simulator.cpp:129-150). Output: interior primitive variables (rho, u..., p)
// or (u), one block per variable, x fastest. Built with -ffp-contract=off;
// the C library's sin/cos make the values identical to any other evaluation of
// the same expressions through the same library.
#include <cmath>

#include "gbfv.h"

int gbfv_internal_fail(int code, const char* msg);

namespace {

const double kPi = 3.141592653589793;

double midpoint(const double lower[3], const double upper[3], const int n[3], int d, int i) {
    const double h = (upper[d] - lower[d]) / n[d];
    return lower[d] + h * i + h / 2.0;
}

double kh_perturbation(double x, const double* a, const double* b) {
    double s = 0.0;
    for (int j = 0; j < 10; ++j) s += a[j] * std::cos(b[j] + 2 * kPi * (j + 1) * x);
    return 0.01 * s;
}

}  // namespace

extern "C" {

int gbfv_init_sod(const int n[3], const double lower[3], const double upper[3], double* prim) {
    if (!n || !lower || !upper || !prim || n[0] < 1) return gbfv_internal_fail(GBFV_ERR_ARGUMENT, "bad arguments");
    const long long cells = n[0];
    for (int i = 0; i < n[0]; ++i) {
        const bool left = midpoint(lower, upper, n, 0, i) < 0;
        prim[i] = left ? 1.0 : 0.125;
        prim[cells + i] = 0.0;
        prim[2 * cells + i] = left ? 1.0 : 0.1;
    }
    return GBFV_OK;
}

int gbfv_init_kelvin_helmholtz(const int n[3], const double lower[3], const double upper[3], const double X[40],
                               double* prim) {
    if (!n || !lower || !upper || !X || !prim || n[0] < 1 || n[1] < 1)
        return gbfv_internal_fail(GBFV_ERR_ARGUMENT, "bad arguments");
    // a_j normalised to sum 1 and b_j = 2 pi X for each interface:
    // X[0:10] a1, X[10:20] b1, X[20:30] a2, X[30:40] b2
    double a1[10], b1[10], a2[10], b2[10];
    double s1 = 0, s2 = 0;
    for (int j = 0; j < 10; ++j) {
        s1 += X[j];
        s2 += X[20 + j];
    }
    for (int j = 0; j < 10; ++j) {
        a1[j] = X[j] / s1;
        b1[j] = 2 * kPi * X[10 + j];
        a2[j] = X[20 + j] / s2;
        b2[j] = 2 * kPi * X[30 + j];
    }
    const long long cells = (long long)n[0] * n[1];
    double* d1 = new double[n[0]];
    double* d2 = new double[n[0]];
    for (int i = 0; i < n[0]; ++i) {
        const double x = midpoint(lower, upper, n, 0, i);
        d1[i] = kh_perturbation(x, a1, b1);
        d2[i] = kh_perturbation(x, a2, b2);
    }
    for (int j = 0; j < n[1]; ++j) {
        const double y = midpoint(lower, upper, n, 1, j);
        for (int i = 0; i < n[0]; ++i) {
            const bool inside = (0.25 + d1[i] < y) && (y < 0.75 + d2[i]);
            const long long k = (long long)j * n[0] + i;
            prim[k] = inside ? 2.0 : 1.0;
            prim[cells + k] = inside ? -0.5 : 0.5;
            prim[2 * cells + k] = 0.0;
            prim[3 * cells + k] = 2.5;
        }
    }
    delete[] d1;
    delete[] d2;
    return GBFV_OK;
}

int gbfv_init_taylor_green(const int n[3], const double lower[3], const double upper[3], double* prim) {
    if (!n || !lower || !upper || !prim || n[0] < 1 || n[1] < 1 || n[2] < 1)
        return gbfv_internal_fail(GBFV_ERR_ARGUMENT, "bad arguments");
    const long long cells = (long long)n[0] * n[1] * n[2];
    for (int kz = 0; kz < n[2]; ++kz) {
        const double z = midpoint(lower, upper, n, 2, kz);
        for (int j = 0; j < n[1]; ++j) {
            const double y = midpoint(lower, upper, n, 1, j);
            for (int i = 0; i < n[0]; ++i) {
                const double x = midpoint(lower, upper, n, 0, i);
                const long long k = ((long long)kz * n[1] + j) * n[0] + i;
                prim[k] = 1.0;
                prim[cells + k] = std::sin(x) * std::cos(y) * std::cos(z);
                prim[2 * cells + k] = -std::cos(x) * std::sin(y) * std::cos(z);
                prim[3 * cells + k] = 0.0;
                prim[4 * cells + k] =
                    100 + ((std::cos(2 * x) + std::cos(2 * y)) * (std::cos(2 * z) + 2) - 2) / 16;
            }
        }
    }
    return GBFV_OK;
}

int gbfv_init_burgers_sine(const int n[3], const double lower[3], const double upper[3], double phase,
                           double* prim) {
    if (!n || !lower || !upper || !prim || n[0] < 1) return gbfv_internal_fail(GBFV_ERR_ARGUMENT, "bad arguments");
    const long long nx = n[0], ny = n[1] > 0 ? n[1] : 1, nz = n[2] > 0 ? n[2] : 1;
    for (long long k = 0; k < nz; ++k)
        for (long long j = 0; j < ny; ++j)
            for (int i = 0; i < n[0]; ++i) {
                const double x = midpoint(lower, upper, n, 0, i);
                prim[(k * ny + j) * nx + i] = std::sin(2 * kPi * x) + 0.5 * phase;
            }
    return GBFV_OK;
}

}  // extern "C"
