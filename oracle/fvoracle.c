/* CPU oracle: plain-C restatement of the reference's CPU implementation of the
 * explicit finite-volume step (alsfvm) and of the mean/variance statistics and
 * the uniform sample generator (alsuq).
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT CODE: only tests/, the smoke check and the
 * CPU-baseline leg of bench.py load this library, as the checker.
 *
 * Build with -ffp-contract=off and without fast-math: every expression below
 * keeps the reference's operand order so that results are bit-identical to the
 * reference compiled the same way, on x86-64 and on aarch64.
 * Parity is pinned against the reference itself (oracle/refbuild builds the
 * unmodified reference sources) and against the fixtures in tests/golden/. */
#include "fvoracle.h"

#include <math.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static __thread char g_err[512];

static int fail(int code, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
    return code;
}

const char* fv_last_error(void) { return g_err; }

/* Wall time of the last fv_run's step loop alone (initial data, allocation
 * and the final copy excluded), from the monotonic clock. */
static __thread double g_loop_seconds;

double fv_last_loop_seconds(void) { return g_loop_seconds; }

static double now_seconds(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

void fv_set_threads(int n) {
#ifdef _OPENMP
    omp_set_num_threads(n > 0 ? n : 1);
#else
    (void)n;
#endif
}

int fv_get_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------ names */

enum { EQ_BURGERS = 0, EQ_EULER1 = 1, EQ_EULER2 = 2, EQ_EULER3 = 3 };
enum { FL_HLL, FL_HLL3, FL_GODUNOV, FL_CENTRAL, FL_RUSANOV, FL_ROE };
enum { RC_NONE, RC_WENO2, RC_ENO2, RC_ENO3, RC_ENO4, RC_MC, RC_MM, RC_WENOF2 };
enum { IN_FE, IN_RK2, IN_RK3 };
enum { BC_NEUMANN, BC_PERIODIC };

static int parse_eq(const char* s) {
    if (!strcmp(s, "burgers")) return EQ_BURGERS;
    if (!strcmp(s, "euler1")) return EQ_EULER1;
    if (!strcmp(s, "euler2")) return EQ_EULER2;
    if (!strcmp(s, "euler3")) return EQ_EULER3;
    return -1;
}
static int parse_flux(const char* s) {
    if (!strcmp(s, "hll")) return FL_HLL;
    if (!strcmp(s, "hll3")) return FL_HLL3;
    if (!strcmp(s, "godunov")) return FL_GODUNOV;
    if (!strcmp(s, "central")) return FL_CENTRAL;
    if (!strcmp(s, "rusanov")) return FL_RUSANOV;
    if (!strcmp(s, "roe")) return FL_ROE;
    return -1;
}
static int parse_recon(const char* s) {
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
static int parse_integrator(const char* s) {
    if (!strcmp(s, "forwardeuler")) return IN_FE;
    if (!strcmp(s, "rungekutta2")) return IN_RK2;
    if (!strcmp(s, "rungekutta3")) return IN_RK3;
    return -1;
}
static int parse_bc(const char* s) {
    if (!strcmp(s, "neumann")) return BC_NEUMANN;
    if (!strcmp(s, "periodic")) return BC_PERIODIC;
    return -1;
}

/* Reconstruction ghost width: none 1, weno2 2, enoK K
 * (alsfvm/src/reconstruction/NoReconstruction.cpp:71-73, WENO2.hpp:93-95,
 * ENOCPU.cpp:180-183); the two-point flux stencil needs 1. */
/* numerical_flux_list.hpp:41-113: Euler takes hll, hll3, central; Burgers
 * takes godunov, central, rusanov, roe */
static int flux_applies(int eq, int fl) {
    if (eq == EQ_BURGERS) return fl == FL_GODUNOV || fl == FL_CENTRAL || fl == FL_RUSANOV || fl == FL_ROE;
    return fl == FL_HLL || fl == FL_HLL3 || fl == FL_CENTRAL;
}

static int recon_ghosts(int rc) {
    switch (rc) {
        case RC_NONE: return 1;
        case RC_WENO2: return 2;
        case RC_ENO2: return 2;
        case RC_ENO3: return 3;
        case RC_ENO4: return 4;
        case RC_MC: return 2;
        case RC_MM: return 2;
        case RC_WENOF2: return 2;
    }
    return -1;
}

int fv_ghost_cells(const char* recon) {
    int rc = parse_recon(recon);
    if (rc < 0) return fail(-1, "unknown reconstruction %s", recon);
    return recon_ghosts(rc);
}

/* ------------------------------------------------------------------ grid */

typedef struct {
    int eq, nsd, nvar, dim;
    int n[3], g[3], t[3];
    long total;
    double gamma;
} grid_t;

static int nvar_of(int eq) { return eq == EQ_BURGERS ? 1 : eq + 2; }

/* Ghost cells exist only in active dimensions (alsfvm/src/volume/Volume.cpp:52-53). */
static void make_grid(grid_t* G, int eq, const int n[3], int ghosts, double gamma) {
    G->eq = eq;
    G->nsd = eq == EQ_BURGERS ? 1 : eq;
    G->nvar = nvar_of(eq);
    G->dim = n[2] > 1 ? 3 : (n[1] > 1 ? 2 : 1);
    for (int d = 0; d < 3; ++d) {
        G->n[d] = n[d];
        G->g[d] = d < G->dim ? ghosts : 0;
        G->t[d] = n[d] + 2 * G->g[d];
    }
    G->total = (long)G->t[0] * G->t[1] * G->t[2];
    G->gamma = gamma;
}

static inline long IDX(const grid_t* G, long x, long y, long z) {
    return (z * G->t[1] + y) * G->t[0] + x;
}

/* ------------------------------------------------------------- equations */

typedef struct {
    double rho, m[3], E, p, u[3];
} euler_all;

/* Euler<nsd>::computeExtra: ie = E - 0.5 m.m / rho; u = m / rho;
 * p = (gamma - 1) ie (alsfvm/include/alsfvm/equation/euler/Euler.hpp:204-211). */
static inline void euler_fetch(euler_all* a, const double* U, long total, long i, int nsd,
                               double gamma) {
    a->rho = U[i];
    for (int k = 0; k < nsd; ++k) a->m[k] = U[(1 + k) * total + i];
    a->E = U[(1 + nsd) * total + i];
    double dot = a->m[0] * a->m[0]; /* nsd >= 1 */
    for (int k = 1; k < nsd; ++k) dot = dot + a->m[k] * a->m[k];
    const double ie = a->E - 0.5 * dot / a->rho;
    for (int k = 0; k < nsd; ++k) a->u[k] = a->m[k] / a->rho;
    a->p = (gamma - 1) * ie;
}

/* Euler<nsd>::computePointFlux (Euler.hpp:172-181). F has nsd+2 entries. */
static inline void euler_point_flux(const euler_all* a, int d, int nsd, double* F) {
    F[0] = a->m[d];
    for (int k = 0; k < nsd; ++k) F[1 + k] = a->u[d] * a->m[k];
    F[1 + d] += a->p;
    F[1 + nsd] = (a->E + a->p) * a->u[d];
}

static inline void euler_conserved(const euler_all* a, int nsd, double* c) {
    c[0] = a->rho;
    for (int k = 0; k < nsd; ++k) c[1 + k] = a->m[k];
    c[1 + nsd] = a->E;
}

/* HLL3<nsd>::computeFlux + computeHLLSpeeds
 * (alsfvm/include/alsfvm/numflux/euler/HLL3.hpp:52-148). */
static double flux_hll3(const euler_all* L, const euler_all* R, int d, int nsd, double gamma,
                        double* F) {
    const double waveLeft = sqrt(L->rho);
    const double waveRight = sqrt(R->rho);
    const double rho = (L->rho + R->rho) / 2;
    const double ud = (waveLeft * L->u[d] + waveRight * R->u[d]) / (waveLeft + waveRight);
    const double p = (waveLeft * L->p + waveRight * R->p) / (waveLeft + waveRight);
    const double cfLeft = sqrt(gamma * L->p / L->rho);
    const double cfRight = sqrt(gamma * R->p / R->rho);
    const double correct = 0.5 * fmax(0.0, L->u[d] - R->u[d]);
    const double cs = sqrt(gamma * p / rho);
    const double speedLeft = fmin(L->u[d] + correct - cfLeft, ud - cs);
    const double speedRight = fmax(R->u[d] - correct + cfRight, ud + cs);

    double fluxLeft[5], fluxRight[5];
    euler_point_flux(L, d, nsd, fluxLeft);
    euler_point_flux(R, d, nsd, fluxRight);
    const double pressureLeft = L->p, pressureRight = R->p;
    const double udl = L->u[d] - speedLeft;
    const double udr = R->u[d] - speedRight;
    const double aa = udr * R->rho - udl * L->rho;
    const double sm = (R->m[d] * udr - L->m[d] * udl + pressureRight - pressureLeft) / aa;
    double us[3];
    for (int k = 0; k < nsd; ++k)
        us[k] = (fluxRight[1 + k] - fluxLeft[1 + k] - speedRight * R->m[k] + speedLeft * L->m[k]) / aa;
    us[d] = sm;
    const int nv = nsd + 2;
    if (speedLeft == 0) {
        for (int k = 0; k < nv; ++k) F[k] = 0;
    } else if (speedLeft > 0) {
        for (int k = 0; k < nv; ++k) F[k] = fluxLeft[k];
    } else if (speedRight < 0) {
        for (int k = 0; k < nv; ++k) F[k] = fluxRight[k];
    } else if (sm >= 0) {
        double mid[5], c[5];
        mid[0] = L->rho * udl / (sm - speedLeft);
        for (int k = 0; k < nsd; ++k) mid[1 + k] = mid[0] * us[k];
        const double pp = pressureLeft + L->rho * (L->u[d] - sm) * udl;
        mid[1 + nsd] = (udl * L->E + pressureLeft * L->u[d] - pp * sm) / (sm - speedLeft);
        euler_conserved(L, nsd, c);
        for (int k = 0; k < nv; ++k) F[k] = fluxLeft[k] + speedLeft * (mid[k] - c[k]);
    } else {
        double mid[5], c[5];
        mid[0] = R->rho * udr / (sm - speedRight);
        for (int k = 0; k < nsd; ++k) mid[1 + k] = mid[0] * us[k];
        const double pp = pressureRight + R->rho * (R->u[d] - sm) * udr;
        mid[1 + nsd] = (udr * R->E + pressureRight * R->u[d] - pp * sm) / (sm - speedRight);
        euler_conserved(R, nsd, c);
        for (int k = 0; k < nv; ++k) F[k] = fluxRight[k] + speedRight * (mid[k] - c[k]);
    }
    return fmax(fabs(speedLeft), fabs(speedRight));
}

/* HLL<nsd>::computeFlux + computeHLLSpeeds
 * (alsfvm/include/alsfvm/numflux/euler/HLL.hpp:51-115). */
static double flux_hll(const euler_all* L, const euler_all* R, int d, int nsd, double gamma,
                       double* F) {
    const double waveLeft = sqrt(L->rho);
    const double waveRight = sqrt(R->rho);
    const double rho = (L->rho + R->rho) / 2;
    const double ud = (waveLeft * L->u[d] + waveRight * R->u[d]) / (waveLeft + waveRight);
    const double p = (L->p * waveLeft + R->p * waveRight) / (waveLeft + waveRight);
    const double cs = sqrt(gamma * p / rho);
    const double speedLeft = fmin(L->u[d] - sqrt(gamma * L->p / L->rho), ud - cs);
    const double speedRight = fmax(R->u[d] + sqrt(gamma * R->p / R->rho), ud + cs);
    const int nv = nsd + 2;
    if (speedLeft == 0) {
        for (int k = 0; k < nv; ++k) F[k] = 0;
    } else if (speedLeft > 0) {
        euler_point_flux(L, d, nsd, F);
    } else if (speedRight < 0) {
        euler_point_flux(R, d, nsd, F);
    } else {
        double fl[5], fr[5], cl[5], cr[5];
        euler_point_flux(L, d, nsd, fl);
        euler_point_flux(R, d, nsd, fr);
        euler_conserved(L, nsd, cl);
        euler_conserved(R, nsd, cr);
        for (int k = 0; k < nv; ++k)
            F[k] = (speedRight * fl[k] - speedLeft * fr[k] + speedRight * speedLeft * (cr[k] - cl[k])) /
                   (speedRight - speedLeft);
    }
    return fmax(fabs(speedLeft), fabs(speedRight));
}

/* burgers::Godunov: F = max(f(max(uL,0)), f(min(uR,0))), f(u) = u*u/2; wave
 * speed max(|uL|,|uR|) (alsfvm/include/alsfvm/numflux/burgers/Godunov.hpp:40-60,
 * alsfvm/include/alsfvm/equation/burgers/Burgers.hpp:135-139). */
static double flux_godunov(double uL, double uR, double* F) {
    const double a = fmax(uL, 0.0);
    const double b = fmin(uR, 0.0);
    const double fl = a * a / 2;
    const double fr = b * b / 2;
    F[0] = fmax(fl, fr);
    return fmax(fabs(uL), fabs(uR));
}

/* Central<Euler<nsd>>: F = 0.5 (f(L) + f(R)); wave speed max over the two
 * states of |u_d| + sqrt(gamma p / rho) (alsfvm/include/alsfvm/numflux/
 * Central.hpp:31-55, Euler.hpp:251-258). */
static double flux_central_euler(const euler_all* L, const euler_all* R, int d, int nsd, double gamma,
                                 double* F) {
    double fl[5], fr[5];
    euler_point_flux(L, d, nsd, fl);
    euler_point_flux(R, d, nsd, fr);
    for (int k = 0; k < nsd + 2; ++k) F[k] = 0.5 * (fl[k] + fr[k]);
    const double wl = fabs(L->u[d]) + sqrt(gamma * L->p / L->rho);
    const double wr = fabs(R->u[d]) + sqrt(gamma * R->p / R->rho);
    return fmax(wl, wr);
}

/* Central<Burgers>, Rusanov<Burgers> (eigenvalue u: Burgers.hpp:298-301) and
 * burgers::Roe (alsfvm/include/alsfvm/numflux/Rusanov.hpp:31-59,
 * alsfvm/include/alsfvm/numflux/burgers/Roe.hpp:30-58); f(u) = u u / 2. */
static double flux_burgers(int fl, double uL, double uR, double* F) {
    const double fL = uL * uL / 2, fR = uR * uR / 2;
    if (fl == FL_CENTRAL) {
        F[0] = 0.5 * (fL + fR);
    } else if (fl == FL_RUSANOV) {
        const double eigenMax = fmax(fabs(uL), fabs(uR));
        F[0] = 0.5 * (fL + fR) - 0.5 * eigenMax * (uR - uL);
    } else {
        if (uL >= -uR) {
            const double a = fmax(uL, 0.0);
            F[0] = a * a / 2;
        } else {
            const double b = fmin(uR, 0.0);
            F[0] = b * b / 2;
        }
    }
    return fmax(fabs(uL), fabs(uR));
}

/* -------------------------------------------------------- reconstruction */

/* sign and minmod (alsfvm/include/alsfvm/reconstruction/sign.hpp,
 * minmod.hpp): sign is 1, 0 or -1 (-1 for NaN). */
static double sign_of(double a) { return a > 0 ? 1.0 : (a == 0 ? 0.0 : -1.0); }
static double minmod2(double a, double b) {
    return sign_of(a) == sign_of(b) ? sign_of(a) * fmin(fabs(a), fabs(b)) : 0.0;
}
static double minmod3(double a, double b, double c) {
    return (sign_of(a) == sign_of(b) && sign_of(b) == sign_of(c)) ? sign_of(a) * fmin(fabs(a), fmin(fabs(b), fabs(c)))
                                                                  : 0.0;
}

/* ENO reconstruction coefficients, row r gives the value at the cell's
 * left face for stencil shift r (row r+1 the right face); the standard
 * uniform-grid ENO table (alsfvm/src/reconstruction/ENOCoefficients.cpp:21-49). */
static const double ENO2C[3][2] = {{3.0 / 2.0, -1.0 / 2.0}, {1.0 / 2.0, 1.0 / 2.0}, {-1.0 / 2.0, 3.0 / 2.0}};
static const double ENO3C[4][3] = {{11.0 / 6.0, -7.0 / 6.0, 1.0 / 3.0},
                                   {1.0 / 3.0, 5.0 / 6.0, -1.0 / 6.0},
                                   {-1.0 / 6.0, 5.0 / 6.0, 1.0 / 3.0},
                                   {1.0 / 3.0, -7.0 / 6.0, 11.0 / 6.0}};
static const double ENO4C[5][4] = {{25.0 / 12.0, -23.0 / 12.0, 13.0 / 12.0, -1.0 / 4.0},
                                   {1.0 / 4.0, 13.0 / 12.0, -5.0 / 12.0, 1.0 / 12.0},
                                   {-1.0 / 12.0, 7.0 / 12.0, 7.0 / 12.0, -1.0 / 12.0},
                                   {1.0 / 12.0, -5.0 / 12.0, 13.0 / 12.0, 1.0 / 4.0},
                                   {-1.0 / 4.0, 13.0 / 12.0, -23.0 / 12.0, 25.0 / 12.0}};

#define WENO_EPSILON 1e-8 /* alsfvm/include/alsfvm/reconstruction/WENOCoefficients.hpp:21 */

/* Reconstructs cells [g-1, n-g+1) in the active direction and the interior in
 * the other directions (ReconstructionCPU.cpp:37-97, ENOCPU.cpp:41-171). The
 * weight / stencil-indicator variable is variable 0 (rho for Euler, u for
 * Burgers: Euler.hpp:286-288, Burgers.hpp:225-227). */
/* WENOF2<Euler<nsd>>::reconstruct (alsfvm/include/alsfvm/reconstruction/
 * WENOF2.hpp:31-112): WENO2 weights from rho, applied to the primitive
 * variables (rho, u, p); the rho and p increments bounded by 1.9 times the
 * cell's value; the increment scaled by aijk = sqrt(R / max(R, LL)) / 2 with
 * R = p / (gamma - 1) and LL a kinetic-energy bound; back to conserved
 * variables with Euler::computeConserved (Euler.hpp:236-245). Vector dot
 * products accumulate x, y, z in order. */
typedef struct { double rho, u[3], p; } prim_t;

static prim_t to_prim(const double* U, long total, long i, int nsd, double gamma) {
    prim_t q;
    const double rho = U[i];
    double m[3], dot = 0;
    for (int k = 0; k < nsd; ++k) m[k] = U[(1 + k) * total + i];
    for (int k = 0; k < nsd; ++k) q.u[k] = m[k] / rho;
    dot = m[0] * m[0];
    for (int k = 1; k < nsd; ++k) dot = dot + m[k] * m[k];
    const double ie = U[(1 + nsd) * total + i] - 0.5 * dot / rho;
    q.rho = rho;
    q.p = (gamma - 1) * ie;
    return q;
}

static double dot_n(const double* a, const double* b, int nsd) {
    double d = a[0] * b[0];
    for (int k = 1; k < nsd; ++k) d = d + a[k] * b[k];
    return d;
}

static void wenof2_side(const prim_t* L, const prim_t* M, const prim_t* R, double w0, double w1, int sgn, int nsd,
                        double gamma, double* out) {
    const double BOUND = 1.9;
    prim_t d;
    d.rho = w1 * (M->rho - L->rho) + w0 * (R->rho - M->rho);
    for (int k = 0; k < nsd; ++k) d.u[k] = w1 * (M->u[k] - L->u[k]) + w0 * (R->u[k] - M->u[k]);
    d.p = w1 * (M->p - L->p) + w0 * (R->p - M->p);
    d.rho = fmax(-BOUND * M->rho, fmin(BOUND * M->rho, d.rho));
    d.p = fmax(-BOUND * M->p, fmin(BOUND * M->p, d.p));
    const double dd = dot_n(d.u, d.u, nsd);
    const double LL = 0.125 * M->rho * dd - 0.5 * fmin(0.0, d.rho * dot_n(M->u, d.u, nsd)) +
                      0.5 * d.rho * d.rho * dd / M->rho;
    const double Rr = M->p / (gamma - 1);
    const double a = 0.5 * sqrt(Rr / fmax(Rr, LL));
    prim_t q;
    if (sgn < 0) {
        q.rho = M->rho - a * d.rho;
        for (int k = 0; k < nsd; ++k) q.u[k] = M->u[k] - a * d.u[k];
        q.p = M->p - a * d.p;
    } else {
        q.rho = M->rho + a * d.rho;
        for (int k = 0; k < nsd; ++k) q.u[k] = M->u[k] + a * d.u[k];
        q.p = M->p + a * d.p;
    }
    out[0] = q.rho;
    for (int k = 0; k < nsd; ++k) out[1 + k] = q.rho * q.u[k];
    out[1 + nsd] = q.p / (gamma - 1) + 0.5 * q.rho * dot_n(q.u, q.u, nsd);
}

static void wenof2_cell(const grid_t* G, const double* U, long i, long stride, double* left, double* right) {
    const long total = G->total;
    const int nsd = G->nsd;
    const long il = i - stride, ir = i + stride;
    const double i0 = U[i];
    const double b0 = (U[ir] - i0) * (U[ir] - i0);
    const double b1 = (i0 - U[il]) * (i0 - U[il]);
    const double a0Left = 1 / (3 * (WENO_EPSILON + b0) * (WENO_EPSILON + b0));
    const double a1Left = 2 / (3 * (WENO_EPSILON + b1) * (WENO_EPSILON + b1));
    const double w0Left = a0Left / (a0Left + a1Left);
    const double w1Left = a1Left / (a0Left + a1Left);
    const double a0Right = 2 / (3 * (WENO_EPSILON + b0) * (WENO_EPSILON + b0));
    const double a1Right = 1 / (3 * (WENO_EPSILON + b1) * (WENO_EPSILON + b1));
    const double w0Right = a0Right / (a0Right + a1Right);
    const double w1Right = a1Right / (a0Right + a1Right);
    const prim_t L = to_prim(U, total, il, nsd, G->gamma);
    const prim_t M = to_prim(U, total, i, nsd, G->gamma);
    const prim_t R = to_prim(U, total, ir, nsd, G->gamma);
    double l[5], r[5];
    wenof2_side(&L, &M, &R, w0Left, w1Left, -1, nsd, G->gamma, l);
    wenof2_side(&L, &M, &R, w0Right, w1Right, +1, nsd, G->gamma, r);
    for (int v = 0; v < nsd + 2; ++v) {
        left[v * total + i] = l[v];
        right[v * total + i] = r[v];
    }
}

static void reconstruct(const grid_t* G, int rc, int dir, const double* U, double* left,
                        double* right) {
    const long total = G->total;
    const int nvar = G->nvar;
    const int dx = dir == 0, dy = dir == 1, dz = dir == 2;
    const long stride = dir == 0 ? 1 : (dir == 1 ? G->t[0] : (long)G->t[0] * G->t[1]);
    const int ng = recon_ghosts(rc);
    int lo[3], hi[3];
    for (int d = 0; d < 3; ++d) {
        const int act = d == dir;
        lo[d] = G->g[d] - act;
        hi[d] = G->t[d] - G->g[d] + act;
    }
    (void)ng;
    if (rc == RC_NONE) {
        /* NoReconstruction copies every cell (NoReconstruction.cpp:52-64). */
        for (int v = 0; v < nvar; ++v) {
            memcpy(left + v * total, U + v * total, total * sizeof(double));
            memcpy(right + v * total, U + v * total, total * sizeof(double));
        }
        return;
    }
    (void)dx; (void)dy; (void)dz;
    for (int z = lo[2]; z < hi[2]; ++z) {
#pragma omp parallel for schedule(static)
        for (int y = lo[1]; y < hi[1]; ++y) {
            for (int x = lo[0]; x < hi[0]; ++x) {
                const long i = IDX(G, x, y, z);
                if (rc == RC_WENOF2) {
                    wenof2_cell(G, U, i, stride, left, right);
                } else if (rc == RC_MC || rc == RC_MM) {
                    /* MC / MM slope limiters on every variable
                     * (alsfvm/include/alsfvm/reconstruction/MC.hpp:27-52, MM.hpp:25-47) */
                    for (int v = 0; v < nvar; ++v) {
                        const double* u = U + v * total;
                        const double l = u[i - stride], m = u[i], r = u[i + stride];
                        const double sigma = rc == RC_MC ? minmod3(2 * (r - m), (r - l) / 2, 2 * (m - l))
                                                         : minmod2(r - m, m - l);
                        left[v * total + i] = m - sigma / 2;
                        right[v * total + i] = m + sigma / 2;
                    }
                } else if (rc == RC_WENO2) {
                    /* WENO2::reconstruct (alsfvm/include/alsfvm/reconstruction/WENO2.hpp:31-91) */
                    const long il = i - stride, ir = i + stride;
                    const double i0 = U[i];
                    const double d0 = U[ir] - i0;
                    const double d1 = i0 - U[il];
                    const double b0 = d0 * d0;
                    const double b1 = d1 * d1;
                    const double a0Left = 1 / (3 * (WENO_EPSILON + b0) * (WENO_EPSILON + b0));
                    const double a1Left = 2 / (3 * (WENO_EPSILON + b1) * (WENO_EPSILON + b1));
                    const double w0Left = a0Left / (a0Left + a1Left);
                    const double w1Left = a1Left / (a0Left + a1Left);
                    const double a0Right = 2 / (3 * (WENO_EPSILON + b0) * (WENO_EPSILON + b0));
                    const double a1Right = 1 / (3 * (WENO_EPSILON + b1) * (WENO_EPSILON + b1));
                    const double w0Right = a0Right / (a0Right + a1Right);
                    const double w1Right = a1Right / (a0Right + a1Right);
                    for (int v = 0; v < nvar; ++v) {
                        const double* u = U + v * total;
                        left[v * total + i] =
                            0.5 * (w1Left * u[il] + (3 * w0Left + w1Left) * u[i] - w0Left * u[ir]);
                        right[v * total + i] =
                            0.5 * (w0Right * u[ir] + (3 * w1Right + w0Right) * u[i] - w1Right * u[il]);
                    }
                } else {
                    /* ENOCPU<order>::performReconstruction: undivided differences of
                     * variable 0 up to order-1 levels; at each level the shift grows
                     * when |left difference| < |right difference|. */
                    const int order = rc == RC_ENO2 ? 2 : (rc == RC_ENO3 ? 3 : 4);
                    double w[9];
                    for (int k = -(order - 1); k <= order - 1; ++k) w[k + order - 1] = U[i + k * stride];
                    /* dd[level][j] for j = offset - (order-1) .. covering cells i-1, i */
                    double dd[3][9];
                    const int c = order - 1; /* position of cell i in w[] */
                    for (int j = 0; j + 1 < 2 * order - 1; ++j) dd[0][j] = w[j + 1] - w[j];
                    for (int l = 1; l < order - 1; ++l)
                        for (int j = 0; j + 1 + l < 2 * order - 1; ++j) dd[l][j] = dd[l - 1][j + 1] - dd[l - 1][j];
                    int shift = 0;
                    for (int l = 0; l < order - 1; ++l) {
                        const double ddRight = dd[l][c];
                        const double ddLeft = dd[l][c - 1];
                        if (fabs(ddLeft) < fabs(ddRight)) shift++;
                    }
                    const double* cL;
                    const double* cR;
                    if (order == 2) { cL = ENO2C[shift]; cR = ENO2C[shift + 1]; }
                    else if (order == 3) { cL = ENO3C[shift]; cR = ENO3C[shift + 1]; }
                    else { cL = ENO4C[shift]; cR = ENO4C[shift + 1]; }
                    for (int v = 0; v < nvar; ++v) {
                        const double* u = U + v * total;
                        double leftValue = 0.0, rightValue = 0.0;
                        for (int j = 0; j < order; ++j) {
                            const double value = u[i - (long)(shift - j) * stride];
                            leftValue += cL[j] * value;
                            rightValue += cR[j] * value;
                        }
                        left[v * total + i] = leftValue;
                        right[v * total + i] = rightValue;
                    }
                }
            }
        }
    }
}

int fv_reconstruct(const char* equation, const char* recon, const int n[3], double gamma,
                   int direction, const double* U, double* left, double* right) {
    const int eq = parse_eq(equation), rc = parse_recon(recon);
    if (eq < 0 || rc < 0) return fail(-1, "bad equation/reconstruction");
    grid_t G;
    make_grid(&G, eq, n, recon_ghosts(rc), gamma);
    if (direction < 0 || direction >= G.dim) return fail(-1, "bad direction %d", direction);
    reconstruct(&G, rc, direction, U, left, right);
    return 0;
}

/* -------------------------------------------------------------- net flux */

/* computeNetFlux<Flux, Equation, direction> (alsfvm/src/numflux/NumericalFluxCPU.cpp:
 * 32-118): face x between cells x and x+1 for x in [ng-1, n-ng) stores -F into
 * temp; then out[x+1] += temp[x+1] + (-temp[x]). Returns the maximum face speed. */
static double net_flux(const grid_t* G, int fl, int dir, const double* left, const double* right,
                       double* out, double* temp) {
    const long total = G->total;
    const int nvar = G->nvar, nsd = G->nsd;
    const long stride = dir == 0 ? 1 : (dir == 1 ? G->t[0] : (long)G->t[0] * G->t[1]);
    int lo[3], hi[3];
    for (int d = 0; d < 3; ++d) {
        const int act = d == dir;
        lo[d] = G->g[d] - act;
        hi[d] = G->t[d] - G->g[d];
    }
    double ws = 0;
    for (int z = lo[2]; z < hi[2]; ++z) {
        double wsz = 0;
#pragma omp parallel for schedule(static) reduction(max : wsz)
        for (int y = lo[1]; y < hi[1]; ++y) {
            for (int x = lo[0]; x < hi[0]; ++x) {
                const long i = IDX(G, x, y, z);
                double F[5];
                double wl;
                if (G->eq == EQ_BURGERS) {
                    wl = fl == FL_GODUNOV ? flux_godunov(right[i], left[i + stride], F)
                                          : flux_burgers(fl, right[i], left[i + stride], F);
                } else {
                    euler_all A, B;
                    euler_fetch(&A, right, total, i, nsd, G->gamma);
                    euler_fetch(&B, left, total, i + stride, nsd, G->gamma);
                    wl = fl == FL_HLL3 ? flux_hll3(&A, &B, dir, nsd, G->gamma, F)
                         : fl == FL_HLL ? flux_hll(&A, &B, dir, nsd, G->gamma, F)
                                        : flux_central_euler(&A, &B, dir, nsd, G->gamma, F);
                }
                for (int v = 0; v < nvar; ++v) temp[v * total + i] = (-1.0) * F[v];
                wsz = (wsz < wl) ? wl : wsz; /* std::max */
            }
        }
        ws = (ws < wsz) ? wsz : ws;
    }
    for (int d = 0; d < 3; ++d) hi[d] -= d == dir;
    for (int z = lo[2]; z < hi[2]; ++z) {
#pragma omp parallel for schedule(static)
        for (int y = lo[1]; y < hi[1]; ++y) {
            for (int x = lo[0]; x < hi[0]; ++x) {
                const long i = IDX(G, x, y, z);
                for (int v = 0; v < nvar; ++v) {
                    const double fmr = temp[v * total + i + stride];
                    const double flm = (-1.0) * temp[v * total + i];
                    out[v * total + i + stride] += fmr + flm;
                }
            }
        }
    }
    return ws;
}

typedef struct {
    grid_t G;
    int fl, rc;
    double *left, *right, *temp;
} flux_ctx;

static int flux_ctx_init(flux_ctx* c, int eq, int fl, int rc, const int n[3], double gamma) {
    make_grid(&c->G, eq, n, recon_ghosts(rc), gamma);
    c->fl = fl;
    c->rc = rc;
    const size_t bytes = (size_t)c->G.nvar * c->G.total * sizeof(double);
    c->left = (double*)calloc(1, bytes);
    c->right = (double*)calloc(1, bytes);
    c->temp = (double*)calloc(1, bytes);
    if (!c->left || !c->right || !c->temp) return fail(-3, "out of host memory");
    return 0;
}

static void flux_ctx_free(flux_ctx* c) {
    free(c->left);
    free(c->right);
    free(c->temp);
}

/* NumericalFluxCPU::computeFlux over the whole domain (makeZero, then per
 * direction reconstruct + net flux; alsfvm/src/numflux/NumericalFluxCPU.cpp:
 * 170-221). ConservedSystem's interior + side-strip calls cover the same faces
 * and cells, so the result equals a single whole-domain call. */
static void compute_flux(flux_ctx* c, const double* U, double* out, double ws[3]) {
    const grid_t* G = &c->G;
    const long total = G->total;
    for (int z = G->g[2]; z < G->t[2] - G->g[2]; ++z) {
#pragma omp parallel for schedule(static)
        for (int y = G->g[1]; y < G->t[1] - G->g[1]; ++y)
            for (int x = G->g[0]; x < G->t[0] - G->g[0]; ++x)
                for (int v = 0; v < G->nvar; ++v) out[v * total + IDX(G, x, y, z)] = 0;
    }
    ws[0] = ws[1] = ws[2] = 0;
    for (int d = 0; d < G->dim; ++d) {
        reconstruct(G, c->rc, d, U, c->left, c->right);
        ws[d] = net_flux(G, c->fl, d, c->left, c->right, out, c->temp);
    }
}

int fv_compute_flux(const char* equation, const char* flux, const char* recon, const int n[3],
                    double gamma, const double* U, double* out, double ws[3]) {
    const int eq = parse_eq(equation), fl = parse_flux(flux), rc = parse_recon(recon);
    if (eq < 0 || fl < 0 || rc < 0) return fail(-1, "bad equation/flux/reconstruction");
    if (!flux_applies(eq, fl)) return fail(-1, "flux %s not for %s", flux, equation);
    flux_ctx c;
    int r = flux_ctx_init(&c, eq, fl, rc, n, gamma);
    if (r == 0) compute_flux(&c, U, out, ws);
    flux_ctx_free(&c);
    return r;
}

/* -------------------------------------------------------------- boundary */

/* BoundaryCPU<Neumann|Periodic>::applyBoundaryConditions
 * (alsfvm/src/boundary/BoundaryCPU.cpp:30-106): per variable, per dimension,
 * bottom then top side, over every cell of the other dimensions (ghosts
 * included). Neumann ghost k copies interior k-1 from the edge (a mirror,
 * Neumann.hpp:24-35); periodic copies from the opposite side (Periodic.hpp:24-42). */
static void apply_boundary(const grid_t* G, int bc, double* U) {
    const long total = G->total;
    for (int v = 0; v < G->nvar; ++v) {
        double* u = U + v * total;
        for (int d = 0; d < G->dim; ++d) {
            const int ng = G->g[d];
            const long stride = d == 0 ? 1 : (d == 1 ? G->t[0] : (long)G->t[0] * G->t[1]);
            const int nint = G->t[d] - 2 * ng;
            for (int side = 0; side < 2; ++side) {
                const int sign = side == 1 ? -1 : 1;
                const int edge = side == 0 ? ng : G->t[d] - ng - 1;
                int lo[3] = {0, 0, 0}, hi[3] = {G->t[0], G->t[1], G->t[2]};
                lo[d] = edge;
                hi[d] = edge + 1;
                for (int z = lo[2]; z < hi[2]; ++z)
                    for (int y = lo[1]; y < hi[1]; ++y)
                        for (int x = lo[0]; x < hi[0]; ++x) {
                            const long i = IDX(G, x, y, z);
                            for (int k = 1; k <= ng; ++k) {
                                const long dst = i - (long)sign * k * stride;
                                const long src = bc == BC_NEUMANN ? i + (long)sign * (k - 1) * stride
                                                                  : i + (long)sign * (nint - k) * stride;
                                u[dst] = u[src];
                            }
                        }
            }
        }
    }
}

int fv_boundary(const char* boundary, const int n[3], int ghosts, int nvar, double* U) {
    const int bc = parse_bc(boundary);
    if (bc < 0) return fail(-1, "unknown boundary %s", boundary);
    grid_t G;
    make_grid(&G, nvar == 1 ? EQ_BURGERS : nvar - 2, n, ghosts, 1.4);
    for (int d = 0; d < G.dim; ++d)
        if (G.t[d] < 2 * ghosts) return fail(-1, "too few cells for the boundary");
    apply_boundary(&G, bc, U);
    return 0;
}

/* ----------------------------------------------------------- cell ops */

/* Euler<nsd>::computeConserved: m = rho u, E = p/(gamma-1) + 0.5 rho u.u
 * (Euler.hpp:236-245); Burgers copies u. Primitive order (rho, u..., p). */
int fv_prim_to_cons(const char* equation, const int n[3], int ghosts, double gamma,
                    const double* prim, double* cons) {
    const int eq = parse_eq(equation);
    if (eq < 0) return fail(-1, "unknown equation %s", equation);
    grid_t G;
    make_grid(&G, eq, n, ghosts, gamma);
    const long total = G.total;
    const int nsd = G.nsd;
    for (long i = 0; i < total; ++i) {
        if (eq == EQ_BURGERS) {
            cons[i] = prim[i];
            continue;
        }
        const double rho = prim[i];
        double u[3], dot;
        for (int k = 0; k < nsd; ++k) u[k] = prim[(1 + k) * total + i];
        const double p = prim[(1 + nsd) * total + i];
        dot = u[0] * u[0];
        for (int k = 1; k < nsd; ++k) dot = dot + u[k] * u[k];
        cons[i] = rho;
        for (int k = 0; k < nsd; ++k) cons[(1 + k) * total + i] = u[k] * rho;
        cons[(1 + nsd) * total + i] = p / (gamma - 1) + 0.5 * rho * dot;
    }
    return 0;
}

/* CPUCellComputer::obeysConstraints: every cell, ghosts included, has finite
 * conserved and extra variables, rho > 0 and p > 0 (Euler) or finite u
 * (Burgers) (alsfvm/src/equation/CPUCellComputer.cpp:79-125, Euler.hpp:269-277). */
static int obeys(const grid_t* G, const double* U) {
    const long total = G->total;
    int ok = 1;
#pragma omp parallel for schedule(static) reduction(&& : ok)
    for (long i = 0; i < total; ++i) {
        if (G->eq == EQ_BURGERS) {
            const double u = U[i];
            ok = ok && isfinite(u);
            continue;
        }
        euler_all a;
        euler_fetch(&a, U, total, i, G->nsd, G->gamma);
        int c = isfinite(a.rho) && isfinite(a.E) && isfinite(a.p);
        for (int k = 0; k < G->nsd; ++k) c = c && isfinite(a.m[k]) && isfinite(a.u[k]);
        c = c && a.rho > 0 && a.p > 0;
        ok = ok && c;
    }
    return ok;
}

int fv_obeys_constraints(const char* equation, const int n[3], int ghosts, double gamma,
                         const double* U) {
    const int eq = parse_eq(equation);
    if (eq < 0) return fail(-1, "unknown equation %s", equation);
    grid_t G;
    make_grid(&G, eq, n, ghosts, gamma);
    return obeys(&G, U);
}

/* ------------------------------------------------------------ simulation */

/* Simulator::performStep / incrementSolution (alsfvm/src/simulator/Simulator.cpp:
 * 81-85, 191-214) with RungeKutta3/RungeKutta2/ForwardEuler::performSubstep
 * (alsfvm/src/integrator/RungeKutta3.cpp:49-86, RungeKutta2.cpp:37-67,
 * ForwardEuler.cpp:32-51), Integrator::computeTimestep (Integrator.cpp:20-46),
 * the FixedIntervalWriter dt clamp (alsfvm/src/io/FixedIntervalWriter.cpp:
 * 45-53), Grid cell lengths (alsfvm/src/grid/Grid.cpp:24-42) and the
 * constraint check after every step. */
int fv_run(const char* equation, const char* flux, const char* recon, const char* integrator,
           const char* boundary, const int n[3], const double lower[3], const double upper[3],
           double gamma, double cfl, double end_time, int number_of_saves, int max_steps,
           const double* prim, double* out, double* t_out, int* steps_out, double* dts,
           int max_dts) {
    const int eq = parse_eq(equation), fl = parse_flux(flux), rc = parse_recon(recon);
    const int in = parse_integrator(integrator), bc = parse_bc(boundary);
    if (eq < 0 || fl < 0 || rc < 0 || in < 0 || bc < 0) return fail(-1, "bad configuration name");
    if (!flux_applies(eq, fl)) return fail(-1, "flux %s not for %s", flux, equation);
    flux_ctx c;
    int r = flux_ctx_init(&c, eq, fl, rc, n, gamma);
    if (r) { flux_ctx_free(&c); return r; }
    const grid_t* G = &c.G;
    const long total = G->total;
    const int nvar = G->nvar;
    const int nsub = in == IN_FE ? 1 : (in == IN_RK2 ? 2 : 3);
    double* U[4];
    double* primPad = (double*)calloc((size_t)nvar * total, sizeof(double));
    for (int s = 0; s <= nsub; ++s) U[s] = (double*)calloc((size_t)nvar * total, sizeof(double));

    /* initial data: interior primitives -> padded primitive volume -> conserved
     * over every cell (CPUCellComputer::computeFromPrimitive, CPUCellComputer.cpp:
     * 127-140), then the boundary (Simulator.cpp:117-162). */
    const long cells = (long)n[0] * n[1] * n[2];
    for (int v = 0; v < nvar; ++v)
        for (int z = 0; z < n[2]; ++z)
            for (int y = 0; y < n[1]; ++y)
                for (int x = 0; x < n[0]; ++x)
                    primPad[v * total + IDX(G, x + G->g[0], y + G->g[1], z + G->g[2])] =
                        prim[v * cells + ((long)z * n[1] + y) * n[0] + x];
    int gh = G->g[0];
    fv_prim_to_cons(equation, n, gh, gamma, primPad, U[0]);
    apply_boundary(G, bc, U[0]);

    double cellLengths[3];
    for (int d = 0; d < 3; ++d) cellLengths[d] = (upper[d] - lower[d]) / n[d];
    if (n[1] == 1) cellLengths[1] = 1;
    if (n[2] == 1) cellLengths[2] = 1;

    const double timeInterval = number_of_saves > 0 ? end_time / number_of_saves : 0;
    long numberSaved = 1;
    double t = 0;
    int steps = 0;
    const double loop_start = now_seconds();
    while (!(t >= end_time) && (max_steps <= 0 || steps < max_steps)) {
        double dt = 0;
        for (int s = 0; s < nsub; ++s) {
            double* o = U[s + 1];
            double ws[3];
            compute_flux(&c, U[s], o, ws);
            if (s == 0) {
                double waveSpeedTotal = 0;
                for (int d = 0; d < 3; ++d) {
                    if (cellLengths[d] == 0) continue;
                    waveSpeedTotal += ws[d] / cellLengths[d];
                }
                dt = cfl / waveSpeedTotal;
                if (number_of_saves > 0) {
                    const double nextSaveTime = numberSaved * timeInterval + 0.0;
                    const double lim = nextSaveTime - t;
                    dt = lim < dt ? lim : dt;
                }
            }
            const double scale = dt / cellLengths[0];
            const double* us = U[s];
            const double* u0 = U[0];
#pragma omp parallel for schedule(static)
            for (long i = 0; i < (long)nvar * total; ++i) {
                double v = o[i];
                v *= scale;
                v += us[i];
                if (in == IN_RK3) {
                    if (s == 1) {
                        v *= 1. / 3.;
                        v += u0[i];
                        v *= 3. / 4.;
                    } else if (s == 2) {
                        v *= 2;
                        v += u0[i];
                        v *= 1. / 3.;
                    }
                } else if (in == IN_RK2 && s == 1) {
                    v += u0[i];
                    v *= 0.5;
                }
                o[i] = v;
            }
            apply_boundary(G, bc, o);
        }
        double* tmp = U[0];
        U[0] = U[nsub];
        U[nsub] = tmp;
        t += dt;
        if (dts && steps < max_dts) dts[steps] = dt;
        ++steps;
        if (!obeys(G, U[0])) {
            r = fail(-2, "Simulation state does not obey constraints! At time %.17g, number of timesteps performed %d",
                     t, steps);
            break;
        }
        if (number_of_saves > 0 && t >= numberSaved * timeInterval + 0.0) numberSaved++;
    }
    g_loop_seconds = now_seconds() - loop_start;
    memcpy(out, U[0], (size_t)nvar * total * sizeof(double));
    *t_out = t;
    *steps_out = steps;
    for (int s = 0; s <= nsub; ++s) free(U[s]);
    free(primPad);
    flux_ctx_free(&c);
    return r;
}

/* ---------------------------------------------------------- generator */

/* 64-bit Mersenne Twister, MT19937-64 (Matsumoto and Nishimura; the
 * parameters of std::mt19937_64), default seed 5489. */
typedef struct {
    uint64_t mt[312];
    int mti;
} mt64;

static void mt64_seed(mt64* g, uint64_t seed) {
    g->mt[0] = seed;
    for (int i = 1; i < 312; ++i)
        g->mt[i] = 6364136223846793005ULL * (g->mt[i - 1] ^ (g->mt[i - 1] >> 62)) + (uint64_t)i;
    g->mti = 312;
}

static uint64_t mt64_next(mt64* g) {
    const uint64_t UM = 0xFFFFFFFF80000000ULL, LM = 0x7FFFFFFFULL;
    const uint64_t A = 0xB5026F5AA96619E9ULL;
    if (g->mti >= 312) {
        for (int i = 0; i < 312; ++i) {
            const uint64_t x = (g->mt[i] & UM) | (g->mt[(i + 1) % 312] & LM);
            g->mt[i] = g->mt[(i + 156) % 312] ^ (x >> 1) ^ ((x & 1ULL) ? A : 0ULL);
        }
        g->mti = 0;
    }
    uint64_t x = g->mt[g->mti++];
    x ^= (x >> 29) & 0x5555555555555555ULL;
    x ^= (x << 17) & 0x71D67FFFEDA60000ULL;
    x ^= (x << 37) & 0xFFF7EEE000000000ULL;
    x ^= x >> 43;
    return x;
}

/* std::uniform_real_distribution<double>(0,1) over a 64-bit engine uses one
 * draw: double(x) / 2^64, and nextafter(1,0) if that rounds to 1 (libstdc++
 * generate_canonical). Uniform::scale maps it to x (b - a) + a
 * (alsuq/src/distribution/Uniform.cpp:27-34). Draw number sample*dimension +
 * component of the default-seeded engine, as STLMersenne fast-forwards
 * (alsuq/src/generator/STLMersenne.cpp:38-85). */
int fv_uniform(int dimension, int sample, double lower, double upper, double* out) {
    if (dimension <= 0 || sample < 0) return fail(-1, "bad dimension/sample");
    mt64 g;
    mt64_seed(&g, 5489ULL);
    for (long k = 0; k < (long)sample * dimension; ++k) mt64_next(&g);
    for (int c = 0; c < dimension; ++c) {
        double r = (double)mt64_next(&g) / 18446744073709551616.0;
        if (r >= 1.0) r = nextafter(1.0, 0.0);
        const double x = r * (1.0 - 0.0) + 0.0;
        out[c] = x * (upper - lower) + lower;
    }
    return 0;
}

/* The Runner's parameter draws (alsuq/src/run/Runner.cpp:39-52) through the
 * process-wide engine of STLMersenne (alsuq/src/generator/STLMersenne.cpp:
 * 24-85): per sample (ascending from sample_start), per parameter in the
 * given order, per component: skip forward to draw sample * dim of that
 * parameter when the count of numbers produced is behind it, then to the
 * component within the block, draw one canonical double, scale it by
 * Uniform (alsuq/src/distribution/Uniform.cpp:27-34). One fresh engine per
 * call. */
int fv_generate_sequence(int nparams, const int* dims, const double* lowers, const double* uppers,
                         long long sample_start, long long nsamples, double* out) {
    if (nparams <= 0 || sample_start < 0 || nsamples < 0) return fail(-1, "bad arguments");
    for (int p = 0; p < nparams; ++p)
        if (dims[p] <= 0) return fail(-1, "bad dimension");
    mt64 g;
    mt64_seed(&g, 5489ULL);
    long long drawn = 0, k = 0;
    for (long long s = sample_start; s < sample_start + nsamples; ++s)
        for (int p = 0; p < nparams; ++p)
            for (int c = 0; c < dims[p]; ++c) {
                const long long dim = dims[p];
                if (drawn / dim < s) {
                    const long long skip = s * dim - drawn;
                    for (long long i = 0; i < skip; ++i) mt64_next(&g);
                    drawn += skip;
                }
                if (drawn % dim < c) {
                    const long long skip = c - drawn % dim;
                    for (long long i = 0; i < skip; ++i) mt64_next(&g);
                    drawn += skip;
                }
                drawn += 1;
                double r = (double)mt64_next(&g) / 18446744073709551616.0;
                if (r >= 1.0) r = nextafter(1.0, 0.0);
                out[k++] = r * (uppers[p] - lowers[p]) + lowers[p];
            }
    return 0;
}

/* ------------------------------------------------- structure functions */

/* |x|^p as the reference evaluates it: FastPower<p> (x * FastPower<p-1>(x))
 * for p = 1..5, pow otherwise (alsutils/include/alsutils/math/FastPower.hpp,
 * PowPower.hpp, dispatched in structure_common.hpp:156-180). */
static double structure_power(double x, double p, int ip) {
    switch (ip) {
        case 1: return x;
        case 2: return x * x;
        case 3: return x * (x * x);
        case 4: return x * (x * (x * x));
        case 5: return x * (x * (x * (x * x)));
        default: return pow(x, p);
    }
}

/* ValueAtBoundary<PERIODIC / NEUMANN> (alsfvm/include/alsfvm/boundary/
 * ValueAtBoundary.hpp): periodic wraps the interior position, Neumann clamps
 * it to the interior. */
static long structure_index(const grid_t* G, int periodic, int x, int y, int z) {
    const int n[3] = {G->n[0], G->n[1], G->n[2]};
    int q[3] = {x, y, z};
    for (int d = 0; d < 3; ++d) {
        if (periodic) {
            while (q[d] < 0) q[d] += n[d];
            q[d] = q[d] % n[d];
        } else {
            q[d] = q[d] < n[d] - 1 ? q[d] : n[d] - 1;
            q[d] = q[d] > 0 ? q[d] : 0;
        }
    }
    return IDX(G, q[0] + G->g[0], q[1] + G->g[1], q[2] + G->g[2]);
}

/* computeStructureCubeCPU (alsfvm/include/alsfvm/functional/
 * structure_common.hpp:37-154): for every variable, cell (k, j, i) and h in
 * 1 .. number_of_h - 1, out[h] += |u - u_h|^p / (nx ny nz) over the points
 * of the cube surface at distance h, visited per direction d and side in
 * the reference's loop bounds. */
int fv_structure_cube(const char* equation, const char* boundary, const int n[3], int ghosts, int number_of_h,
                      double p, const double* U, double* out) {
    const int eq = parse_eq(equation), bc = parse_bc(boundary);
    if (eq < 0 || bc < 0 || number_of_h < 1) return fail(-1, "bad arguments");
    grid_t G;
    make_grid(&G, eq, n, ghosts, 1.4);
    const int ip = (p == 1.0) ? 1 : (p == 2.0) ? 2 : (p == 3.0) ? 3 : (p == 4.0) ? 4 : (p == 5.0) ? 5 : 0;
    const int dims = G.dim, nx = n[0], ny = n[1], nz = n[2];
    const int periodic = bc == BC_PERIODIC;
    for (int v = 0; v < G.nvar; ++v) {
        const double* u = U + (long)v * G.total;
        double* o = out + (long)v * number_of_h;
        for (int h = 0; h < number_of_h; ++h) o[h] = 0.0;
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i)
                    for (int h = 1; h < number_of_h; ++h) {
                        const double uc = u[IDX(&G, i + G.g[0], j + G.g[1], k + G.g[2])];
                        for (int d = 0; d < dims; d++)
                            for (int side = 0; side < 2; side++) {
                                const int zDir = d == 2, yDir = d == 1, xDir = d == 0;
                                const int zStart = zDir ? (side == 0 ? k - h : k + h) : (dims > 2 ? k - h : 0);
                                const int zEnd = zDir ? (zStart + 1) : (dims > 2 ? k + h + 1 : 1);
                                const int yStart = yDir ? (side == 0 ? j - h : j + h)
                                                        : (dims == 2 ? j - h + 1 : (dims == 3 ? j - h + 1 : 0));
                                const int yEnd = yDir ? (yStart + 1) : (dims == 2 ? j + h : (dims == 3 ? j + h : 1));
                                int xStart = xDir ? (side == 0 ? i - h : i + h) : i - h;
                                int xEnd = xDir ? (xStart + 1) : i + h + 1;
                                if (zDir) {
                                    xStart += 1;
                                    xEnd -= 1;
                                }
                                for (int z = zStart; z < zEnd; z++)
                                    for (int y = yStart; y < yEnd; y++)
                                        for (int x = xStart; x < xEnd; x++) {
                                            const double uh = u[structure_index(&G, periodic, x, y, z)];
                                            o[h] += structure_power(fabs(uc - uh), p, ip) / (nx * ny * nz);
                                        }
                            }
                    }
    }
    return 0;
}

/* StructureBasic::computeStructure (alsuq/src/stats/StructureBasic.cpp:
 * 50-92): per variable, for every interior cell in the reference's loop
 * order and h = 0 .. H-1, out[h] += pow(|u(x) - u(x + h e_d)|, p) / (nx ny nz),
 * the shifted point through ValueAtBoundary (wrap or clamp). */
int fv_structure_basic(const char* equation, const char* boundary, const int n[3], int ghosts, int number_of_h,
                       double p, int direction, const double* U, double* out) {
    const int eq = parse_eq(equation), bc = parse_bc(boundary);
    if (eq < 0 || bc < 0 || number_of_h < 1) return fail(-1, "bad arguments");
    grid_t G;
    make_grid(&G, eq, n, ghosts, 1.4);
    if (direction < 0 || direction >= G.dim) return fail(-1, "bad direction");
    const int nx = n[0], ny = n[1], nz = n[2];
    const int periodic = bc == BC_PERIODIC;
    for (int v = 0; v < G.nvar; ++v) {
        const double* u = U + (long)v * G.total;
        double* o = out + (long)v * number_of_h;
        for (int h = 0; h < number_of_h; ++h) o[h] = 0.0;
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i)
                    for (int h = 0; h < number_of_h; ++h) {
                        const double uc = u[IDX(&G, i + G.g[0], j + G.g[1], k + G.g[2])];
                        const double uh = u[structure_index(&G, periodic, i + (direction == 0) * h,
                                                            j + (direction == 1) * h, k + (direction == 2) * h)];
                        o[h] += pow(fabs(uc - uh), p) / (nx * ny * nz);
                    }
    }
    return 0;
}

/* ---------------------------------------------------------- functionals */

enum { FN_IDENTITY, FN_MOMENT, FN_LEGENDRE, FN_LOG_ENTROPY, FN_BV, FN_BV_DIRECTION, FN_STRUCTURE_CUBE };

static int parse_functional(const char* s) {
    if (!strcmp(s, "identity")) return FN_IDENTITY;
    if (!strcmp(s, "moment")) return FN_MOMENT;
    if (!strcmp(s, "legendre_pointwise")) return FN_LEGENDRE;
    if (!strcmp(s, "log_entropy")) return FN_LOG_ENTROPY;
    if (!strcmp(s, "bv")) return FN_BV;
    if (!strcmp(s, "bv_direction")) return FN_BV_DIRECTION;
    if (!strcmp(s, "structure_cube")) return FN_STRUCTURE_CUBE;
    return -1;
}

/* Legendre polynomial P_l(x) by Bonnet's three-term recurrence in the order
 * of Boost.Math's legendre_p / legendre_next (the reference's CPU
 * LegendrePointWise calls boost::math::legendre_p,
 * alsfvm/src/functional/LegendrePointWise.cpp:57-82):
 *   P_0 = 1, P_1 = x, P_{n+1} = ((2n+1) x P_n - n P_{n-1}) / (n+1),
 * with P_{-l-1} = P_l. The caller checks -1 <= x <= 1. */
static double legendre_p(int l, double x) {
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

/* HostMemory::getTotalVariation(p, start, end) over one padded variable
 * (alsfvm/src/memory/HostMemory.cpp:325-362): 1D and 2D only; the sum over
 * z in [0, end.z), y from start.y + 1 (1D: 0), x from start.x + 1, of
 * (sqrt((u - u_below)^2 + (u - u_left)^2))^p, u_below = u itself in 1D. */
static double total_variation(const grid_t* G, const double* u, int p) {
    const long nx = G->t[0], ny = G->t[1];
    const long sx = G->g[0] + 1, sy = G->g[1] + (ny > 1 ? 1 : 0);
    const long ex = G->t[0] - G->g[0], ey = G->t[1] - G->g[1], ez = G->t[2] - G->g[2];
    double bv = 0;
    for (long z = 0; z < ez; z++)
        for (long y = sy; y < ey; y++)
            for (long x = sx; x < ex; x++) {
                const long i = z * nx * ny + y * nx + x;
                const long il = z * nx * ny + y * nx + (x - 1);
                const long yb = ny > 1 ? y - 1 : 0;
                const long ib = z * nx * ny + yb * nx + x;
                bv += pow(sqrt(pow(u[i] - u[ib], 2) + pow(u[i] - u[il], 2)), p);
            }
    return bv;
}

/* HostMemory::getTotalVariation(direction, p, start, end)
 * (alsfvm/src/memory/HostMemory.cpp:365-400): sum over the cells from
 * start + e_d to end of |u - u(- e_d)|^p. */
static double total_variation_direction(const grid_t* G, const double* u, int d, int p) {
    const long s[3] = {G->g[0] + (d == 0), G->g[1] + (d == 1), G->g[2] + (d == 2)};
    const long e[3] = {G->t[0] - G->g[0], G->t[1] - G->g[1], G->t[2] - G->g[2]};
    const long off = d == 0 ? 1 : (d == 1 ? G->t[0] : (long)G->t[0] * G->t[1]);
    double bv = 0;
    for (long z = s[2]; z < e[2]; z++)
        for (long y = s[1]; y < e[1]; y++)
            for (long x = s[0]; x < e[0]; x++) {
                const long i = IDX(G, x, y, z);
                bv += pow(fabs(u[i] - u[i - off]), p);
            }
    return bv;
}

int fv_functional(const char* name, const char* equation, const char* boundary, const int n[3], int ghosts,
                  const double lower[3], const double upper[3], int degree, double min_value, double max_value,
                  unsigned variable_mask, double gamma, double p, int number_of_h, int direction, double weight,
                  const double* U, double* out, int size_out[3]) {
    const int fn = parse_functional(name), eq = parse_eq(equation);
    if (fn < 0) return fail(-1, "Unknown functional: %s", name);
    if (eq < 0) return fail(-1, "unknown equation");
    grid_t G;
    make_grid(&G, eq, n, ghosts, gamma);
    /* Grid::computeCellLengths (alsfvm/src/grid/Grid.cpp:24-42) */
    double len[3];
    for (int d = 0; d < 3; ++d) len[d] = (upper[d] - lower[d]) / n[d];
    if (n[1] == 1) len[1] = 1;
    if (n[2] == 1) len[2] = 1;
    const long cells = (long)n[0] * n[1] * n[2];
    int o[3] = {n[0], n[1], n[2]};
    if (fn == FN_LOG_ENTROPY || fn == FN_BV || fn == FN_BV_DIRECTION) o[0] = o[1] = o[2] = 1;
    if (fn == FN_STRUCTURE_CUBE) {
        o[0] = number_of_h;
        o[1] = o[2] = 1;
    }
    if (size_out) memcpy(size_out, o, sizeof o);
    const long oc = (long)o[0] * o[1] * o[2];
    switch (fn) {
        case FN_IDENTITY:    /* alsfvm/src/functional/Identity.cpp:25-49 */
        case FN_MOMENT:      /* Moment.cpp:27-41 -> HostMemory::addPower(other, power, factor) */
        case FN_LEGENDRE: {  /* LegendrePointWise.cpp:37-87 */
            if (fn == FN_LEGENDRE && (len[2] > 1 || len[1] == 1))
                return fail(-1, "For now, Legendre polynomials only support 2d");
            for (int v = 0; v < G.nvar; ++v) {
                if (fn == FN_LEGENDRE && variable_mask && !((variable_mask >> v) & 1u)) continue;
                const double* u = U + (long)v * G.total;
                double* w = out + (long)v * oc;
                for (int k = 0; k < n[2]; ++k)
                    for (int j = 0; j < n[1]; ++j)
                        for (int i = 0; i < n[0]; ++i) {
                            const double x = u[IDX(&G, i + G.g[0], j + G.g[1], k + G.g[2])];
                            const long c = ((long)k * n[1] + j) * n[0] + i;
                            if (fn == FN_IDENTITY) {
                                w[c] += weight * x;
                            } else if (fn == FN_MOMENT) {
                                w[c] += weight * pow(x, (double)degree);
                            } else {
                                const double s = (x - min_value) / (max_value - min_value);
                                if (!(s >= -1.0 && s <= 1.0))
                                    return fail(-1, "The Legendre Polynomial is defined for -1 <= x <= 1, but got x = %.17g", s);
                                w[c] += legendre_p(degree, s) * weight;
                            }
                        }
            }
            return 0;
        }
        case FN_LOG_ENTROPY: {  /* LogEntropy.cpp:21-83 */
            if (eq == EQ_BURGERS) return fail(-1, "log_entropy needs the Euler variables");
            const double dxdydz = len[0] * len[1] * len[2];
            const double* rho = U;
            const double* E = U + (long)(G.nvar - 1) * G.total;
            double integral = 0.0;
            for (int k = 0; k < n[2]; ++k)
                for (int j = 0; j < n[1]; ++j)
                    for (int i = 0; i < n[0]; ++i) {
                        const long c = IDX(&G, i + G.g[0], j + G.g[1], k + G.g[2]);
                        const double density = rho[c], energy = E[c];
                        double momentumSquared = 0.0;
                        for (int m = 0; m < G.nsd; ++m) {
                            const double mm = U[(long)(1 + m) * G.total + c];
                            momentumSquared += mm * mm;
                        }
                        const double pressure = (gamma - 1) * (energy - 1.0 / (2 * density) * momentumSquared);
                        const double s = log(pressure) - gamma * log(density);
                        const double e = (-density * s) / (gamma - 1);
                        integral += e * dxdydz;
                    }
            out[(long)(G.nvar - 1) * oc] += weight * integral;
            return 0;
        }
        case FN_BV: {  /* functional/BoundedVariation.cpp:21-40 */
            if (len[2] > 1) return fail(-1, "For now, BoundedVariation  only support 2d and 1d");
            if (G.t[2] > 1) return fail(-1, "Not supported for 3d yet");
            for (int v = 0; v < G.nvar; ++v) out[(long)v * oc] += weight * total_variation(&G, U + (long)v * G.total, degree);
            return 0;
        }
        case FN_BV_DIRECTION: {
            if (direction < 0 || direction >= G.dim) return fail(-1, "direction = %d is bigger than current dimension", direction);
            for (int v = 0; v < G.nvar; ++v)
                out[(long)v * oc] += weight * total_variation_direction(&G, U + (long)v * G.total, direction, degree);
            return 0;
        }
        default: {  /* functional/StructureCube.cpp:24-60: zeroes its output first */
            (void)cells;
            return fv_structure_cube(equation, boundary, n, ghosts, number_of_h, p, U, out);
        }
    }
}

/* ---------------------------------------------------------- statistics */

/* MeanVariance::computeStatistics adds u and pow(u,2) per sample
 * (alsuq/src/stats/MeanVariance.cpp:30-53); StatisticsHelper::combineStatistics
 * divides by the sample count (StatisticsHelper.cpp:35-79); finalizeStatistics
 * subtracts pow(mean,2) (MeanVariance.cpp:55-67). */
int fv_meanvar(long count, int nsamples, const double* const* samples, double* mean,
               double* var) {
    if (count < 0 || nsamples <= 0) return fail(-1, "bad sizes");
    /* the exponent is read at run time so the compiler keeps the libm pow call
     * the reference makes (HostMemory::addPower takes the power as an argument) */
    volatile double two_v = 2.0;
    const double two = two_v;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < count; ++i) {
        double m = 0, v = 0;
        for (int s = 0; s < nsamples; ++s) {
            m += samples[s][i];
            v += pow(samples[s][i], two);
        }
        m /= (double)nsamples;
        v /= (double)nsamples;
        v -= pow(m, two);
        mean[i] = m;
        var[i] = v;
    }
    return 0;
}
