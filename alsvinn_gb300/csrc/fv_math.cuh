// Device arithmetic of the finite-volume step: Euler and Burgers point
// quantities, the HLL / HLL3 / Godunov numerical fluxes and the WENO2 / ENO2-4 /
// none reconstructions.
//
// Two policies share this header:
//  * Exact (FV_EXACT defined, translation unit built with -fmad=false): every
//    expression keeps the reference's operand order with IEEE-rounded + - * /
//    and sqrt, so results are bit-identical to the reference CPU path.
//  * Fast: the same mathematics with reciprocals shared between uses and the
//    WENO weights reduced to two reciprocals per cell. Its translation units
//    are built with -fmad=false too, and every fused multiply-add is written
//    out (mac, fma): the rounding is fixed by the source, so every tile
//    configuration of a scheme (the autotuner's candidates) gives the same
//    bits. Results agree with the reference to rounding level (relative 1e-15
//    per operation), well inside the 1e-10 relative L1 contract.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "fv_df.cuh"
#include "fv_types.h"

// Kernel code is compiled once per arithmetic variant; each variant's
// templates live in their own namespace so that identically named
// instantiations of different translation units never merge at link time.
#ifndef GBFV_VARIANT_NS
#define GBFV_VARIANT_NS common
#endif

namespace gbfv {
namespace GBFV_VARIANT_NS {

#ifdef FV_EXACT
constexpr bool kExact = true;
#else
constexpr bool kExact = false;
#endif

template <class R> __device__ __forceinline__ R rsqrt_(R x);
template <> __device__ __forceinline__ double rsqrt_<double>(double x) { return rsqrt(x); }
template <> __device__ __forceinline__ float rsqrt_<float>(float x) { return rsqrtf(x); }

template <class R> __device__ __forceinline__ R rcp_(R x) { return R(1) / x; }

// a * b + c: one rounding (an explicit FMA) in the fast policy, two in the
// exact one
template <class R> __device__ __forceinline__ R mac(R a, R b, R c) {
    if constexpr (kExact)
        return a * b + c;
    else
        return fma(a, b, c);
}

// FP64 reciprocal and reciprocal square root for the fast policy: a hardware
// approximation (PTX rcp.approx / rsqrt.approx .f64) refined by one step of a
// third-order iteration, which triples the number of correct bits:
//   reciprocal:  e = 1 - x y,    y' = y (1 + e + e^2)             (error e^3)
//   rsqrt:       d = 1 - x y^2,  y' = y (1 + d/2 + 3 d^2 / 8)     (error ~5 d^3 / 16)
// (truncated binomial series of (1 - e)^-1 and (1 - d)^-1/2, the
// Householder-type corrections of the Newton-Raphson family). The results
// are within about an ulp of the correctly rounded values
// (tests/cpp/test_special_functions.cu measures the ulp error against CUDA's
// IEEE division and sqrt), in fewer FP64 instructions than an IEEE division
// or square root.
template <> __device__ __forceinline__ double rcp_<double>(double x) {
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    const double e = fma(-x, y, 1.0);
    return fma(y, fma(e, e, e), y);
}

__device__ __forceinline__ double rsqrt_nr(double x) {
    double y;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    const double d = fma(-x * y, y, 1.0);
    return fma(y * d, fma(d, 0.375, 0.5), y);
}

// Tests on a double's bit pattern, evaluated on the integer pipes: GB300
// executes FP64 compares and minima / maxima at the FP64 rate (1/64 of the
// FP32 rate), which makes them as costly as an FMA in this FP64-bound kernel.
// Each helper returns what the IEEE operation returns, NaN cases included.
__device__ __forceinline__ long long dbits(double x) { return __double_as_longlong(x); }
constexpr long long kInfBits = 0x7ff0000000000000LL;
constexpr long long kAbsMask = 0x7fffffffffffffffLL;

// 0 < x < 1e300 (a positive finite value whose reciprocal square root stays
// normal): one unsigned compare of bits - 1 against the bits of 1e300 - 1
__device__ __forceinline__ bool in_rsqrt_range(double x) {
    return (unsigned long long)(dbits(x) - 1) < (unsigned long long)(0x7e37e43c8800759cLL - 1);
}

template <class R> __device__ __forceinline__ bool gt0(R x) { return x > R(0); }
template <class R> __device__ __forceinline__ bool lt0(R x) { return x < R(0); }
template <class R> __device__ __forceinline__ bool ge0(R x) { return x >= R(0); }
template <class R> __device__ __forceinline__ bool is0(R x) { return x == R(0); }
template <class R> __device__ __forceinline__ R fmin_(R a, R b) { return fmin(a, b); }
template <class R> __device__ __forceinline__ R fmax_(R a, R b) { return fmax(a, b); }

template <> __device__ __forceinline__ bool gt0<double>(double x) {
    if (kExact) return x > 0.0;
    const long long b = dbits(x);
    return b > 0 && b <= kInfBits;
}
template <> __device__ __forceinline__ bool lt0<double>(double x) {
    if (kExact) return x < 0.0;
    const long long b = dbits(x), m = b & kAbsMask;
    return b < 0 && m != 0 && m <= kInfBits;
}
template <> __device__ __forceinline__ bool ge0<double>(double x) {
    if (kExact) return x >= 0.0;
    const long long b = dbits(x);
    return b >= 0 ? b <= kInfBits : (b & kAbsMask) == 0;
}
template <> __device__ __forceinline__ bool is0<double>(double x) {
    if (kExact) return x == 0.0;
    return (dbits(x) & kAbsMask) == 0;
}
// total order of the non-NaN doubles as signed integers (-0 just below +0)
__device__ __forceinline__ long long order_key(long long b) { return b ^ ((b >> 63) & kAbsMask); }
template <> __device__ __forceinline__ double fmin_<double>(double a, double b) {
    if (kExact) return fmin(a, b);
    const long long x = dbits(a), y = dbits(b);
    if ((x & kAbsMask) > kInfBits) return b;
    if ((y & kAbsMask) > kInfBits) return a;
    return order_key(x) <= order_key(y) ? a : b;
}
template <> __device__ __forceinline__ double fmax_<double>(double a, double b) {
    if (kExact) return fmax(a, b);
    const long long x = dbits(a), y = dbits(b);
    if ((x & kAbsMask) > kInfBits) return b;
    if ((y & kAbsMask) > kInfBits) return a;
    return order_key(x) >= order_key(y) ? a : b;
}

// Double-float evaluation of the nonlinear coefficients of the fast FP64
// policy: the WENO2 weights and the HLL / HLL3 wave-speed estimates. They
// enter the fluxes multiplied by differences of the state -- the weights by
// the one-sided differences, the speeds through s (U* - U) and a star state
// whose sensitivity to s vanishes with the jump -- so their 2^-48 relative
// precision moves a flux by 2^-48 of those differences, well below the FP64
// rounding of the fluxes themselves, while ~30 FP64 instructions per face and
// ~20 per reconstructed cell move to the FP32 pipes (GB300 issues FP64 at 1/64
// of the FP32 rate). Inputs whose squares or products could leave the FP32
// exponent range take the FP64 formulas instead.
__device__ __forceinline__ bool df_range(double x, int max_exp) {  // |x| < 2^max_exp, finite
    return (dbits(x) & kAbsMask) < ((long long)(1023 + max_exp) << 52);
}

// The double-float split of an input of those coefficients: a magnitude
// below 2^-80 (a velocity or a one-sided difference far below the O(1) terms
// it is added to, or a zero) splits to a signed zero on the integer pipes;
// the general split takes conversion instructions there, FP64-pipe
// instructions that would then run for the few lanes of a warp holding such
// values. The coefficients do not change: 2^-80 is below their double-float
// resolution next to the terms beside it (eps = 1e-8 in the WENO weights,
// the sound speeds in the wave speeds).
__device__ __forceinline__ dfloat df_coef(double v) {
    const unsigned hw = (unsigned)((unsigned long long)__double_as_longlong(v) >> 32);
    if (((hw >> 20) & 0x7ffu) < 1023u - 80u) return dfloat(__uint_as_float(hw & 0x80000000u), 0.f);
    return dfloat(v);
}

// A double-float coefficient back to a double on the integer pipes: hi's 24
// significant bits and lo's aligned under them in one 53-bit integer
// significand (a normalised pair has lo at least 24 bits below hi's leading
// bit; lo's bits past the 53rd are dropped, an error under one ulp), with the
// one-bit renormalisation a lo of the other sign can need. A zero lo widens
// hi alone; pairs with a subnormal or non-finite part take the FP64 addition.
__device__ __forceinline__ double df_coef_to_double(const dfloat& a) {
    const unsigned uh = __float_as_uint(a.hi), ul = __float_as_uint(a.lo);
    const unsigned eh = (uh >> 23) & 0xffu, el = (ul >> 23) & 0xffu;
    if (eh - 1u < 254u) {
        if ((ul << 1) == 0u) return df_widen(a.hi);
        const int sh = (int)eh - (int)el;
        if (el - 1u < 254u && sh >= 24 && sh < 64) {
            const unsigned long long mh = (unsigned long long)((uh & 0x7fffffu) | 0x800000u) << 29;
            const unsigned long long mlo = (unsigned long long)((ul & 0x7fffffu) | 0x800000u);
            const unsigned long long ml = sh <= 29 ? mlo << (29 - sh) : mlo >> (sh - 29);
            unsigned long long m;
            int e = (int)eh - 127 + 1023;
            if ((uh ^ ul) & 0x80000000u) {
                m = mh - ml;
                if (m < (1ull << 52)) {
                    m <<= 1;
                    e -= 1;
                }
            } else {
                m = mh + ml;
            }
            return __longlong_as_double((long long)(((unsigned long long)(uh & 0x80000000u) << 32) |
                                                    ((unsigned long long)e << 52) | (m & ((1ull << 52) - 1))));
        }
    }
    return df_widen(a.hi) + df_widen(a.lo);
}

// The integer-pipe edges of the double-float coefficients (df_coef,
// df_coef_to_double) pay in the 1D and 2D kernels; the 3D kernels (five
// variables, 108 registers, two CTAs per SM) have too few warps to hide
// their integer latency and keep the general split and the FP64 addition.
template <int NSD> struct CoefEdges { static constexpr bool integer = NSD <= 2; };

template <bool INT> __device__ __forceinline__ dfloat coef_in(double v) {
    if constexpr (INT)
        return df_coef(v);
    else
        return dfloat(v);
}
template <bool INT> __device__ __forceinline__ double coef_out(const dfloat& a) {
    if constexpr (INT)
        return df_coef_to_double(a);
    else
        return (double)a;
}

template <bool CORRECT, bool INT>
__device__ __forceinline__ void wave_speeds_df(const dfloat& Wl, const dfloat& Wr, double ul, double ur, double pl,
                                               double pr, double il, double ir, double rl, double rr, double gamma,
                                               double& sL, double& sR) {
    const dfloat Ul = coef_in<INT>(ul), Ur = coef_in<INT>(ur), Pl = coef_in<INT>(pl), Pr = coef_in<INT>(pr),
                 Il(il), Ir(ir), G(gamma);
    const dfloat winv = dfloat(1) / (Wl + Wr);
    const dfloat ud = (Wl * Ul + Wr * Ur) * winv;
    const dfloat p = (Wl * Pl + Wr * Pr) * winv;
    const dfloat cl = sqrt(G * Pl * Il), cr = sqrt(G * Pr * Ir);
    const dfloat cs = sqrt((G + G) * p / (dfloat(rl) + dfloat(rr)));
    dfloat corr(0.f);
    if (CORRECT) corr = dfloat(0.5f) * fmax(dfloat(0), Ul - Ur);
    sL = coef_out<INT>(fmin(Ul + corr - cl, ud - cs));
    sR = coef_out<INT>(fmax(Ur - corr + cr, ud + cs));
}

// sqrt(x) = x / sqrt(x) for positive finite x; zero, negative and NaN
// arguments take the IEEE square root
template <class R> __device__ __forceinline__ R sqrt_(R x) { return sqrt(x); }
template <> __device__ __forceinline__ double sqrt_<double>(double x) {
    return in_rsqrt_range(x) ? x * rsqrt_nr(x) : sqrt(x);
}

// FP32 state (its tolerance is set by FP32 rounding): the special-function
// unit's approximations, within ~2 ulp, instead of the multi-instruction IEEE
// division and square root
template <> __device__ __forceinline__ float rcp_<float>(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
template <> __device__ __forceinline__ float sqrt_<float>(float x) {
    float y;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// 1/rho and sqrt(rho) of a density: one reciprocal square root for FP64 and
// FP32
template <class R> __device__ __forceinline__ void inv_sqrt_pair(R rho, R& rinv, R& w) {
    rinv = rcp_(rho);
    w = sqrt(rho);
}
template <> __device__ __forceinline__ void inv_sqrt_pair<float>(float rho, float& rinv, float& w) {
    if (rho > 0.f) {
        float rs;
        asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(rs) : "f"(rho));
        rinv = rs * rs;
        w = rho * rs;
    } else {
        rinv = 1.f / rho;
        w = sqrtf(rho);
    }
}
// FP64: sqrt(rho) enters only the wave-speed estimates, which the fast
// policy evaluates in double-float (wave_speeds_df), so the root is formed
// there directly: the double-float split of rho and its double-float square
// root run on the FP32 and integer pipes, and the FP64 pipe computes only the
// reciprocal (three FMAs after the hardware approximation, instead of the
// five of a refined reciprocal square root plus two products). States outside
// the double-float range (df_root_range) take the FP64 formulas, which form
// the root themselves (wave_root).
__device__ __forceinline__ void inv_sqrt_pair(double rho, double& rinv, dfloat& w) {
    if (in_rsqrt_range(rho)) {
        rinv = rcp_(rho);
        w = sqrt(dfloat(rho));
    } else {
        rinv = 1.0 / rho;
        w = dfloat(0.f);
    }
}

// 2^-100 <= rho < 2^120: the double-float root of rho and the wave-speed
// products stay normal FP32 numbers
__device__ __forceinline__ bool df_root_range(double rho) {
    constexpr long long lo = (1023LL - 100) << 52, hi = (1023LL + 120) << 52;
    return (unsigned long long)(dbits(rho) - lo) < (unsigned long long)(hi - lo);
}

// ---------------------------------------------------------------- Euler

// Conserved variables of one cell side plus the derived pressure and velocity
// (Euler<nsd>::computeExtra, alsfvm/include/alsfvm/equation/euler/Euler.hpp:204-211).
// sqrt(rho) as the fast policy keeps it: a double-float for the FP64 state
// (see inv_sqrt_pair), the state's own type otherwise
template <class R> struct WaveRoot { using type = R; };
template <> struct WaveRoot<double> { using type = dfloat; };

template <class R, int NSD> struct EulerState {
    R rho, m[NSD], E, p, u[NSD];
    R rinv;                        // 1/rho (fast policy only)
    typename WaveRoot<R>::type w;  // sqrt(rho) (fast policy only)
};

// sqrt(rho) in the state's type, for the FP64 formulas of the fast policy
template <class R, int NSD> __device__ __forceinline__ R wave_root(const EulerState<R, NSD>& s) {
    if constexpr (std::is_same<R, double>::value)
        return sqrt_(s.rho);
    else
        return s.w;
}

template <class R, int NSD>
__device__ __forceinline__ void euler_extra(EulerState<R, NSD>& a, R gamma) {
    if (kExact) {
        R dot = a.m[0] * a.m[0];
#pragma unroll
        for (int k = 1; k < NSD; ++k) dot = dot + a.m[k] * a.m[k];
        const R ie = a.E - R(0.5) * dot / a.rho;
#pragma unroll
        for (int k = 0; k < NSD; ++k) a.u[k] = a.m[k] / a.rho;
        a.p = (gamma - R(1)) * ie;
    } else {
        // m.m / rho as m.u: the velocities are needed anyway
        inv_sqrt_pair(a.rho, a.rinv, a.w);
#pragma unroll
        for (int k = 0; k < NSD; ++k) a.u[k] = a.m[k] * a.rinv;
        R mu = a.m[0] * a.u[0];
#pragma unroll
        for (int k = 1; k < NSD; ++k) mu = fma(a.m[k], a.u[k], mu);
        a.p = (gamma - R(1)) * fma(R(-0.5), mu, a.E);
    }
}

// Euler<nsd>::computePointFlux (Euler.hpp:172-181).
template <class R, int NSD, int D>
__device__ __forceinline__ void euler_point_flux(const EulerState<R, NSD>& a, R* F) {
    F[0] = a.m[D];
#pragma unroll
    for (int k = 0; k < NSD; ++k) F[1 + k] = (k == D) ? mac(a.u[D], a.m[k], a.p) : a.u[D] * a.m[k];
    F[1 + NSD] = (a.E + a.p) * a.u[D];
}

template <class R, int NSD>
__device__ __forceinline__ void euler_conserved(const EulerState<R, NSD>& a, R* c) {
    c[0] = a.rho;
#pragma unroll
    for (int k = 0; k < NSD; ++k) c[1 + k] = a.m[k];
    c[1 + NSD] = a.E;
}

// The HLL3 branches given the wave-speed estimates, computing the point flux
// of the one side each branch uses (the FP32 and double-float kernels: the
// FP64 kernel computes both before branching, which costs fewer registers
// there). The star branch's transverse velocities use
// fR - fL - sR mR + sL mL = (uR - sR) mR - (uL - sL) mL, since the momentum
// point fluxes are u_D m_k.
template <class R, int NSD, int D>
__device__ __forceinline__ R hll3_branches_one_side(const EulerState<R, NSD>& L, const EulerState<R, NSD>& Rs,
                                                    R speedLeft, R speedRight, R* F) {
    constexpr int NV = NSD + 2;
    if (is0(speedLeft)) {
#pragma unroll
        for (int k = 0; k < NV; ++k) F[k] = R(0);
    } else if (gt0(speedLeft)) {
        euler_point_flux<R, NSD, D>(L, F);
    } else if (lt0(speedRight)) {
        euler_point_flux<R, NSD, D>(Rs, F);
    } else {
        const R udl = L.u[D] - speedLeft;
        const R udr = Rs.u[D] - speedRight;
        const R ainv = rcp_(fma(udr, Rs.rho, -(udl * L.rho)));
        const R sm = (fma(Rs.m[D], udr, -(L.m[D] * udl)) + Rs.p - L.p) * ainv;
        const bool leftSide = ge0(sm);
        const EulerState<R, NSD>& S = leftSide ? L : Rs;
        const R s = leftSide ? speedLeft : speedRight;
        const R ud = leftSide ? udl : udr;
        R fS[NV];
        euler_point_flux<R, NSD, D>(S, fS);
        // F = fS + s (U* - U) with each star component formed as a product
        // minus the conserved value in one FMA
        const R sinv = rcp_(sm - s);
        const R mid0 = S.rho * ud * sinv;
        F[0] = fma(s, mid0 - S.rho, fS[0]);
#pragma unroll
        for (int k = 0; k < NSD; ++k) {
            const R usk = (k == D) ? sm : fma(udr, Rs.m[k], -(udl * L.m[k])) * ainv;
            F[1 + k] = fma(s, fma(mid0, usk, -S.m[k]), fS[1 + k]);
        }
        const R pp = fma(S.rho * (S.u[D] - sm), ud, S.p);
        const R eS = fma(ud, S.E, fma(S.p, S.u[D], -(pp * sm)));
        F[1 + NSD] = fma(s, fma(eS, sinv, -S.E), fS[1 + NSD]);
    }
    return fmax_(fabs(speedLeft), fabs(speedRight));
}

// HLL3 (HLLC-type) flux F(left, right) in direction D with the reference's
// extended speed estimate and its speedLeft == 0 -> F = 0 rule
// (alsfvm/include/alsfvm/numflux/euler/HLL3.hpp:52-148). Returns
// max(|speedLeft|, |speedRight|).
template <class R, int NSD, int D>
__device__ __forceinline__ R flux_hll3(const EulerState<R, NSD>& L, const EulerState<R, NSD>& Rs,
                                       R gamma, R* F) {
    constexpr int NV = NSD + 2;
    R speedLeft, speedRight;
    if (kExact) {
        const R waveLeft = sqrt(L.rho);
        const R waveRight = sqrt(Rs.rho);
        const R rho = (L.rho + Rs.rho) / R(2);
        const R ud = (waveLeft * L.u[D] + waveRight * Rs.u[D]) / (waveLeft + waveRight);
        const R p = (waveLeft * L.p + waveRight * Rs.p) / (waveLeft + waveRight);
        const R cfLeft = sqrt(gamma * L.p / L.rho);
        const R cfRight = sqrt(gamma * Rs.p / Rs.rho);
        const R correct = R(0.5) * fmax(R(0), L.u[D] - Rs.u[D]);
        const R cs = sqrt(gamma * p / rho);
        speedLeft = fmin(L.u[D] + correct - cfLeft, ud - cs);
        speedRight = fmax(Rs.u[D] - correct + cfRight, ud + cs);
    } else {
        bool done = false;
        if constexpr (std::is_same<R, double>::value) {
            if (df_root_range(L.rho) && df_root_range(Rs.rho) && df_range(L.u[D], 60) && df_range(Rs.u[D], 60) &&
                df_range(L.p, 60) && df_range(Rs.p, 60) && df_range(L.rinv, 60) && df_range(Rs.rinv, 60)) {
                wave_speeds_df<true, CoefEdges<NSD>::integer>(L.w, Rs.w, L.u[D], Rs.u[D], L.p, Rs.p, L.rinv, Rs.rinv, L.rho, Rs.rho, gamma,
                                     speedLeft, speedRight);
                done = true;
            }
        }
        if (!done) {
            const R waveLeft = wave_root(L);
            const R waveRight = wave_root(Rs);
            const R winv = rcp_(waveLeft + waveRight);
            const R ud = fma(waveLeft, L.u[D], waveRight * Rs.u[D]) * winv;
            const R p = fma(waveLeft, L.p, waveRight * Rs.p) * winv;
            const R cfLeft = sqrt_(gamma * L.p * L.rinv);
            const R cfRight = sqrt_(gamma * Rs.p * Rs.rinv);
            const R correct = R(0.5) * fmax_(R(0), L.u[D] - Rs.u[D]);
            const R cs = sqrt_(R(2) * gamma * p * rcp_(L.rho + Rs.rho));
            speedLeft = fmin_(L.u[D] + correct - cfLeft, ud - cs);
            speedRight = fmax_(Rs.u[D] - correct + cfRight, ud + cs);
        }
    }
    if constexpr (!kExact && !std::is_same<R, double>::value) {
        // FP32 and double-float: evaluate only the point flux a branch uses
        return hll3_branches_one_side<R, NSD, D>(L, Rs, speedLeft, speedRight, F);
    }
    if constexpr (!kExact) {
        // FP64: the contact speed first, then one point flux -- of the side
        // every branch but the zero-speed one uses (the upwind state, or the
        // star state's side of sm) -- selected without branching, and the
        // star's transverse velocities as ((uR - sR) mR - (uL - sL) mL) / a
        const R udl = L.u[D] - speedLeft;
        const R udr = Rs.u[D] - speedRight;
        const R ainv = rcp_(fma(udr, Rs.rho, -(udl * L.rho)));
        const R sm = (fma(Rs.m[D], udr, -(L.m[D] * udl)) + Rs.p - L.p) * ainv;
        const bool upLeft = gt0(speedLeft), upRight = lt0(speedRight);
        const bool useLeft = upLeft || (!upRight && ge0(sm));
        const EulerState<R, NSD>& S = useLeft ? L : Rs;
        R fS[NV];
        euler_point_flux<R, NSD, D>(S, fS);
        if (is0(speedLeft)) {
#pragma unroll
            for (int k = 0; k < NV; ++k) F[k] = R(0);
        } else if (upLeft || upRight) {
#pragma unroll
            for (int k = 0; k < NV; ++k) F[k] = fS[k];
        } else {
            const R s = useLeft ? speedLeft : speedRight;
            const R ud = useLeft ? udl : udr;
            const R sinv = rcp_(sm - s);
            const R mid0 = S.rho * ud * sinv;
            F[0] = fma(s, mid0 - S.rho, fS[0]);
#pragma unroll
            for (int k = 0; k < NSD; ++k) {
                const R usk = (k == D) ? sm : fma(udr, Rs.m[k], -(udl * L.m[k])) * ainv;
                F[1 + k] = fma(s, fma(mid0, usk, -S.m[k]), fS[1 + k]);
            }
            const R pp = fma(S.rho * (S.u[D] - sm), ud, S.p);
            const R eS = fma(ud, S.E, fma(S.p, S.u[D], -(pp * sm)));
            F[1 + NSD] = fma(s, fma(eS, sinv, -S.E), fS[1 + NSD]);
        }
        return fmax_(fabs(speedLeft), fabs(speedRight));
    }
    R fluxLeft[NV], fluxRight[NV];
    euler_point_flux<R, NSD, D>(L, fluxLeft);
    euler_point_flux<R, NSD, D>(Rs, fluxRight);
    const R udl = L.u[D] - speedLeft;
    const R udr = Rs.u[D] - speedRight;
    const R aa = kExact ? udr * Rs.rho - udl * L.rho : fma(udr, Rs.rho, -(udl * L.rho));
    const R ainv = kExact ? R(0) : rcp_(aa);
    const R sm = kExact ? (Rs.m[D] * udr - L.m[D] * udl + Rs.p - L.p) / aa
                        : (fma(Rs.m[D], udr, -(L.m[D] * udl)) + Rs.p - L.p) * ainv;
    if (is0(speedLeft)) {
#pragma unroll
        for (int k = 0; k < NV; ++k) F[k] = R(0);
    } else if (gt0(speedLeft)) {
#pragma unroll
        for (int k = 0; k < NV; ++k) F[k] = fluxLeft[k];
    } else if (lt0(speedRight)) {
#pragma unroll
        for (int k = 0; k < NV; ++k) F[k] = fluxRight[k];
    } else {
        // Star state on the side of the contact speed sm.
        const bool leftSide = ge0(sm);
        const EulerState<R, NSD>& S = leftSide ? L : Rs;
        const R s = leftSide ? speedLeft : speedRight;
        const R ud = leftSide ? udl : udr;
        const R* fS = leftSide ? fluxLeft : fluxRight;
        R mid[NV], c[NV];
        if (kExact) {
            R us[NSD];
#pragma unroll
            for (int k = 0; k < NSD; ++k)
                us[k] = (fluxRight[1 + k] - fluxLeft[1 + k] - speedRight * Rs.m[k] + speedLeft * L.m[k]) / aa;
            us[D] = sm;
            mid[0] = S.rho * ud / (sm - s);
#pragma unroll
            for (int k = 0; k < NSD; ++k) mid[1 + k] = mid[0] * us[k];
            const R pp = S.p + S.rho * (S.u[D] - sm) * ud;
            mid[1 + NSD] = (ud * S.E + S.p * S.u[D] - pp * sm) / (sm - s);
        } else {
            // F = fS + s (U* - U) with each star component formed as a
            // product minus the conserved value in one FMA
            const R sinv = rcp_(sm - s);
            const R mid0 = S.rho * ud * sinv;
            F[0] = fma(s, mid0 - S.rho, fS[0]);
#pragma unroll
            for (int k = 0; k < NSD; ++k) {
                const R usk = (k == D) ? sm
                                       : fma(speedLeft, L.m[k],
                                             fma(-speedRight, Rs.m[k], fluxRight[1 + k] - fluxLeft[1 + k])) *
                                             ainv;
                F[1 + k] = fma(s, fma(mid0, usk, -S.m[k]), fS[1 + k]);
            }
            const R pp = fma(S.rho * (S.u[D] - sm), ud, S.p);
            const R eS = fma(ud, S.E, fma(S.p, S.u[D], -(pp * sm)));
            F[1 + NSD] = fma(s, fma(eS, sinv, -S.E), fS[1 + NSD]);
            return fmax_(fabs(speedLeft), fabs(speedRight));
        }
        euler_conserved<R, NSD>(S, c);
#pragma unroll
        for (int k = 0; k < NV; ++k) F[k] = fS[k] + s * (mid[k] - c[k]);
    }
    return fmax_(fabs(speedLeft), fabs(speedRight));
}

// HLL flux (alsfvm/include/alsfvm/numflux/euler/HLL.hpp:51-115).
template <class R, int NSD, int D>
__device__ __forceinline__ R flux_hll(const EulerState<R, NSD>& L, const EulerState<R, NSD>& Rs,
                                      R gamma, R* F) {
    constexpr int NV = NSD + 2;
    R speedLeft, speedRight;
    if (kExact) {
        const R waveLeft = sqrt(L.rho);
        const R waveRight = sqrt(Rs.rho);
        const R rho = (L.rho + Rs.rho) / R(2);
        const R ud = (waveLeft * L.u[D] + waveRight * Rs.u[D]) / (waveLeft + waveRight);
        const R p = (L.p * waveLeft + Rs.p * waveRight) / (waveLeft + waveRight);
        const R cs = sqrt(gamma * p / rho);
        speedLeft = fmin(L.u[D] - sqrt(gamma * L.p / L.rho), ud - cs);
        speedRight = fmax(Rs.u[D] + sqrt(gamma * Rs.p / Rs.rho), ud + cs);
    } else {
        bool done = false;
        if constexpr (std::is_same<R, double>::value) {
            if (df_root_range(L.rho) && df_root_range(Rs.rho) && df_range(L.u[D], 60) && df_range(Rs.u[D], 60) &&
                df_range(L.p, 60) && df_range(Rs.p, 60) && df_range(L.rinv, 60) && df_range(Rs.rinv, 60)) {
                wave_speeds_df<false, CoefEdges<NSD>::integer>(L.w, Rs.w, L.u[D], Rs.u[D], L.p, Rs.p, L.rinv, Rs.rinv, L.rho, Rs.rho, gamma,
                                      speedLeft, speedRight);
                done = true;
            }
        }
        if (!done) {
            const R waveLeft = wave_root(L);
            const R waveRight = wave_root(Rs);
            const R winv = rcp_(waveLeft + waveRight);
            const R ud = fma(waveLeft, L.u[D], waveRight * Rs.u[D]) * winv;
            const R p = fma(L.p, waveLeft, Rs.p * waveRight) * winv;
            const R cs = sqrt_(R(2) * gamma * p * rcp_(L.rho + Rs.rho));
            speedLeft = fmin_(L.u[D] - sqrt_(gamma * L.p * L.rinv), ud - cs);
            speedRight = fmax_(Rs.u[D] + sqrt_(gamma * Rs.p * Rs.rinv), ud + cs);
        }
    }
    if (is0(speedLeft)) {
#pragma unroll
        for (int k = 0; k < NV; ++k) F[k] = R(0);
    } else if (gt0(speedLeft)) {
        euler_point_flux<R, NSD, D>(L, F);
    } else if (lt0(speedRight)) {
        euler_point_flux<R, NSD, D>(Rs, F);
    } else {
        R fl[NV], fr[NV], cl[NV], cr[NV];
        euler_point_flux<R, NSD, D>(L, fl);
        euler_point_flux<R, NSD, D>(Rs, fr);
        euler_conserved<R, NSD>(L, cl);
        euler_conserved<R, NSD>(Rs, cr);
        if (kExact) {
#pragma unroll
            for (int k = 0; k < NV; ++k)
                F[k] = (speedRight * fl[k] - speedLeft * fr[k] + speedRight * speedLeft * (cr[k] - cl[k])) /
                       (speedRight - speedLeft);
        } else {
            const R inv = rcp_(speedRight - speedLeft);
            const R srl = speedRight * speedLeft;
#pragma unroll
            for (int k = 0; k < NV; ++k)
                F[k] = fma(srl, cr[k] - cl[k], fma(speedRight, fl[k], -(speedLeft * fr[k]))) * inv;
        }
    }
    return fmax_(fabs(speedLeft), fabs(speedRight));
}

// Godunov flux for Burgers: F = max(f(max(uL,0)), f(min(uR,0))), f = u^2/2,
// wave speed max(|uL|,|uR|) (alsfvm/include/alsfvm/numflux/burgers/Godunov.hpp:40-60).
template <class R>
__device__ __forceinline__ R flux_godunov(R uL, R uR, R* F) {
    const R a = fmax_(uL, R(0));
    const R b = fmin_(uR, R(0));
    F[0] = fmax_(a * a / R(2), b * b / R(2));
    return fmax_(fabs(uL), fabs(uR));
}

// Central flux F = (f(L) + f(R)) / 2 with the wave speed max over the two
// states of |u_d| + sqrt(gamma p / rho) (alsfvm/include/alsfvm/numflux/
// Central.hpp:31-55, Euler.hpp:251-258).
template <class R, int NSD, int D>
__device__ __forceinline__ R flux_central(const EulerState<R, NSD>& L, const EulerState<R, NSD>& Rs, R gamma,
                                          R* F) {
    constexpr int NV = NSD + 2;
    R fl[NV], fr[NV];
    euler_point_flux<R, NSD, D>(L, fl);
    euler_point_flux<R, NSD, D>(Rs, fr);
#pragma unroll
    for (int k = 0; k < NV; ++k) F[k] = R(0.5) * (fl[k] + fr[k]);
    R wl, wr;
    if (kExact) {
        wl = fabs(L.u[D]) + sqrt(gamma * L.p / L.rho);
        wr = fabs(Rs.u[D]) + sqrt(gamma * Rs.p / Rs.rho);
    } else {
        wl = fabs(L.u[D]) + sqrt_(gamma * L.p * L.rinv);
        wr = fabs(Rs.u[D]) + sqrt_(gamma * Rs.p * Rs.rinv);
    }
    return fmax_(wl, wr);
}

// Burgers fluxes beyond Godunov, f(u) = u u / 2, wave speed max(|uL|, |uR|):
// Central, Rusanov with the eigenvalue u (alsfvm/include/alsfvm/numflux/
// Rusanov.hpp:31-59, Burgers.hpp:298-301) and Roe (alsfvm/include/alsfvm/
// numflux/burgers/Roe.hpp:30-58).
template <class R, int FLUX>
__device__ __forceinline__ R flux_burgers(R uL, R uR, R* F) {
    const R fL = uL * uL / R(2), fR = uR * uR / R(2);
    if constexpr (FLUX == 3) {  // central
        F[0] = R(0.5) * (fL + fR);
    } else if constexpr (FLUX == 4) {  // rusanov
        const R eigenMax = fmax_(fabs(uL), fabs(uR));
        F[0] = R(0.5) * (fL + fR) - R(0.5) * eigenMax * (uR - uL);
    } else {  // roe
        if (uL >= -uR) {
            const R a = fmax_(uL, R(0));
            F[0] = a * a / R(2);
        } else {
            const R b = fmin_(uR, R(0));
            F[0] = b * b / R(2);
        }
    }
    return fmax_(fabs(uL), fabs(uR));
}

// ------------------------------------------------------- reconstruction

// sign (1, 0, -1; -1 for NaN) and minmod of the limiter reconstructions
// (alsfvm/include/alsfvm/reconstruction/sign.hpp, minmod.hpp)
template <class R> __device__ __forceinline__ R sign_of(R a) { return gt0(a) ? R(1) : (is0(a) ? R(0) : R(-1)); }
template <class R> __device__ __forceinline__ R minmod2(R a, R b) {
    const R sa = sign_of(a);
    return sa == sign_of(b) ? sa * fmin_(fabs(a), fabs(b)) : R(0);
}
template <class R> __device__ __forceinline__ R minmod3(R a, R b, R c) {
    const R sa = sign_of(a), sb = sign_of(b);
    return (sa == sb && sb == sign_of(c)) ? sa * fmin_(fabs(a), fmin_(fabs(b), fabs(c))) : R(0);
}


template <int RC> struct ReconTraits;
template <> struct ReconTraits<RC_NONE> { static constexpr int ghosts = 1; static constexpr int reach = 0; };
template <> struct ReconTraits<RC_WENO2> { static constexpr int ghosts = 2; static constexpr int reach = 1; };
template <> struct ReconTraits<RC_ENO2> { static constexpr int ghosts = 2; static constexpr int reach = 1; };
template <> struct ReconTraits<RC_ENO3> { static constexpr int ghosts = 3; static constexpr int reach = 2; };
template <> struct ReconTraits<RC_ENO4> { static constexpr int ghosts = 4; static constexpr int reach = 3; };
template <> struct ReconTraits<RC_MC> { static constexpr int ghosts = 2; static constexpr int reach = 1; };
template <> struct ReconTraits<RC_MM> { static constexpr int ghosts = 2; static constexpr int reach = 1; };
template <> struct ReconTraits<RC_WENOF2> { static constexpr int ghosts = 2; static constexpr int reach = 1; };

// ENO coefficient rows (alsfvm/src/reconstruction/ENOCoefficients.cpp:21-49):
// row r weights the stencil starting r cells to the left for the value at the
// cell's left face; row r+1 gives the right-face value.
template <int ORDER> struct EnoC;
template <> struct EnoC<2> {
    static __device__ __forceinline__ double c(int r, int j) {
        const double t[3][2] = {{3.0 / 2.0, -1.0 / 2.0}, {1.0 / 2.0, 1.0 / 2.0}, {-1.0 / 2.0, 3.0 / 2.0}};
        return t[r][j];
    }
};
template <> struct EnoC<3> {
    static __device__ __forceinline__ double c(int r, int j) {
        const double t[4][3] = {{11.0 / 6.0, -7.0 / 6.0, 1.0 / 3.0},
                                {1.0 / 3.0, 5.0 / 6.0, -1.0 / 6.0},
                                {-1.0 / 6.0, 5.0 / 6.0, 1.0 / 3.0},
                                {1.0 / 3.0, -7.0 / 6.0, 11.0 / 6.0}};
        return t[r][j];
    }
};
template <> struct EnoC<4> {
    static __device__ __forceinline__ double c(int r, int j) {
        const double t[5][4] = {{25.0 / 12.0, -23.0 / 12.0, 13.0 / 12.0, -1.0 / 4.0},
                                {1.0 / 4.0, 13.0 / 12.0, -5.0 / 12.0, 1.0 / 12.0},
                                {-1.0 / 12.0, 7.0 / 12.0, 7.0 / 12.0, -1.0 / 12.0},
                                {1.0 / 12.0, -5.0 / 12.0, 13.0 / 12.0, 1.0 / 4.0},
                                {-1.0 / 4.0, 13.0 / 12.0, -23.0 / 12.0, 25.0 / 12.0}};
        return t[r][j];
    }
};

// |a| < |b| (false if either is NaN): on the magnitude bits for doubles in
// the fast policy
template <class R> __device__ __forceinline__ bool abs_less(R a, R b) { return fabs(a) < fabs(b); }
template <> __device__ __forceinline__ bool abs_less<double>(double a, double b) {
    if (kExact) return fabs(a) < fabs(b);
    const long long x = dbits(a) & kAbsMask, y = dbits(b) & kAbsMask;
    return x < y && y <= kInfBits;
}

#define FV_WENO_EPSILON 1e-8  // alsfvm/include/alsfvm/reconstruction/WENOCoefficients.hpp:21

// Reconstructs the values of one cell at its left (i-1/2) and right (i+1/2)
// faces for all NV variables. `u` points at the cell's variable 0 in a strided
// store: variable k sits at u[k * vs], neighbour j along the direction at
// u[j * ds]. Variable 0 is the WENO weight / ENO indicator (rho for Euler,
// u for Burgers: Euler.hpp:286-288).
// WENOF2<Euler<nsd>>::reconstruct (alsfvm/include/alsfvm/reconstruction/
// WENOF2.hpp:31-112): the WENO2 weights of the density applied to the
// primitive variables (rho, u, p) of the three cells, the density and
// pressure increments bounded by 1.9 times the cell's values, the increment
// scaled by aijk = sqrt(R / max(R, LL)) / 2 (R = p / (gamma - 1), LL a
// kinetic-energy bound), then back to conserved variables
// (Euler::computeConserved, Euler.hpp:236-245). The reference's operand
// order throughout; vector dot products accumulate x, y, z in order.
template <class R, int NSD>
__device__ __forceinline__ void wenof2_prim(const R* c, int vs, R gamma, R* q) {
    const R rho = c[0];
    R dot = c[vs] * c[vs];
#pragma unroll
    for (int k = 0; k < NSD; ++k) q[1 + k] = c[(1 + k) * vs] / rho;
#pragma unroll
    for (int k = 1; k < NSD; ++k) dot = dot + c[(1 + k) * vs] * c[(1 + k) * vs];
    const R ie = c[(1 + NSD) * vs] - R(0.5) * dot / rho;
    q[0] = rho;
    q[1 + NSD] = (gamma - R(1)) * ie;
}

template <class R, int NSD>
__device__ __forceinline__ R dot_n(const R* a, const R* b) {
    R d = a[0] * b[0];
#pragma unroll
    for (int k = 1; k < NSD; ++k) d = d + a[k] * b[k];
    return d;
}

template <class R, int NSD, int SIDE>
__device__ __forceinline__ void wenof2_side(const R* L, const R* M, const R* Rr, R w0, R w1, R gamma, R* out) {
    constexpr int NV = NSD + 2;
    const R BOUND = R(1.9);
    R d[NV];
#pragma unroll
    for (int c = 0; c < NV; ++c) d[c] = w1 * (M[c] - L[c]) + w0 * (Rr[c] - M[c]);
    d[0] = fmax(-BOUND * M[0], fmin(BOUND * M[0], d[0]));
    d[NV - 1] = fmax(-BOUND * M[NV - 1], fmin(BOUND * M[NV - 1], d[NV - 1]));
    const R dd = dot_n<R, NSD>(d + 1, d + 1);
    const R LL = R(0.125) * M[0] * dd - R(0.5) * fmin(R(0), d[0] * dot_n<R, NSD>(M + 1, d + 1)) +
                 R(0.5) * d[0] * d[0] * dd / M[0];
    const R Rp = M[NV - 1] / (gamma - R(1));
    const R a = R(0.5) * sqrt(Rp / fmax(Rp, LL));
    R q[NV];
#pragma unroll
    for (int c = 0; c < NV; ++c) q[c] = SIDE < 0 ? M[c] - a * d[c] : M[c] + a * d[c];
    out[0] = q[0];
#pragma unroll
    for (int k = 0; k < NSD; ++k) out[1 + k] = q[0] * q[1 + k];
    out[1 + NSD] = q[NV - 1] / (gamma - R(1)) + R(0.5) * q[0] * dot_n<R, NSD>(q + 1, q + 1);
}

template <class R, int NV, int RC>
__device__ __forceinline__ void reconstruct_cell(const R* __restrict__ u, int vs, int ds, R* left, R* right,
                                                 R gamma = R(1.4)) {
    if constexpr (RC == RC_NONE) {
#pragma unroll
        for (int k = 0; k < NV; ++k) left[k] = right[k] = u[k * vs];
    } else if constexpr (RC == RC_WENOF2) {
        constexpr int NSD = NV - 2;
        static_assert(NSD >= 1, "WENOF2 reconstructs the Euler equations only");
        const R i0 = u[0];
        const R b0 = (u[ds] - i0) * (u[ds] - i0);
        const R b1 = (i0 - u[-ds]) * (i0 - u[-ds]);
        const R eps = R(FV_WENO_EPSILON);
        const R a0Left = R(1) / (R(3) * (eps + b0) * (eps + b0));
        const R a1Left = R(2) / (R(3) * (eps + b1) * (eps + b1));
        const R w0Left = a0Left / (a0Left + a1Left);
        const R w1Left = a1Left / (a0Left + a1Left);
        const R a0Right = R(2) / (R(3) * (eps + b0) * (eps + b0));
        const R a1Right = R(1) / (R(3) * (eps + b1) * (eps + b1));
        const R w0Right = a0Right / (a0Right + a1Right);
        const R w1Right = a1Right / (a0Right + a1Right);
        R pl[NV], pm[NV], pr[NV];
        wenof2_prim<R, NSD>(u - ds, vs, gamma, pl);
        wenof2_prim<R, NSD>(u, vs, gamma, pm);
        wenof2_prim<R, NSD>(u + ds, vs, gamma, pr);
        wenof2_side<R, NSD, -1>(pl, pm, pr, w0Left, w1Left, gamma, left);
        wenof2_side<R, NSD, 1>(pl, pm, pr, w0Right, w1Right, gamma, right);
    } else if constexpr (RC == RC_MC || RC == RC_MM) {
        // MC / MM slope limiters on every variable (alsfvm/include/alsfvm/
        // reconstruction/MC.hpp:27-52, MM.hpp:25-47)
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            const R* v = u + k * vs;
            const R l = v[-ds], m = v[0], r = v[ds];
            R sigma;
            if constexpr (RC == RC_MC)
                sigma = minmod3(R(2) * (r - m), (r - l) / R(2), R(2) * (m - l));
            else
                sigma = minmod2(r - m, m - l);
            left[k] = m - sigma / R(2);
            right[k] = m + sigma / R(2);
        }
    } else if constexpr (RC == RC_WENO2) {
        // WENO2::reconstruct (alsfvm/include/alsfvm/reconstruction/WENO2.hpp:31-91).
        const R i0 = u[0];
        const R d0 = u[ds] - i0;
        const R d1 = i0 - u[-ds];
        const R b0 = d0 * d0;
        const R b1 = d1 * d1;
        R w0Left, w1Left, w0Right, w1Right;
        if (kExact) {
            const R eps = R(FV_WENO_EPSILON);
            const R a0Left = R(1) / (R(3) * (eps + b0) * (eps + b0));
            const R a1Left = R(2) / (R(3) * (eps + b1) * (eps + b1));
            w0Left = a0Left / (a0Left + a1Left);
            w1Left = a1Left / (a0Left + a1Left);
            const R a0Right = R(2) / (R(3) * (eps + b0) * (eps + b0));
            const R a1Right = R(1) / (R(3) * (eps + b1) * (eps + b1));
            w0Right = a0Right / (a0Right + a1Right);
            w1Right = a1Right / (a0Right + a1Right);
        } else {
            // alpha0 ~ 1/(eps+b0)^2, alpha1 ~ 2/(eps+b1)^2 (left face), and the
            // mirrored pair on the right face; normalising gives weights in
            // terms of s_k = (eps+b_k)^2 with one reciprocal per face.
            const R eps = R(FV_WENO_EPSILON);
            if constexpr (std::is_same<R, double>::value || std::is_same<R, float>::value) {
                // half weights and hardware FMAs: with w0 + w1 = 1,
                // left = u_i - (w1/2)(u_i - u_{i-1}) - (w0/2)(u_{i+1} - u_i),
                // right = u_i + (w0/2)(u_{i+1} - u_i) + (w1/2)(u_i - u_{i-1})
                R h0L, h1L, h0R, h1R;
                bool done = false;
                if constexpr (std::is_same<R, double>::value) {
                    if (df_range(d0, 30) && df_range(d1, 30)) {
                        constexpr bool kInt = CoefEdges<NV - 2>::integer;  // Euler: NV = NSD + 2
                        const dfloat D0 = coef_in<kInt>(d0), D1 = coef_in<kInt>(d1), E(FV_WENO_EPSILON);
                        const dfloat e0 = E + D0 * D0, e1 = E + D1 * D1;
                        const dfloat s0 = e0 * e0, s1 = e1 * e1;
                        const dfloat iL = dfloat(1) / (s1 + s0 + s0), iR = dfloat(1) / (s1 + s1 + s0);
                        h0L = coef_out<kInt>(dfloat(0.5f) * s1 * iL);
                        h1L = coef_out<kInt>(s0 * iL);
                        h0R = coef_out<kInt>(s1 * iR);
                        h1R = coef_out<kInt>(dfloat(0.5f) * s0 * iR);
                        done = true;
                    }
                }
                if (!done) {
                    const R e0 = fma(d0, d0, eps), e1 = fma(d1, d1, eps);
                    const R s0 = e0 * e0;
                    const R s1 = e1 * e1;
                    const R iL = rcp_(fma(R(2), s0, s1));
                    const R iR = rcp_(fma(R(2), s1, s0));
                    h0L = R(0.5) * s1 * iL;
                    h1L = s0 * iL;
                    h0R = s1 * iR;
                    h1R = R(0.5) * s0 * iR;
                }
#pragma unroll
                for (int k = 0; k < NV; ++k) {
                    const R* v = u + k * vs;
                    const R uc = v[0];
                    const R dp = v[ds] - uc, dm = uc - v[-ds];
                    left[k] = fma(-h1L, dm, fma(-h0L, dp, uc));
                    right[k] = fma(h0R, dp, fma(h1R, dm, uc));
                }
                return;
            }
            const R s0 = (eps + b0) * (eps + b0);
            const R s1 = (eps + b1) * (eps + b1);
            const R iL = rcp_(s1 + R(2) * s0);
            const R iR = rcp_(R(2) * s1 + s0);
            w0Left = s1 * iL;
            w1Left = R(2) * s0 * iL;
            w0Right = R(2) * s1 * iR;
            w1Right = s0 * iR;
        }
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            const R* v = u + k * vs;
            const R um = v[-ds], uc = v[0], up = v[ds];
            left[k] = R(0.5) * (w1Left * um + (R(3) * w0Left + w1Left) * uc - w0Left * up);
            right[k] = R(0.5) * (w0Right * up + (R(3) * w1Right + w0Right) * uc - w1Right * um);
        }
    } else {
        // ENOCPU<order> (alsfvm/src/reconstruction/ENOCPU.cpp:41-171): undivided
        // differences of variable 0; at each level the shift grows when the
        // left difference is smaller in magnitude than the right one.
        constexpr int ORDER = RC;  // RC_ENO2 == 2, ...
        constexpr int W = 2 * ORDER - 1;
        R w[W];
#pragma unroll
        for (int j = 0; j < W; ++j) w[j] = u[(j - (ORDER - 1)) * ds];
        R dd[W];
#pragma unroll
        for (int j = 0; j < W - 1; ++j) dd[j] = w[j + 1] - w[j];
        int shift = 0;
        constexpr int c = ORDER - 1;
#pragma unroll
        for (int l = 0; l < ORDER - 1; ++l) {
            if (abs_less(dd[c - 1], dd[c])) shift++;
            if (l + 1 < ORDER - 1) {
#pragma unroll
                for (int j = 0; j < W - 2 - l; ++j) dd[j] = dd[j + 1] - dd[j];
            }
        }
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            const R* v = u + k * vs;
            R lv = R(0), rv = R(0);
#pragma unroll
            for (int j = 0; j < ORDER; ++j) {
                // both rows for every shift, selected without divergence
                R cl = R(0), cr = R(0);
#pragma unroll
                for (int s = 0; s < ORDER; ++s) {
                    if (s == shift) {
                        cl = R(EnoC<ORDER>::c(s, j));
                        cr = R(EnoC<ORDER>::c(s + 1, j));
                    }
                }
                const R value = v[(j - shift) * ds];
                lv = mac(cl, value, lv);
                rv = mac(cr, value, rv);
            }
            left[k] = lv;
            right[k] = rv;
        }
    }
}

}  // namespace GBFV_VARIANT_NS
}  // namespace gbfv
