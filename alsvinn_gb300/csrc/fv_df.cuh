// Double-float arithmetic: a value is the unevaluated sum hi + lo of two FP32
// numbers (|lo| <= ulp(hi)/2), about 48 significant bits, computed entirely on
// the FP32 pipes. GB300 issues FP64 at 1/64 of its FP32 rate, so the FP64
// state path evaluates its reconstruction and flux arithmetic in this type
// (roughly 1e-14 relative per operation) and keeps the Runge-Kutta update of
// the FP64 state in FP64.
//
// Algorithms: Dekker's two-product via FMA and Knuth's two-sum (error-free
// transformations), the "sloppy" double-float addition, one Newton-style
// correction for division and Karp's correction for the square root
// (Hida, Li, Bailey, "Library for double-double and quad-double arithmetic",
// 2001; Joldes, Muller, Popescu, "Tight and rigorous error bounds for basic
// building blocks of double-word arithmetic", 2017).
#pragma once
#include <cuda_runtime.h>

#include <cmath>

namespace gbfv {

// keep the float / double overloads visible next to the double-float ones
using ::fabs;
using ::fmax;
using ::fmin;
using ::sqrt;
using std::isfinite;

struct dfloat {
    float hi, lo;
    __device__ __forceinline__ dfloat() : hi(0.f), lo(0.f) {}
    __device__ __forceinline__ dfloat(float h, float l) : hi(h), lo(l) {}
    __device__ __forceinline__ dfloat(int v) : hi((float)v), lo(0.f) {}
    __device__ __forceinline__ dfloat(float v) : hi(v), lo(0.f) {}
    __device__ __forceinline__ explicit dfloat(double v) {
        hi = __double2float_rn(v);
        lo = __double2float_rn(v - (double)hi);
    }
    __device__ __forceinline__ explicit operator double() const { return (double)hi + (double)lo; }
    __device__ __forceinline__ dfloat& operator+=(const dfloat& b);
};

__device__ __forceinline__ dfloat df_quick_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float e = __fsub_rn(b, __fsub_rn(s, a));
    return dfloat(s, e);
}

__device__ __forceinline__ dfloat df_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return dfloat(s, e);
}

// "Sloppy" double-float addition: error below about 2^-44 (|a| + |b|). The
// accurate variant (two two-sums) bounds the error by the result instead; on
// the benchmark flows it changed the state error by less than a factor two
// (the ~2^-47 precision of the type itself dominates) for 30 % more time.
__device__ __forceinline__ dfloat operator+(const dfloat& a, const dfloat& b) {
    const dfloat s = df_two_sum(a.hi, b.hi);
    const float e = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
    return df_quick_two_sum(s.hi, e);
}

__device__ __forceinline__ dfloat operator-(const dfloat& a) { return dfloat(-a.hi, -a.lo); }

__device__ __forceinline__ dfloat operator-(const dfloat& a, const dfloat& b) { return a + (-b); }

__device__ __forceinline__ dfloat operator*(const dfloat& a, const dfloat& b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return df_quick_two_sum(p, e);
}

// 1/b to ~24 bits from the special-function unit
__device__ __forceinline__ float df_rcp_approx(float b) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(b));
    return r;
}

__device__ __forceinline__ dfloat operator/(const dfloat& a, const dfloat& b) {
    const float r = df_rcp_approx(b.hi);
    const float q1 = __fmul_rn(a.hi, r);
    // remainder a - q1 * b, its leading part exact through the FMA
    const float p = __fmul_rn(q1, b.hi);
    const float pe = __fmaf_rn(q1, b.hi, -p);
    const float rem = __fadd_rn(__fsub_rn(__fsub_rn(a.hi, p), pe), __fsub_rn(a.lo, __fmul_rn(q1, b.lo)));
    const float q2 = __fmul_rn(rem, r);
    // the first quotient is off by a few ulp of hi: one more correction
    const dfloat q = df_quick_two_sum(q1, q2);
    const dfloat qb = q * b;
    const dfloat d = a - qb;
    return q + dfloat(__fmul_rn(d.hi, r), 0.f);
}

__device__ __forceinline__ dfloat sqrt(const dfloat& a) {
    if (!(a.hi > 0.f)) return dfloat(sqrtf(a.hi), 0.f);  // 0, negative -> NaN, NaN
    float x;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(x) : "f"(a.hi));
    const float s = __fmul_rn(a.hi, x);
    // s^2 exactly as a double-float, then s + (a - s^2) * x / 2
    const float p = __fmul_rn(s, s);
    const float pe = __fmaf_rn(s, s, -p);
    const float d = __fadd_rn(__fsub_rn(__fsub_rn(a.hi, p), pe), a.lo);
    const dfloat r = df_quick_two_sum(s, __fmul_rn(d, __fmul_rn(0.5f, x)));
    // second correction for the few ulp the approximate rsqrt leaves
    const dfloat r2 = r * r;
    const dfloat e = a - r2;
    return r + dfloat(__fmul_rn(e.hi, __fmul_rn(0.5f, x)), 0.f);
}

__device__ __forceinline__ dfloat& dfloat::operator+=(const dfloat& b) {
    *this = *this + b;
    return *this;
}

__device__ __forceinline__ bool operator<(const dfloat& a, const dfloat& b) {
    return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo);
}
__device__ __forceinline__ bool operator>(const dfloat& a, const dfloat& b) { return b < a; }
__device__ __forceinline__ bool operator<=(const dfloat& a, const dfloat& b) { return !(b < a); }
__device__ __forceinline__ bool operator>=(const dfloat& a, const dfloat& b) { return !(a < b); }
__device__ __forceinline__ bool operator==(const dfloat& a, const dfloat& b) { return a.hi == b.hi && a.lo == b.lo; }

__device__ __forceinline__ dfloat fabs(const dfloat& a) { return a.hi < 0.f ? -a : a; }
// NaN operands follow fmax/fmin: the other operand wins
__device__ __forceinline__ dfloat fmax(const dfloat& a, const dfloat& b) {
    if (a.hi != a.hi) return b;
    if (b.hi != b.hi) return a;
    return a < b ? b : a;
}
__device__ __forceinline__ dfloat fmin(const dfloat& a, const dfloat& b) {
    if (a.hi != a.hi) return b;
    if (b.hi != b.hi) return a;
    return b < a ? b : a;
}
__device__ __forceinline__ bool isfinite(const dfloat& a) { return isfinite(a.hi); }

}  // namespace gbfv
