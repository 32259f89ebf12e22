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
using ::fma;
using ::fmax;
using ::fmin;
using ::sqrt;
using std::isfinite;

// float -> double by bit construction for normal floats: GB300 executes the
// F2F conversions on its FP64 pipe (1/64 of the FP32 rate), so the
// conversions at the edges of the double-float arithmetic are built from
// integer operations instead. Zero keeps its sign; subnormal, infinite and NaN
// floats take the conversion instruction.
__device__ __forceinline__ double df_widen(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xffu;
    if (e - 1u < 254u)
        return __longlong_as_double((long long)(((unsigned long long)(u & 0x80000000u) << 32) |
                                                ((unsigned long long)(e + (1023u - 127u)) << 52) |
                                                ((unsigned long long)(u & 0x7fffffu) << 29)));
    if ((u & 0x7fffffffu) == 0u) return __longlong_as_double((long long)((unsigned long long)u << 32));
    return (double)f;
}

struct dfloat {
    float hi, lo;
    __device__ __forceinline__ dfloat() : hi(0.f), lo(0.f) {}
    __device__ __forceinline__ dfloat(float h, float l) : hi(h), lo(l) {}
    __device__ __forceinline__ dfloat(int v) : hi((float)v), lo(0.f) {}
    __device__ __forceinline__ dfloat(float v) : hi(v), lo(0.f) {}
    // Split of a double from its bit pattern: hi takes the leading 24
    // significant bits (truncated), lo the remaining 29 bits rounded to 24,
    // then one renormalisation. The tail is assembled from two exact float
    // subtractions: a float with a fixed exponent field and k in its mantissa
    // field, minus the bare power of two, is k times that power's ulp. The
    // pair carries the double to 2^-48 relative, like a rounding split.
    // Doubles outside [2^-80, 2^128) take the conversion instructions.
    __device__ __forceinline__ explicit dfloat(double v) {
        const unsigned long long b = (unsigned long long)__double_as_longlong(v);
        const unsigned hw = (unsigned)(b >> 32), lw = (unsigned)b;
        const int E = (int)((hw >> 20) & 0x7ffu) - 1023;
        if (E >= -80 && E <= 127) {
            const unsigned sign = hw & 0x80000000u;
            const float h = __uint_as_float(sign | ((unsigned)(E + 127) << 23) | ((hw & 0xfffffu) << 3) | (lw >> 29));
            const unsigned r = lw & 0x1fffffffu;
            const unsigned xa = (unsigned)(E - 23 + 127) << 23, xb = (unsigned)(E - 46 + 127) << 23;
            const float pa = __fsub_rn(__uint_as_float(xa | (r >> 6)), __uint_as_float(xa));
            const float pb = __fsub_rn(__uint_as_float(xb | ((r & 63u) << 17)), __uint_as_float(xb));
            const float l = __uint_as_float(__float_as_uint(__fadd_rn(pa, pb)) | sign);
            hi = __fadd_rn(h, l);
            lo = __fsub_rn(l, __fsub_rn(hi, h));
        } else if ((b << 1) == 0ull) {
            hi = __uint_as_float(hw);  // signed zero
            lo = 0.f;
        } else {
            hi = __double2float_rn(v);
            lo = __double2float_rn(v - (double)hi);
        }
    }
    // hi + lo is exact in double (48 significant bits at most)
    __device__ __forceinline__ explicit operator double() const { return df_widen(hi) + df_widen(lo); }
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
__device__ __forceinline__ dfloat fma(const dfloat& a, const dfloat& b, const dfloat& c) { return a * b + c; }

}  // namespace gbfv
