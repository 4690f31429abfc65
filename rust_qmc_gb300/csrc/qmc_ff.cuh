// qmc_ff.cuh -- float-float ("double-single") arithmetic for the FP64-class
// refresh on the FP32 pipe.
//
// A value is the unevaluated sum hi + lo of two FP32 numbers with
// |lo| <= ulp(hi)/2: a 48-bit significand with FP32's exponent range.  The
// GB300's FP64 units issue at 1/64 of the FP32 rate, so one float-float
// operation (5-11 FP32 instructions) costs a fraction of one FP64 operation
// while keeping ~2^-46 relative accuracy, far inside the walker path's
// 1e-6 Ha local-energy budget.
//
// Building blocks (error-free transformations):
//   TwoSum      Knuth, TAOCP vol. 2 (4.2.2): s + e == a + b exactly;
//   FastTwoSum  Dekker, Numer. Math. 18 (1971): the same for |a| >= |b|;
//   TwoProd     p + e == a * b exactly, e = fma(a, b, -p).
// Addition is the "sloppy" double-word sum and multiplication the
// FMA-based product of Dekker's paper, as collected in the double-double
// algorithms of Hida, Li & Bailey (QD library, ARITH-15, 2001).  Division,
// reciprocal and square roots take one Newton correction from the FP32
// hardware seed; exp uses a Cody-Waite reduction by ln 2, a 2^-5 scaling,
// a degree-6 Taylor polynomial and five squarings.  Every intrinsic below is
// an IEEE round-to-nearest FP32 operation (__fadd_rn etc.), which the
// compiler neither contracts nor reassociates.
#pragma once
#include <cuda_runtime.h>

namespace qmc {

struct ff {
    float hi, lo;
    ff() = default;
    __host__ __device__ constexpr ff(float h, float l) : hi(h), lo(l) {}
    __host__ __device__ constexpr ff(float f) : hi(f), lo(0.0f) {}
    __host__ __device__ constexpr ff(int i) : hi((float)i), lo(0.0f) {}
    __host__ __device__ constexpr ff(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
    __host__ __device__ explicit constexpr operator double() const { return (double)hi + (double)lo; }
    __host__ __device__ explicit constexpr operator float() const { return hi + lo; }
};

// ---- error-free transformations ---------------------------------------------
__device__ __forceinline__ ff ff_two_sum(float a, float b) {
    float s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return ff(s, e);
}
__device__ __forceinline__ ff ff_fast_two_sum(float a, float b) {
    float s = __fadd_rn(a, b);
    return ff(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ ff ff_two_prod(float a, float b) {
    float p = __fmul_rn(a, b);
    return ff(p, __fmaf_rn(a, b, -p));
}

// ---- arithmetic ----------------------------------------------------------------
__device__ __forceinline__ ff operator+(ff a, ff b) {
    ff s = ff_two_sum(a.hi, b.hi);
    float e = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
    return ff_fast_two_sum(s.hi, e);
}
__device__ __forceinline__ ff operator-(ff a) { return ff(-a.hi, -a.lo); }
__device__ __forceinline__ ff operator-(ff a, ff b) { return a + ff(-b.hi, -b.lo); }
__device__ __forceinline__ ff operator*(ff a, ff b) {
    ff p = ff_two_prod(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.lo, p.lo);
    e = __fmaf_rn(a.lo, b.hi, e);
    return ff_fast_two_sum(p.hi, e);
}
// product with a single FP32 factor
__device__ __forceinline__ ff ff_mul_f(ff a, float b) {
    ff p = ff_two_prod(a.hi, b);
    return ff_fast_two_sum(p.hi, __fmaf_rn(a.lo, b, p.lo));
}
// a / b: quotient of the leading parts, then one remainder correction.
__device__ __forceinline__ ff operator/(ff a, ff b) {
    const float x = __frcp_rn(b.hi);
    const float q1 = __fmul_rn(a.hi, x);
    ff r = a - ff_mul_f(b, q1);
    const float q2 = __fmul_rn(r.hi, x);
    return ff_fast_two_sum(q1, q2);
}
__device__ __forceinline__ ff& operator+=(ff& a, ff b) { return a = a + b; }
__device__ __forceinline__ ff& operator-=(ff& a, ff b) { return a = a - b; }
__device__ __forceinline__ ff& operator*=(ff& a, ff b) { return a = a * b; }
__device__ __forceinline__ ff& operator/=(ff& a, ff b) { return a = a / b; }

__device__ __forceinline__ bool operator<(ff a, ff b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool operator>(ff a, ff b) { return b < a; }
__device__ __forceinline__ bool operator<=(ff a, ff b) { return !(b < a); }
__device__ __forceinline__ bool operator>=(ff a, ff b) { return !(a < b); }
__device__ __forceinline__ bool operator==(ff a, ff b) { return a.hi == b.hi && a.lo == b.lo; }
__device__ __forceinline__ bool operator!=(ff a, ff b) { return !(a == b); }

// The float-float overload joins the global FP32/FP64 ones (not hiding them).
using ::fabs;
__device__ __forceinline__ ff fabs(ff a) { return a.hi < 0.0f ? ff(-a.hi, -a.lo) : a; }

// ---- square roots and reciprocals (one Newton correction) ------------------
__device__ __forceinline__ ff frcp(ff b) {
    const float x = __frcp_rn(b.hi);
    ff e = ff(1.0f) - ff_mul_f(b, x);          // 1 - b x, ~2^-23
    return ff_fast_two_sum(x, __fmul_rn(e.hi, x));
}
__device__ __forceinline__ ff fsqrt(ff a) {
    if (!(a.hi > 0.0f)) return ff(0.0f);
    const float x = rsqrtf(a.hi);
    const float y = __fmul_rn(a.hi, x);        // sqrt(a) to ~2^-22
    ff d = a - ff_two_prod(y, y);              // a - y^2, exact product
    return ff_fast_two_sum(y, __fmul_rn(d.hi, __fmul_rn(0.5f, x)));
}
template <class T>
__device__ __forceinline__ T frsqrt(T x);
template <>
__device__ __forceinline__ ff frsqrt<ff>(ff a) {
    if (!(a.hi > 0.0f)) return ff(0.0f);
    const float x = rsqrtf(a.hi);
    ff t = ff_mul_f(ff_mul_f(a, x), x);        // a x^2 = 1 - e
    ff e = ff(1.0f) - t;
    return ff_fast_two_sum(x, __fmul_rn(e.hi, __fmul_rn(0.5f, x)));
}

// ---- exponential ----------------------------------------------------------------
// Cody-Waite reduction a = n ln2 + r with ln2 carried as a float pair,
// r scaled by 2^-5 (|r| <= 0.0109), e^r by the degree-6 Taylor series
// (truncation < 4e-18), then squared five times and scaled by 2^n.
// Arguments below -87 underflow FP32 and return 0.
__device__ __forceinline__ ff fexp(ff a) {
    if (a.hi < -87.0f) return ff(0.0f);
    constexpr double LN2 = 0.6931471805599453094172321;
    constexpr ff ln2 = ff(LN2);
    const float nf = rintf(__fmul_rn(a.hi, 1.44269504088896341f));
    const ff ln2n = ff_fast_two_sum(__fmul_rn(ln2.hi, nf), __fmaf_rn(ln2.hi, nf, -__fmul_rn(ln2.hi, nf)) +
                                                           __fmul_rn(ln2.lo, nf));
    ff r = a - ln2n;
    r = ff(__fmul_rn(r.hi, 0.03125f), __fmul_rn(r.lo, 0.03125f));
    // Horner: 1 + r (1 + r/2 (1 + r/3 (1 + r/4 (1 + r/5 (1 + r/6)))))
    constexpr ff c6 = ff(1.0 / 720.0), c5 = ff(1.0 / 120.0), c4 = ff(1.0 / 24.0), c3 = ff(1.0 / 6.0);
    ff p = c6;
    p = p * r + c5;
    p = p * r + c4;
    p = p * r + c3;
    p = p * r + ff(0.5f);
    p = p * r + ff(1.0f);
    p = p * r + ff(1.0f);
#pragma unroll
    for (int i = 0; i < 5; ++i) p = p * p;
    const int n = (int)nf;
    const float s = __int_as_float((n + 127) << 23);   // 2^n, n in [-126, 127]
    return ff(__fmul_rn(p.hi, s), __fmul_rn(p.lo, s));
}

// A running product kept as mantissa * 2^e: the mantissa is brought back to
// [0.5, 1) by exact power-of-two multiplies read off its exponent bits.
// Zero, subnormal, infinite and NaN mantissas are left unchanged.
__device__ __forceinline__ void ff_rescale(ff& m, int& e) {
    const int be = (__float_as_int(m.hi) >> 23) & 0xff;
    if (be == 0 || be == 0xff) return;
    const int k = be - 126;                      // in [-125, 128]
    const int k1 = k / 2, k2 = k - k1;           // two normal factors 2^-k1, 2^-k2
    const float s1 = __int_as_float((127 - k1) << 23), s2 = __int_as_float((127 - k2) << 23);
    m = ff(__fmul_rn(__fmul_rn(m.hi, s1), s2), __fmul_rn(__fmul_rn(m.lo, s1), s2));
    e += k;
}

// Float-float values in memory as float2 (hi, lo).
__device__ __forceinline__ void ff_store(float2* p, ff v) { *p = make_float2(v.hi, v.lo); }
__device__ __forceinline__ ff ff_load(const float2* p) {
    const float2 t = *p;
    return ff(t.x, t.y);
}

// Warp shuffle of a float-float value (two FP32 shuffles).
__device__ __forceinline__ ff wshfl(ff v, int src) {
    return ff(__shfl_sync(0xffffffffu, v.hi, src), __shfl_sync(0xffffffffu, v.lo, src));
}
__device__ __forceinline__ ff shfl_xor(ff v, int m) {
    return ff(__shfl_xor_sync(0xffffffffu, v.hi, m), __shfl_xor_sync(0xffffffffu, v.lo, m));
}

}  // namespace qmc
