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
// hardware seed; exp is table-driven (Tang, ACM TOMS 15 (1989)): a
// Cody-Waite reduction by ln2/32, a 32-entry table of 2^(j/32) and a short
// polynomial, with relative error below 5e-13.  Every intrinsic below is
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
// acc += c x without renormalising (a Dot2 step, Ogita, Rump & Oishi, SIAM J.
// Sci. Comput. 26 (2005)): the leading parts are summed error-free and every
// error term gathers in acc.lo; ff_norm(acc) after the last step gives a
// float pair as accurate as a float-float dot product.
__device__ __forceinline__ void ff_fma_lazy(ff& acc, ff c, ff x) {
    const float p = __fmul_rn(c.hi, x.hi);
    float pe = __fmaf_rn(c.hi, x.hi, -p);
    pe = __fmaf_rn(c.hi, x.lo, pe);
    pe = __fmaf_rn(c.lo, x.hi, pe);
    const ff s = ff_two_sum(acc.hi, p);
    acc.hi = s.hi;
    acc.lo = __fadd_rn(acc.lo, __fadd_rn(s.lo, pe));
}
__device__ __forceinline__ ff ff_norm(ff a) { return ff_fast_two_sum(a.hi, a.lo); }

// acc += c x for any compute type: the lazy float-float step for ff (close
// with macc_norm), a plain multiply-add otherwise.
template <class T>
__device__ __forceinline__ void macc(T& acc, T c, T x) { acc += c * x; }
__device__ __forceinline__ void macc(ff& acc, ff c, ff x) { ff_fma_lazy(acc, c, x); }
template <class T>
__device__ __forceinline__ T macc_norm(T a) { return a; }
__device__ __forceinline__ ff macc_norm(ff a) { return ff_norm(a); }

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

// Leading part as a float (pivot choices and other comparisons that need no
// more than FP32 resolution).
__device__ __forceinline__ float lead(ff a) { return a.hi; }
__device__ __forceinline__ float lead(float a) { return a; }
__device__ __forceinline__ float lead(double a) { return (float)a; }

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
// Table-driven (Tang 1989): a = (32 k + j) ln2/32 + r with |r| <= ln2/64,
// ln2/32 carried as a float pair; e^a = 2^k 2^(j/32) e^r.  e^r = 1 + r +
// r^2/2 + tail: r^2/2 as a float pair, tail = r^3/6 + r^4/24 + r^5/120 in
// FP32 (|tail| < 2e-7, so its rounding is below 2^-46); the truncated r^6/720
// is < 2e-15.  The table entries are 2^(j/32) rounded to float pairs.
// Arguments below -87 underflow FP32 and return 0.
__device__ const ff kExp2Frac[32] = {
    ff(1.0), ff(1.0218971486541166), ff(1.0442737824274138), ff(1.0671404006768237),
    ff(1.0905077326652577), ff(1.1143867425958924), ff(1.1387886347566916), ff(1.1637248587775775),
    ff(1.189207115002721), ff(1.215247359980469), ff(1.241857812073484), ff(1.2690509571917332),
    ff(1.2968395546510096), ff(1.3252366431597413), ff(1.3542555469368927), ff(1.383909881963832),
    ff(1.4142135623730951), ff(1.4451808069770467), ff(1.4768261459394993), ff(1.5091644275934228),
    ff(1.5422108254079407), ff(1.5759808451078865), ff(1.6104903319492543), ff(1.6457554781539649),
    ff(1.681792830507429), ff(1.7186192981224779), ff(1.7562521603732995), ff(1.7947090750031072),
    ff(1.8340080864093424), ff(1.8741676341103), ff(1.9152065613971474), ff(1.9571441241754002),
};

__device__ __forceinline__ ff fexp(ff a) {
    if (a.hi < -87.0f) return ff(0.0f);
    constexpr ff ln2_32 = ff(0.02166084939249829);          // ln(2) / 32
    const float nf = rintf(__fmul_rn(a.hi, 46.166241308446828f));
    const ff p = ff_two_prod(ln2_32.hi, nf);
    const ff t = ff_fast_two_sum(p.hi, __fmaf_rn(ln2_32.lo, nf, p.lo));
    const ff r = a - t;
    // r^2 / 2 (unnormalised pair) and the FP32 tail r^3 (1/6 + r/24 + r^2/120)
    const ff q = ff_two_prod(r.hi, r.hi);
    const ff h = ff(__fmul_rn(q.hi, 0.5f), __fmul_rn(__fmaf_rn(2.0f * r.hi, r.lo, q.lo), 0.5f));
    const float poly = __fmaf_rn(r.hi, __fmaf_rn(r.hi, 1.0f / 60.0f, 1.0f / 12.0f), 1.0f / 3.0f);
    const float tail = __fmul_rn(__fmul_rn(h.hi, r.hi), poly);
    ff s = h + ff(tail);
    s = r + s;
    s = ff(1.0f) + s;
    const int n = (int)nf;
    const ff m = s * kExp2Frac[n & 31];
    const float sc = __int_as_float(((n >> 5) + 127) << 23);   // 2^k, k in [-126, 127]
    return ff(__fmul_rn(m.hi, sc), __fmul_rn(m.lo, sc));
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
