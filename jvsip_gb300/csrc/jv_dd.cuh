// jv_dd.cuh -- double-float arithmetic for the FP64 form of the row kernel.
//
// A value is the unevaluated sum hi + lo of two floats with |lo| <= ulp(hi)/2
// (48 significant bits).  The error-free transformations are the published
// ones: TwoSum (Knuth, TAOCP vol. 2, 4.2.2, theorem B) and FastTwoSum
// (Dekker 1971) for sums, TwoProduct with a fused multiply-add (Ogita, Rump
// and Oishi 2005) for products; addition is the "sloppy" double-double sum
// (error bounded by a small multiple of u*(|a| + |b|) with u = 2^-48), which is
// the bound an FFT's error analysis uses.  Everything runs on the FP32 and
// integer pipes: conversions from and to double work on the bit patterns,
// with a per-row power-of-two shift so that a row's largest element maps to
// [1, 2) and no row can overflow float's exponent range.
#pragma once

#include <stdint.h>

namespace jv {

struct dd {
    float hi, lo;
    __host__ __device__ constexpr dd() : hi(0.f), lo(0.f) {}
    // split of a double constant (folded at compile time for literals)
    __host__ __device__ constexpr dd(double v) : hi((float)v), lo((float)(v - (double)(float)v)) {}
    __host__ __device__ constexpr dd(float h, float l) : hi(h), lo(l) {}
};

struct __align__(16) cdd {
    dd x, y;
};

__device__ __forceinline__ dd dd_fast_two_sum(float a, float b) {  // |a| >= |b|
    const float s = __fadd_rn(a, b);
    return dd(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ void dd_two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ dd operator+(dd a, dd b) {
    float s, e;
    dd_two_sum(a.hi, b.hi, s, e);
    e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    return dd_fast_two_sum(s, e);
}
__device__ __forceinline__ dd operator-(dd a) { return dd(-a.hi, -a.lo); }
__device__ __forceinline__ dd operator-(dd a, dd b) { return a + (-b); }
__device__ __forceinline__ dd operator*(dd a, dd b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return dd_fast_two_sum(p, e);
}
__device__ __forceinline__ dd &operator*=(dd &a, dd b) {
    a = a * b;
    return a;
}

// ---- conversions on bit patterns
// biased exponent of a double (0 for zero and subnormals)
__device__ __forceinline__ int dd_exp_of(double x) {
    return (int)((__double_as_longlong(x) >> 52) & 0x7FF);
}

// x * 2^-sh as a double-float: hi = the leading 24 significant bits, lo = the
// next 29 rounded to 24; elements below 2^-126 after the shift become 0 (they
// lie 2^126 below the row's largest element)
__device__ __forceinline__ dd dd_from_double(double x, int sh) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(x);
    const int E = (int)((u >> 52) & 0x7FF);
    const int e = E - 1023 - sh;  // unbiased exponent after the shift
    if (E == 0 || e < -126) return dd(0.f, 0.f);
    const unsigned sign = (unsigned)(u >> 32) & 0x80000000u;
    const unsigned hb = sign | ((unsigned)(e + 127) << 23) | ((unsigned)(u >> 29) & 0x7FFFFFu);
    const unsigned rem = (unsigned)(u & ((1ull << 29) - 1));
    float lo = 0.f;
    if (rem != 0 && e >= -74) {
        // rem * 2^(e - 52): the integer rounded to float, then the exact power of two
        lo = __uint2float_rn(rem) * __int_as_float((e - 52 + 127) << 23);
        lo = __int_as_float(__float_as_int(lo) | (int)sign);
    }
    return dd(__int_as_float((int)hb), lo);
}

// float f * 2^sh as a double (exact; zero and subnormal floats give 0)
__device__ __forceinline__ double dd_float_to_double(float f, int sh) {
    const unsigned b = (unsigned)__float_as_int(f);
    const int ef = (int)((b >> 23) & 0xFF);
    if (ef == 0) return 0.0;
    const unsigned long long s = (unsigned long long)(b & 0x80000000u) << 32;
    const unsigned long long ed = (unsigned long long)(ef - 127 + 1023 + sh) << 52;
    const unsigned long long m = (unsigned long long)(b & 0x7FFFFFu) << 29;
    return __longlong_as_double((long long)(s | ed | m));
}

// (hi + lo) * 2^sh rounded to double
__device__ __forceinline__ double dd_to_double(dd v, int sh) {
    return __dadd_rn(dd_float_to_double(v.hi, sh), dd_float_to_double(v.lo, sh));
}

}  // namespace jv
