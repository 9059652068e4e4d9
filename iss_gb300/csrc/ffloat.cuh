// Float-float ("double-float") arithmetic: a value is the unevaluated sum
// hi + lo of two floats, about 48 significant bits.  The error-free
// transformations are Knuth's two-sum and the FMA two-product (Dekker 1971);
// the compound operations follow Hida, Li and Bailey's double-double
// algorithms (QD library, 2001) carried over to float pairs.
//
// Used where the reference computes in double on float data and rounds the
// result back to float: the float-float result rounds to the same float as
// the double one unless the exact value lies within about 2^-46 (relative) of
// a float rounding boundary.  The multiplications use explicit fmaf, so the
// transformations stay exact in a translation unit built with --fmad=false.
#pragma once

#include <cuda_runtime.h>

namespace iss {

struct ff {
    float hi, lo;
};

__device__ __forceinline__ ff ff_of(float a) { return ff{a, 0.0f}; }

__device__ __forceinline__ ff ff_two_sum(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    return ff{s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ ff ff_quick_two_sum(float a, float b) {
    const float s = a + b;
    return ff{s, b - (s - a)};
}
__device__ __forceinline__ ff ff_two_prod(float a, float b) {
    const float p = a * b;
    return ff{p, fmaf(a, b, -p)};
}

__device__ __forceinline__ ff ff_add(ff a, ff b) {
    ff s = ff_two_sum(a.hi, b.hi);
    const ff t = ff_two_sum(a.lo, b.lo);
    s.lo += t.hi;
    s = ff_quick_two_sum(s.hi, s.lo);
    s.lo += t.lo;
    return ff_quick_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ ff ff_neg(ff a) { return ff{-a.hi, -a.lo}; }
__device__ __forceinline__ ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }

__device__ __forceinline__ ff ff_mul(ff a, ff b) {
    ff p = ff_two_prod(a.hi, b.hi);
    p.lo = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, p.lo));
    return ff_quick_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ ff ff_mul_f(ff a, float b) {
    ff p = ff_two_prod(a.hi, b);
    p.lo = fmaf(a.lo, b, p.lo);
    return ff_quick_two_sum(p.hi, p.lo);
}

// a / b: three float quotient digits, the long-division scheme of the QD
// library's accurate division
__device__ __forceinline__ ff ff_div(ff a, ff b) {
    const float q1 = a.hi / b.hi;
    ff r = ff_sub(a, ff_mul_f(b, q1));
    const float q2 = r.hi / b.hi;
    r = ff_sub(r, ff_mul_f(b, q2));
    const float q3 = r.hi / b.hi;
    const ff q = ff_quick_two_sum(q1, q2);
    return ff_add(q, ff_of(q3));
}

// sqrt(a), a > 0: one Newton step from the float root (Karp-Markstein form)
__device__ __forceinline__ ff ff_sqrt(ff a) {
    const float x = sqrtf(a.hi);
    const ff r = ff_sub(a, ff_two_prod(x, x));
    return ff_add(ff_of(x), ff_of(r.hi / (2.0f * x)));
}

// the nearest float of hi + lo (one correctly rounded float addition)
__device__ __forceinline__ float ff_to_float(ff a) { return a.hi + a.lo; }

}  // namespace iss
