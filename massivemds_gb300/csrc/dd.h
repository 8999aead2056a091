// Double-float arithmetic: a value is the unevaluated sum hi + lo of two FP32
// numbers with |lo| <= ulp(hi) / 2, about 48 significant bits, computed on the
// FP32 pipes. GB300 issues FP32 work at 64 times its FP64 rate, so FP64-accurate
// pair math is faster in this form than in FP64.
//
// Built from the classical error-free transformations: Knuth's TwoSum, Dekker's
// Fast2Sum and the FMA two-product (Dekker 1971; Ogita, Rump and Oishi 2005),
// with the "sloppy" double-word addition (one TwoSum, error about 2^-48 of the
// operands' magnitudes) that the double-double literature uses when operands do
// not cancel catastrophically. Results are within a few units of 2^-44 of the
// exact value for the operations below, far inside the 1e-10 / 1e-9 relative
// bars the FP64 modes are held to.
#pragma once

#include <cmath>

#if !defined(__CUDACC__) && !defined(__host__)
#define __host__
#endif
#if !defined(__CUDACC__) && !defined(__device__)
#define __device__
#endif
#if !defined(__CUDACC__) && !defined(__forceinline__)
#define __forceinline__ inline
#endif

namespace mdsx {

struct dd {
    float hi, lo;
};

__host__ __device__ __forceinline__ dd dd_of(float hi, float lo = 0.0f) {
    dd r;
    r.hi = hi;
    r.lo = lo;
    return r;
}

// Splits a double into hi = fl32(v) and lo = fl32(v - hi).
__host__ __device__ __forceinline__ dd dd_from_double(double v) {
    const float hi = (float)v;
    return dd_of(hi, (float)(v - (double)hi));
}

__host__ __device__ __forceinline__ double dd_to_double(dd a) { return (double)a.hi + (double)a.lo; }

// s + e = a + b exactly (Knuth).
__host__ __device__ __forceinline__ dd two_sum(float a, float b) {
    const float s = a + b;
    const float bv = s - a;
    const float e = (a - (s - bv)) + (b - bv);
    return dd_of(s, e);
}

// s + e = a + b exactly, given |a| >= |b| or a = 0 (Dekker).
__host__ __device__ __forceinline__ dd fast_two_sum(float a, float b) {
    const float s = a + b;
    return dd_of(s, b - (s - a));
}

// p + e = a * b exactly (FMA).
__host__ __device__ __forceinline__ dd two_prod(float a, float b) {
    const float p = a * b;
    return dd_of(p, fmaf(a, b, -p));
}

__host__ __device__ __forceinline__ dd dd_neg(dd a) { return dd_of(-a.hi, -a.lo); }

__host__ __device__ __forceinline__ dd dd_add(dd a, dd b) {
    const dd s = two_sum(a.hi, b.hi);
    return fast_two_sum(s.hi, s.lo + (a.lo + b.lo));
}

__host__ __device__ __forceinline__ dd dd_sub(dd a, dd b) { return dd_add(a, dd_neg(b)); }

// a + b for a float b.
__host__ __device__ __forceinline__ dd dd_add_f(dd a, float b) {
    const dd s = two_sum(a.hi, b);
    return fast_two_sum(s.hi, s.lo + a.lo);
}

__host__ __device__ __forceinline__ dd dd_mul(dd a, dd b) {
    const dd p = two_prod(a.hi, b.hi);
    return fast_two_sum(p.hi, fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, p.lo)));
}

// a * b for a float b.
__host__ __device__ __forceinline__ dd dd_mul_f(dd a, float b) {
    const dd p = two_prod(a.hi, b);
    return fast_two_sum(p.hi, fmaf(a.lo, b, p.lo));
}

__host__ __device__ __forceinline__ dd dd_sqr(dd a) {
    const dd p = two_prod(a.hi, a.hi);
    return fast_two_sum(p.hi, fmaf(a.hi + a.hi, a.lo, p.lo));
}

// acc += a * b and acc += a^2 for accumulators: the product's exact high part
// enters hi by TwoSum, and every error term gathers in lo without a
// renormalisation per step (the compensated dot product Dot2 of Ogita, Rump and
// Oishi 2005); dd_to_double reads such an accumulator as it stands. Over long
// sums lo's own rounding grows, so callers renormalise (dd_renorm) every few
// dozen terms: 20 000 terms so kept are within 1e-12 of sum |terms|, as with a
// dd_add per term (tests/dd_check.cpp).
__host__ __device__ __forceinline__ void dd_acc_fma(dd& acc, dd a, dd b) {
    const dd p = two_prod(a.hi, b.hi);
    const dd s = two_sum(acc.hi, p.hi);
    acc.hi = s.hi;
    acc.lo += s.lo + fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, p.lo));
}
__host__ __device__ __forceinline__ void dd_acc_sqr(dd& acc, dd a) {
    const dd p = two_prod(a.hi, a.hi);
    const dd s = two_sum(acc.hi, p.hi);
    acc.hi = s.hi;
    acc.lo += s.lo + fmaf(a.hi + a.hi, a.lo, p.lo);
}

// acc += a, with the same unnormalised accumulator as dd_acc_fma.
__host__ __device__ __forceinline__ void dd_acc_add(dd& acc, dd a) {
    const dd s = two_sum(acc.hi, a.hi);
    acc.hi = s.hi;
    acc.lo += s.lo + a.lo;
}

__host__ __device__ __forceinline__ dd dd_renorm(dd a) { return fast_two_sum(a.hi, a.lo); }

// c + a * b, rounded once to double-float.
__host__ __device__ __forceinline__ dd dd_fma(dd a, dd b, dd c) {
    const dd p = two_prod(a.hi, b.hi);
    const float plo = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, p.lo));
    const dd s = two_sum(c.hi, p.hi);
    return fast_two_sum(s.hi, s.lo + (c.lo + plo));
}

// FP32 seeds for the Newton steps below: the MUFU approximations on the device
// (relative error ~2^-23), the exact quotient on the host.
__host__ __device__ __forceinline__ float dd_rsqrt_seed(float x) {
#ifdef __CUDA_ARCH__
    float y;
    asm("rsqrt.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
#else
    return 1.0f / std::sqrt(x);
#endif
}

__host__ __device__ __forceinline__ float dd_rcp_seed(float x) {
#ifdef __CUDA_ARCH__
    float y;
    asm("rcp.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
#else
    return 1.0f / x;
#endif
}

// 1 / sqrt(a) for a > 0: one Newton step r0 (1 + e / 2), e = 1 - a r0^2 taken
// in double-float, from the FP32 estimate r0 (relative error ~2^-23 -> ~2^-45).
// a = 0 gives NaN (0 * inf), as the FP64 path's coincident points do.
__host__ __device__ __forceinline__ dd dd_rsqrt(dd a) {
    const float r0 = dd_rsqrt_seed(a.hi);
    const dd t = dd_mul(a, two_prod(r0, r0));  // ~1
    const float e = (1.0f - t.hi) - t.lo;
    return fast_two_sum(r0, r0 * (0.5f * e));
}

// a / b for b != 0: q1 = a_hi / b_hi from the FP32 seed, the remainder
// a - q1 b in double-float, and one correction q2 = remainder / b_hi.
__host__ __device__ __forceinline__ dd dd_div(dd a, dd b) {
    const float r0 = dd_rcp_seed(b.hi);
    const float q1 = a.hi * r0;
    const dd p = two_prod(q1, b.hi);
    const float rem = ((a.hi - p.hi) - p.lo) + fmaf(-q1, b.lo, a.lo);
    return fast_two_sum(q1, rem * r0);
}

// 1 / a for a != 0: one Newton step r0 (1 + e), e = 1 - a r0.
__host__ __device__ __forceinline__ dd dd_rcp(dd a) {
    const float r0 = dd_rcp_seed(a.hi);
    const dd t = dd_mul_f(a, r0);  // ~1
    const float e = (1.0f - t.hi) - t.lo;
    return fast_two_sum(r0, r0 * e);
}

}  // namespace mdsx
