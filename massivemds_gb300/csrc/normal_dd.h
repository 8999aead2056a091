// log Phi(z) and the ratio H(z) = phi(z) / Phi(z) in double-float for z >= 0,
// the two normal-tail quantities the truncated sweep needs (the likelihood term
// and the gradient's truncation term), from Taylor expansions about the grid
// points z_k = k / 32, k = 0 .. kNormalDDEntries - 1 (z up to 8.5):
//
//   L(z_k + u) = log Phi(z_k + u) = sum_{m=0..6} l_m u^m
//   H(z_k + u) = phi / Phi        = sum_{m=0..6} h_m u^m,   |u| <= 1/64.
//
// The coefficients follow from the definitions: L' = H, and H satisfies
// H' = -z H - H^2 (differentiate phi / Phi with phi' = -z phi), so with
// z = z_k + u the series coefficients obey
//   (m + 1) h_{m+1} = -z_k h_m - h_{m-1} - sum_{i=0..m} h_i h_{m-i},   h_{-1} = 0,
//   l_{m+1} = h_m / (m + 1),
// from h_0 = phi(z_k) / Phi(z_k) and l_0 = log Phi(z_k) = log1p(-Q(z_k)). The
// three leading coefficients of each series are kept in double-float, the
// others in FP32 (their terms are below 4e-6 in magnitude). Beyond the grid
// (z > 8.5 + 1/64) |log Phi| < 1e-17 and H < 1e-16 are returned as 0.
//
// The table is computed on the host from the C library's erfc, exp and log1p in
// long double (normal_dd_table) and copied to shared memory by each CTA. The
// FP64 pair math uses the same series in double (normal_f64_table, normal_f64).
#pragma once

#include <cmath>
#include <cstring>

#include "dd.h"

namespace mdsx {

constexpr int kNormalDDPerUnit = 32;     // grid points per unit of z
constexpr int kNormalDDEntries = 273;    // z_k = 0 .. 8.5
constexpr int kNormalDDStride = 20;      // floats per entry (five 16-byte groups)
constexpr int kNormalDDFloats = kNormalDDEntries * kNormalDDStride;

constexpr int kNormalTerms = 7;           // coefficients per series
constexpr int kNormalF64Stride = 16;      // doubles per entry of the FP64 table: l0..l6, z_k, h0..h6, 0
constexpr int kNormalF64Doubles = kNormalDDEntries * kNormalF64Stride;

// The series coefficients l_m, h_m about z_k = k / 32 (long double).
inline void normal_series(int k, long double (&l)[kNormalTerms], long double (&h)[kNormalTerms]) {
    const long double inv_sqrt_2pi = 0.398942280401432677939946059934381868L;
    const long double z = (long double)k / kNormalDDPerUnit;
    const long double phi = inv_sqrt_2pi * std::exp(-0.5L * z * z);
    const long double q = 0.5L * std::erfc(z / std::sqrt(2.0L));
    h[0] = phi / (1.0L - q);
    for (int m = 0; m + 1 < kNormalTerms; ++m) {
        long double conv = 0.0L;
        for (int i = 0; i <= m; ++i) conv += h[i] * h[m - i];
        h[m + 1] = (-z * h[m] - (m > 0 ? h[m - 1] : 0.0L) - conv) / (long double)(m + 1);
    }
    l[0] = std::log1p(-q);
    for (int m = 1; m < kNormalTerms; ++m) l[m] = h[m - 1] / (long double)m;
}

// Entry layout (floats): l0 (hi, lo), l1 (hi, lo), l2 (hi, lo), l3, l4, l5, l6,
// h0 (hi, lo), h1 (hi, lo), h2 (hi, lo), h3, h4, h5, h6.
inline void normal_dd_table(float* out) {
    constexpr int M = kNormalTerms;
    for (int k = 0; k < kNormalDDEntries; ++k) {
        long double l[M], h[M];
        normal_series(k, l, h);
        float* t = out + k * kNormalDDStride;
        for (int m = 0; m < 3; ++m) {
            const dd lm = dd_from_double((double)l[m]);
            const dd hm = dd_from_double((double)h[m]);
            t[2 * m] = lm.hi;
            t[2 * m + 1] = lm.lo;
            t[10 + 2 * m] = hm.hi;
            t[10 + 2 * m + 1] = hm.lo;
        }
        for (int m = 3; m < M; ++m) {
            t[m + 3] = (float)l[m];
            t[m + 13] = (float)h[m];
        }
    }
}

// log Phi(z) and phi(z) / Phi(z) for a double-float z >= 0 from the table `tab`.
__host__ __device__ __forceinline__ void normal_dd(dd z, const float* tab, dd& log_cdf, dd& ratio) {
    const int k = (int)fmaf(z.hi, (float)kNormalDDPerUnit, 0.5f);
    if (k >= kNormalDDEntries) {
        log_cdf = dd_of(0.0f);
        ratio = dd_of(0.0f);
        return;
    }
    const float* t = tab + k * kNormalDDStride;
    // z_hi - z_k is exact (Sterbenz: z_k / 2 <= z_hi <= 2 z_k for k >= 1)
    const dd u = two_sum(z.hi - (float)k * (1.0f / kNormalDDPerUnit), z.lo);
    float r = fmaf(fmaf(fmaf(t[9], u.hi, t[8]), u.hi, t[7]), u.hi, t[6]);
    dd p = dd_add(dd_of(t[4], t[5]), dd_mul_f(u, r));
    p = dd_fma(u, p, dd_of(t[2], t[3]));
    log_cdf = dd_fma(u, p, dd_of(t[0], t[1]));
    r = fmaf(fmaf(fmaf(t[19], u.hi, t[18]), u.hi, t[17]), u.hi, t[16]);
    p = dd_add(dd_of(t[14], t[15]), dd_mul_f(u, r));
    p = dd_fma(u, p, dd_of(t[12], t[13]));
    ratio = dd_fma(u, p, dd_of(t[10], t[11]));
}

inline void normal_f64_table(double* out) {
    for (int k = 0; k < kNormalDDEntries; ++k) {
        long double l[kNormalTerms], h[kNormalTerms];
        normal_series(k, l, h);
        double* t = out + k * kNormalF64Stride;
        for (int m = 0; m < kNormalF64Stride; ++m) t[m] = 0.0;
        for (int m = 0; m < kNormalTerms; ++m) {
            t[m] = (double)l[m];
            t[8 + m] = (double)h[m];
        }
        t[7] = (double)k / kNormalDDPerUnit;
    }
}

// The grid index k = round(32 z) for 0 <= z < 8.5 + 1/64, by adding 1.5 * 2^52:
// the sum's low word then holds k, with no FP64 conversion instruction.
__host__ __device__ __forceinline__ int normal_f64_index(double z) {
    const double t = fma(z, (double)kNormalDDPerUnit, 6755399441055744.0);
#ifdef __CUDA_ARCH__
    return __double2loint(t);
#else
    unsigned long long b;
    std::memcpy(&b, &t, sizeof b);
    return (int)(unsigned)(b & 0xffffffffull);
#endif
}

// log Phi(z) and phi(z) / Phi(z) in FP64 for z >= 0 from the table `tab`
// (Horner in double; within 2e-16 of the exact values, tests/dd_check.cpp).
__host__ __device__ __forceinline__ void normal_f64(double z, const double* tab, double& log_cdf, double& ratio) {
    if (!(z < 8.5 + 1.0 / (2 * kNormalDDPerUnit))) {  // beyond the grid (or NaN)
        log_cdf = 0.0;
        ratio = 0.0;
        return;
    }
    const double* t = tab + normal_f64_index(z) * kNormalF64Stride;
    const double u = z - t[7];  // z - z_k, exact (Sterbenz)
    log_cdf = fma(fma(fma(fma(fma(fma(t[6], u, t[5]), u, t[4]), u, t[3]), u, t[2]), u, t[1]), u, t[0]);
    ratio = fma(fma(fma(fma(fma(fma(t[14], u, t[13]), u, t[12]), u, t[11]), u, t[10]), u, t[9]), u, t[8]);
}

}  // namespace mdsx
