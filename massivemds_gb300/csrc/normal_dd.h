// Upper normal tail Q(z) = 1 - Phi(z) and density phi(z) in double-float for
// z >= 0, from Taylor expansions about the grid points z_k = k / 32,
// k = 0 .. kNormalDDEntries - 1 (z up to 8.5):
//
//   Q(z_k + u)   = sum_{m=0..6} c_m u^m,  c_m = Q^(m)(z_k) / m!
//   phi(z_k + u) = sum_{m=0..6} e_m u^m,  e_m = phi^(m)(z_k) / m!
//
// with |u| <= 1/64 and, from the definitions, Q' = -phi and
// phi^(m)(z) = (-1)^m He_m(z) phi(z) (probabilists' Hermite polynomials). The
// truncation errors are below 3e-16 (Q) and 3e-15 (phi) in absolute value.
// The three leading coefficients of each expansion are kept in double-float,
// the others in FP32 (their terms are below 4e-6 in magnitude); evaluated, Q and
// phi are within 3e-14 of their exact values (tests/dd_check.cpp). Beyond the grid
// (z > 8.5 + 1/64) Q < 1e-17 and phi < 1e-16 are returned as 0.
//
// The table is computed on the host from the C library's erfc and exp in long
// double (normal_dd_table) and copied to shared memory by each CTA.
#pragma once

#include <cmath>

#include "dd.h"

namespace mdsx {

constexpr int kNormalDDPerUnit = 32;     // grid points per unit of z
constexpr int kNormalDDEntries = 273;    // z_k = 0 .. 8.5
constexpr int kNormalDDStride = 20;      // floats per entry (five 16-byte groups)
constexpr int kNormalDDFloats = kNormalDDEntries * kNormalDDStride;

// Entry layout (floats): c0 (hi, lo), c1 (hi, lo), c2 (hi, lo), c3, c4, c5, c6,
// e0 (hi, lo), e1 (hi, lo), e2 (hi, lo), e3, e4, e5, e6.
inline void normal_dd_table(float* out) {
    const long double inv_sqrt_2pi = 0.398942280401432677939946059934381868L;
    for (int k = 0; k < kNormalDDEntries; ++k) {
        const long double z = (long double)k / kNormalDDPerUnit;
        const long double phi = inv_sqrt_2pi * std::exp(-0.5L * z * z);
        // He_0 .. He_6 at z
        long double he[7];
        he[0] = 1.0L;
        he[1] = z;
        for (int m = 1; m < 6; ++m) he[m + 1] = z * he[m] - (long double)m * he[m - 1];
        long double fact[7];
        fact[0] = 1.0L;
        for (int m = 1; m < 7; ++m) fact[m] = fact[m - 1] * m;
        long double c[7], e[7];
        c[0] = 0.5L * std::erfc(z / std::sqrt(2.0L));
        // Q^(m) = -phi^(m-1) = -(-1)^(m-1) He_{m-1} phi
        for (int m = 1; m < 7; ++m) c[m] = ((m - 1) % 2 ? 1.0L : -1.0L) * he[m - 1] * phi / fact[m];
        for (int m = 0; m < 7; ++m) e[m] = (m % 2 ? -1.0L : 1.0L) * he[m] * phi / fact[m];
        float* t = out + k * kNormalDDStride;
        for (int m = 0; m < 3; ++m) {
            const dd cm = dd_from_double((double)c[m]);
            const dd em = dd_from_double((double)e[m]);
            t[2 * m] = cm.hi;
            t[2 * m + 1] = cm.lo;
            t[10 + 2 * m] = em.hi;
            t[10 + 2 * m + 1] = em.lo;
        }
        for (int m = 3; m < 7; ++m) t[m + 3] = (float)c[m];
        for (int m = 3; m < 7; ++m) t[m + 13] = (float)e[m];
    }
}

// Q(z) and phi(z) for a double-float z >= 0 from the table `tab`.
__host__ __device__ __forceinline__ void normal_dd(dd z, const float* tab, dd& q, dd& phi) {
    const int k = (int)fmaf(z.hi, (float)kNormalDDPerUnit, 0.5f);
    if (k >= kNormalDDEntries) {
        q = dd_of(0.0f);
        phi = dd_of(0.0f);
        return;
    }
    const float* t = tab + k * kNormalDDStride;
    // z_hi - z_k is exact (Sterbenz: z_k / 2 <= z_hi <= 2 z_k for k >= 1)
    const dd u = two_sum(z.hi - (float)k * (1.0f / kNormalDDPerUnit), z.lo);
    float r = fmaf(fmaf(fmaf(t[9], u.hi, t[8]), u.hi, t[7]), u.hi, t[6]);
    dd p = dd_add(dd_of(t[4], t[5]), dd_mul_f(u, r));
    p = dd_fma(u, p, dd_of(t[2], t[3]));
    q = dd_fma(u, p, dd_of(t[0], t[1]));
    r = fmaf(fmaf(fmaf(t[19], u.hi, t[18]), u.hi, t[17]), u.hi, t[16]);
    p = dd_add(dd_of(t[14], t[15]), dd_mul_f(u, r));
    p = dd_fma(u, p, dd_of(t[12], t[13]));
    phi = dd_fma(u, p, dd_of(t[10], t[11]));
}

}  // namespace mdsx
