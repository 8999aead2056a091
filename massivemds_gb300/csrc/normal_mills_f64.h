// Generated by normal_mills_fit_f64.py: FP64 upper-tail normal approximation.
// Q(z) = phi(z) * P(min(z, 8.5)) / S(min(z, 8.5)), degree (6, 6), S(0) = 1;
// our weighted-minimax fit of the Mills ratio (Loeb + Lawson, 50 digits):
// max |Q_fit - Q| = 7.96e-16 in exact arithmetic on [0, 8.5],
// 9.44e-16 (at z = 0.019) evaluated in double on [0, 12];
// S > 0 on the grid: True; all coefficients positive: True.
#pragma once

#include <cmath>

namespace mdsx {

constexpr double kMillsClamp = 8.5;

// P(z) and S(z) for 0 <= z <= kMillsClamp (Horner, all coefficients positive).
__host__ __device__ inline void mills_ratio_f64(double z, double& num, double& den) {
    num = fma(fma(fma(fma(fma(fma(1.7496439111323296889e-8, z, 8.9410058782606006651e-4), z, 1.4796287351222376157e-2), z, 1.0881203656778555212e-1), z, 4.5009831768656056492e-1), z, 1.0492879481396186811), z, 1.2533141373154982789);
    den = fma(fma(fma(fma(fma(fma(8.9473674361989506807e-4, z, 1.4784957454783539226e-2), z, 1.0983841326799522443e-1), z, 4.6376650827836647323e-1), z, 1.1637437255968843161), z, 1.635095214459650678), z, 1.0);
}

}  // namespace mdsx
