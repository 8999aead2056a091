// Generated by normal_rational_fit.py; do not edit by hand.
//
// Upper normal tail Q(z) = phi(z) * P(z) / S(z) for z >= 0, with
// P(z) = p0 + p1 z + p2 z^2 and S(z) = s0 + s1 z + s2 z^2 + z^3 (monic).
// Weighted minimax fit (Loeb iteration); max |Q - approx| = 9.411e-08 over z >= 0.
#pragma once

namespace mdsx {
constexpr double kTailMaxAbsError = 9.410603e-08;
constexpr double kTailP0 = 12.767006636102574;
constexpr double kTailP1 = 5.438272123097468;
constexpr double kTailP2 = 1.0191085229268808;
constexpr double kTailS0 = 10.186597158941739;
constexpr double kTailS1 = 12.46689382237852;
constexpr double kTailS2 = 5.666285483325529;
}  // namespace mdsx
