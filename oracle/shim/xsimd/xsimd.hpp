// Test scaffolding, not product code.
//
// The MassiveMDS CPU engine includes xsimd unconditionally
// (src/NewMultiDimensionalScaling.hpp:16, src/CDF.h:7) and calls xsimd::exp on
// its scalar path (src/NewMultiDimensionalScaling.hpp:440). For the scalar
// (NoSimd) engines that is plain libm exp, which is all this stand-in gives.
#pragma once
#include <cmath>

namespace xsimd {
using std::exp;
}  // namespace xsimd
