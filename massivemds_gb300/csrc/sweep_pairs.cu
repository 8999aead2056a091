// Instances of the unordered-pair sweep (pair_kernel.cuh) -- FP32 pair math
// (FP32 mode), FP64 pair math over FP32-stored delta (DELTA_F32 mode) and over
// FP64-stored delta (default mode), P = 1..kPairMaxP (FP32) / kPairMaxP64 (FP64), truncation on/off -- and
// the host-side dispatch of the sweep and its finish kernel. The double-float
// pair math is instantiated in sweep_pairs_dd.cu.
#include "pair_launch.cuh"

namespace mdsx {
namespace {

int mode_index(Mode mode) { return mode == Mode::kF32 ? 0 : mode == Mode::kF64DeltaF32 ? 1 : 2; }

template <int P>
cudaError_t pair_launch_p(bool trunc, int mode, const PairMaps& maps, const PairArgs& args, cudaStream_t stream) {
    if constexpr (P > kPairMaxP64) {
        if (mode != 0) return cudaErrorInvalidValue;
        return pair_launch_pm<P, 0>(trunc, maps, args, stream);
    } else {
        switch (mode) {
            case 0: return pair_launch_pm<P, 0>(trunc, maps, args, stream);
            case 1: return pair_launch_pm<P, 1>(trunc, maps, args, stream);
            default: return pair_launch_pm<P, 2>(trunc, maps, args, stream);
        }
    }
}

template <int P>
cudaError_t pair_occupancy_p(bool trunc, int mode, int* ctas) {
    if constexpr (P > kPairMaxP64) {
        if (mode != 0) return cudaErrorInvalidValue;
        return pair_occupancy_pm<P, 0>(trunc, ctas);
    } else {
        switch (mode) {
            case 0: return pair_occupancy_pm<P, 0>(trunc, ctas);
            case 1: return pair_occupancy_pm<P, 1>(trunc, ctas);
            default: return pair_occupancy_pm<P, 2>(trunc, ctas);
        }
    }
}

}  // namespace

bool pair_built(Mode mode, int p) { return p >= 1 && p <= (mode == Mode::kF32 ? kPairMaxP : kPairMaxP64); }

cudaError_t pair_occupancy(int p, bool trunc, Mode mode, int* ctas_per_sm, bool dd) {
    if (dd) return pair_occupancy_dd(p, trunc, mode == Mode::kF64DeltaF32, ctas_per_sm);
    const int m = mode_index(mode);
    switch (p) {
        case 1: return pair_occupancy_p<1>(trunc, m, ctas_per_sm);
        case 2: return pair_occupancy_p<2>(trunc, m, ctas_per_sm);
        case 3: return pair_occupancy_p<3>(trunc, m, ctas_per_sm);
        case 4: return pair_occupancy_p<4>(trunc, m, ctas_per_sm);
        case 5: return pair_occupancy_p<5>(trunc, m, ctas_per_sm);
        case 6: return pair_occupancy_p<6>(trunc, m, ctas_per_sm);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t pair_launch(int p, bool trunc, Mode mode, const PairMaps& maps, const PairArgs& args,
                        cudaStream_t stream, bool dd) {
    if (dd) return pair_launch_dd(p, trunc, mode == Mode::kF64DeltaF32, maps, args, stream);
    const int m = mode_index(mode);
    switch (p) {
        case 1: return pair_launch_p<1>(trunc, m, maps, args, stream);
        case 2: return pair_launch_p<2>(trunc, m, maps, args, stream);
        case 3: return pair_launch_p<3>(trunc, m, maps, args, stream);
        case 4: return pair_launch_p<4>(trunc, m, maps, args, stream);
        case 5: return pair_launch_p<5>(trunc, m, maps, args, stream);
        case 6: return pair_launch_p<6>(trunc, m, maps, args, stream);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace mdsx
