// Instances of the unordered-pair sweep with double-float pair math
// (PairMathDD, pair_kernel.cuh): over FP32-stored delta (MODE 3) and over
// double-float delta in 8-byte slots (MODE 4), P = 1..kPairMaxP64, truncation
// on/off.
#include "pair_launch.cuh"

namespace mdsx {
namespace {

template <int P>
cudaError_t launch_dd_p(bool trunc, bool delta_f32, const PairMaps& maps, const PairArgs& args,
                        cudaStream_t stream) {
    return delta_f32 ? pair_launch_pm<P, 3>(trunc, maps, args, stream) : pair_launch_pm<P, 4>(trunc, maps, args, stream);
}

template <int P>
cudaError_t occupancy_dd_p(bool trunc, bool delta_f32, int* ctas) {
    return delta_f32 ? pair_occupancy_pm<P, 3>(trunc, ctas) : pair_occupancy_pm<P, 4>(trunc, ctas);
}

}  // namespace

cudaError_t pair_occupancy_dd(int p, bool trunc, bool delta_f32, int* ctas_per_sm) {
    switch (p) {
        case 1: return occupancy_dd_p<1>(trunc, delta_f32, ctas_per_sm);
        case 2: return occupancy_dd_p<2>(trunc, delta_f32, ctas_per_sm);
        case 3: return occupancy_dd_p<3>(trunc, delta_f32, ctas_per_sm);
        case 4: return occupancy_dd_p<4>(trunc, delta_f32, ctas_per_sm);
        case 5: return occupancy_dd_p<5>(trunc, delta_f32, ctas_per_sm);
        case 6: return occupancy_dd_p<6>(trunc, delta_f32, ctas_per_sm);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t pair_launch_dd(int p, bool trunc, bool delta_f32, const PairMaps& maps, const PairArgs& args,
                           cudaStream_t stream) {
    switch (p) {
        case 1: return launch_dd_p<1>(trunc, delta_f32, maps, args, stream);
        case 2: return launch_dd_p<2>(trunc, delta_f32, maps, args, stream);
        case 3: return launch_dd_p<3>(trunc, delta_f32, maps, args, stream);
        case 4: return launch_dd_p<4>(trunc, delta_f32, maps, args, stream);
        case 5: return launch_dd_p<5>(trunc, delta_f32, maps, args, stream);
        case 6: return launch_dd_p<6>(trunc, delta_f32, maps, args, stream);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace mdsx
