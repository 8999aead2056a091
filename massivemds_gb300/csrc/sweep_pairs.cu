// Instances of the unordered-pair sweep (pair_kernel.cuh) -- FP32 pair math
// (FP32 mode), FP64 pair math over FP32-stored delta (DELTA_F32 mode) and over
// FP64-stored delta (default mode), P = 1..kPairMaxP (FP32) / kPairMaxP64 (FP64), truncation on/off -- and
// the host-side launch of the sweep and its finish kernel.
#include <type_traits>

#include "pair_kernel.cuh"
#include "sweep.h"

namespace mdsx {
namespace {

// MODE: 0 FP32 math, 1 FP64 math over FP32 delta, 2 FP64 math over FP64 delta.
template <int P, bool TRUNC, int MODE>
using MathOf = typename std::conditional<
    MODE == 0, PairMathF32For<P, TRUNC>,
    typename std::conditional<MODE == 1, PairMathF64<P, TRUNC, float>, PairMathF64<P, TRUNC, double>>::type>::type;

template <int P, bool TRUNC, int MODE>
constexpr int pair_smem_bytes() {
    using M = MathOf<P, TRUNC, MODE>;
    return PairShape<P, (int)sizeof(typename M::X), (int)sizeof(typename M::S)>::kSmemBytes;
}

int mode_index(Mode mode) { return mode == Mode::kF32 ? 0 : mode == Mode::kF64DeltaF32 ? 1 : 2; }

template <int P, bool TRUNC, int MODE>
cudaError_t pair_prepare() {
    static bool done = false;  // one engine thread at a time; idempotent if raced
    if (done) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(pair_kernel<P, TRUNC, MathOf<P, TRUNC, MODE>>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, pair_smem_bytes<P, TRUNC, MODE>());
    if (e == cudaSuccess) done = true;
    return e;
}

template <int P, bool TRUNC, int MODE>
cudaError_t pair_launch_one(const PairMaps& maps, const PairArgs& args, cudaStream_t stream) {
    using M = MathOf<P, TRUNC, MODE>;
    cudaError_t e = pair_prepare<P, TRUNC, MODE>();
    if (e != cudaSuccess) return e;
    pair_kernel<P, TRUNC, M><<<args.grid, kPairThreads, pair_smem_bytes<P, TRUNC, MODE>(), stream>>>(
        maps.a, maps.b, maps.xi, maps.xj, args);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    // the finish kernel as a programmatic dependent: launched while the sweep
    // drains, it waits in griddepcontrol.wait for the sweep's results
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)pair_finish_blocks<P, typename M::Part>(args.nc));
    cfg.blockDim = dim3(FinishShape<P, typename M::Part>::kThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, pair_finish_kernel<P, typename M::Part>, args);
}

template <int P, bool TRUNC, int MODE>
cudaError_t pair_occupancy_one(int* ctas) {
    cudaError_t e = pair_prepare<P, TRUNC, MODE>();
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas, pair_kernel<P, TRUNC, MathOf<P, TRUNC, MODE>>,
                                                         kPairThreads, pair_smem_bytes<P, TRUNC, MODE>());
}

template <int P, int MODE>
cudaError_t pair_launch_pm(bool trunc, const PairMaps& maps, const PairArgs& args, cudaStream_t stream) {
    return trunc ? pair_launch_one<P, true, MODE>(maps, args, stream)
                 : pair_launch_one<P, false, MODE>(maps, args, stream);
}

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

template <int P, int MODE>
cudaError_t pair_occupancy_pm(bool trunc, int* ctas) {
    return trunc ? pair_occupancy_one<P, true, MODE>(ctas) : pair_occupancy_one<P, false, MODE>(ctas);
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

cudaError_t pair_occupancy(int p, bool trunc, Mode mode, int* ctas_per_sm) {
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
                        cudaStream_t stream) {
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
