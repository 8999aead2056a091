// Instances of the unordered-pair sweep (pair_kernel.cuh) -- FP32 pair math
// (FP32 mode) and FP64 pair math over FP32-stored delta (DELTA_F32 mode), P = 1..kPairMaxP,
// truncation on/off -- and the host-side launch of the sweep and its finish kernel.
#include <type_traits>

#include "pair_kernel.cuh"
#include "sweep.h"

namespace mdsx {
namespace {

template <int P, bool TRUNC, bool F64>
using MathOf = typename std::conditional<F64, PairMathF64<P, TRUNC>, PairMathF32<P, TRUNC>>::type;

template <int P, bool TRUNC, bool F64>
constexpr int pair_smem_bytes() {
    return PairShape<P, (int)sizeof(typename MathOf<P, TRUNC, F64>::X)>::kSmemBytes;
}

template <int P, bool TRUNC, bool F64>
cudaError_t pair_prepare() {
    static bool done = false;  // one engine thread at a time; idempotent if raced
    if (done) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(pair_kernel<P, TRUNC, MathOf<P, TRUNC, F64>>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, pair_smem_bytes<P, TRUNC, F64>());
    if (e == cudaSuccess) done = true;
    return e;
}

template <int P, bool TRUNC, bool F64>
cudaError_t pair_launch_one(const PairMaps& maps, const PairArgs& args, cudaStream_t stream) {
    using M = MathOf<P, TRUNC, F64>;
    cudaError_t e = pair_prepare<P, TRUNC, F64>();
    if (e != cudaSuccess) return e;
    pair_kernel<P, TRUNC, M><<<args.grid, kPairThreads, pair_smem_bytes<P, TRUNC, F64>(), stream>>>(
        maps.a, maps.b, maps.xi, maps.xj, args);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    // the finish kernel as a programmatic dependent: launched while the sweep
    // drains, it waits in griddepcontrol.wait for the sweep's results
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)args.nc + 1);
    cfg.blockDim = dim3(FinishShape<P>::kThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, pair_finish_kernel<P, typename M::Part>, args);
}

template <int P, bool TRUNC, bool F64>
cudaError_t pair_occupancy_one(int* ctas) {
    cudaError_t e = pair_prepare<P, TRUNC, F64>();
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas, pair_kernel<P, TRUNC, MathOf<P, TRUNC, F64>>,
                                                         kPairThreads, pair_smem_bytes<P, TRUNC, F64>());
}

template <int P>
cudaError_t pair_launch_p(bool trunc, bool f64, const PairMaps& maps, const PairArgs& args, cudaStream_t stream) {
    if (f64)
        return trunc ? pair_launch_one<P, true, true>(maps, args, stream)
                     : pair_launch_one<P, false, true>(maps, args, stream);
    return trunc ? pair_launch_one<P, true, false>(maps, args, stream)
                 : pair_launch_one<P, false, false>(maps, args, stream);
}

template <int P>
cudaError_t pair_occupancy_p(bool trunc, bool f64, int* ctas) {
    if (f64) return trunc ? pair_occupancy_one<P, true, true>(ctas) : pair_occupancy_one<P, false, true>(ctas);
    return trunc ? pair_occupancy_one<P, true, false>(ctas) : pair_occupancy_one<P, false, false>(ctas);
}

}  // namespace

bool pair_built(Mode mode, int p) {
    return (mode == Mode::kF32 || mode == Mode::kF64DeltaF32) && p >= 1 && p <= kPairMaxP;
}

cudaError_t pair_occupancy(int p, bool trunc, bool f64, int* ctas_per_sm) {
    switch (p) {
        case 1: return pair_occupancy_p<1>(trunc, f64, ctas_per_sm);
        case 2: return pair_occupancy_p<2>(trunc, f64, ctas_per_sm);
        case 3: return pair_occupancy_p<3>(trunc, f64, ctas_per_sm);
        case 4: return pair_occupancy_p<4>(trunc, f64, ctas_per_sm);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t pair_launch(int p, bool trunc, bool f64, const PairMaps& maps, const PairArgs& args,
                        cudaStream_t stream) {
    switch (p) {
        case 1: return pair_launch_p<1>(trunc, f64, maps, args, stream);
        case 2: return pair_launch_p<2>(trunc, f64, maps, args, stream);
        case 3: return pair_launch_p<3>(trunc, f64, maps, args, stream);
        case 4: return pair_launch_p<4>(trunc, f64, maps, args, stream);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace mdsx
