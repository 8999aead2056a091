// Host-side launch of the unordered-pair sweep (pair_kernel.cuh) and its finish
// kernel, per (P, truncation, pair-math mode); included by the translation
// units that instantiate the modes (sweep_pairs.cu, sweep_pairs_dd.cu).
#pragma once

#include <type_traits>

#include "pair_kernel.cuh"
#include "sweep.h"

namespace mdsx {
namespace {

// MODE: 0 FP32 math, 1 FP64 math over FP32 delta, 2 FP64 math over FP64 delta,
// 3 double-float math over FP32 delta, 4 double-float math over double-float delta.
template <int P, bool TRUNC, int MODE>
using MathOf = typename std::conditional<
    MODE == 0, PairMathF32For<P, TRUNC>,
    typename std::conditional<
        MODE == 1, PairMathF64<P, TRUNC, float>,
        typename std::conditional<MODE == 2, PairMathF64<P, TRUNC, double>,
                                  typename std::conditional<MODE == 3, PairMathDD<P, TRUNC, float>,
                                                            PairMathDD<P, TRUNC, double>>::type>::type>::type>::type;

template <int P, bool TRUNC, int MODE>
constexpr int pair_smem_bytes() {
    using M = MathOf<P, TRUNC, MODE>;
    return PairShape<P, (int)sizeof(typename M::X), (int)sizeof(typename M::S)>::kSmemBytes;
}

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

template <int P, int MODE>
cudaError_t pair_occupancy_pm(bool trunc, int* ctas) {
    return trunc ? pair_occupancy_one<P, true, MODE>(ctas) : pair_occupancy_one<P, false, MODE>(ctas);
}

}  // namespace
}  // namespace mdsx
