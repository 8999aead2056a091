// Instances of the batched unordered-pair sweep (batch_pairs.cuh): P = 1..kPairMaxP,
// truncation on/off, and its host-side launch (sweep + finish kernel).
#include "batch_sweep.h"

namespace mdsx {
namespace batch {
namespace {

template <int P, bool TRUNC>
constexpr int pairs_smem() {
    return PairShape<P, 4, 4>::kSmemBytes;
}

template <int P, bool TRUNC>
cudaError_t prepare_pairs() {
    static bool done = false;  // one host thread at a time; idempotent if raced
    if (done) return cudaSuccess;
    const cudaError_t e = cudaFuncSetAttribute(batch_pair_kernel<P, TRUNC>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, pairs_smem<P, TRUNC>());
    if (e == cudaSuccess) done = true;
    return e;
}

template <int P, bool TRUNC>
cudaError_t launch_pairs_one(const BatchPairArgs& a, int grid, int finish_blocks, cudaStream_t st) {
    cudaError_t e = prepare_pairs<P, TRUNC>();
    if (e != cudaSuccess) return e;
    batch_pair_kernel<P, TRUNC><<<grid, kPairThreads, pairs_smem<P, TRUNC>(), st>>>(a);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)finish_blocks);
    cfg.blockDim = dim3(FinishShape<P, float>::kThreads);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, batch_pair_finish_kernel<P>, a);
}

template <int P, bool TRUNC>
cudaError_t occupancy_pairs_one(int* ctas) {
    const cudaError_t e = prepare_pairs<P, TRUNC>();
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas, batch_pair_kernel<P, TRUNC>, kPairThreads,
                                                         pairs_smem<P, TRUNC>());
}

template <int P>
cudaError_t launch_p(bool trunc, const BatchPairArgs& a, int grid, int finish_blocks, cudaStream_t st) {
    return trunc ? launch_pairs_one<P, true>(a, grid, finish_blocks, st)
                 : launch_pairs_one<P, false>(a, grid, finish_blocks, st);
}

template <int P>
cudaError_t occupancy_p(bool trunc, int* ctas) {
    return trunc ? occupancy_pairs_one<P, true>(ctas) : occupancy_pairs_one<P, false>(ctas);
}

}  // namespace

cudaError_t occupancy_pairs(int p, bool trunc, int* ctas_per_sm) {
    switch (p) {
        case 1: return occupancy_p<1>(trunc, ctas_per_sm);
        case 2: return occupancy_p<2>(trunc, ctas_per_sm);
        case 3: return occupancy_p<3>(trunc, ctas_per_sm);
        case 4: return occupancy_p<4>(trunc, ctas_per_sm);
        case 5: return occupancy_p<5>(trunc, ctas_per_sm);
        case 6: return occupancy_p<6>(trunc, ctas_per_sm);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_pairs(int p, bool trunc, const BatchPairArgs& a, int grid, int finish_blocks, cudaStream_t st) {
    switch (p) {
        case 1: return launch_p<1>(trunc, a, grid, finish_blocks, st);
        case 2: return launch_p<2>(trunc, a, grid, finish_blocks, st);
        case 3: return launch_p<3>(trunc, a, grid, finish_blocks, st);
        case 4: return launch_p<4>(trunc, a, grid, finish_blocks, st);
        case 5: return launch_p<5>(trunc, a, grid, finish_blocks, st);
        case 6: return launch_p<6>(trunc, a, grid, finish_blocks, st);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace batch
}  // namespace mdsx
