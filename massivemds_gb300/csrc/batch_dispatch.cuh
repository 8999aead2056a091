// Instantiation helpers of the batched sweep kernel (included by
// batch_sweep_lo.cu and batch_sweep_hi.cu).
#pragma once

#include "batch_queue.cuh"
#include "batch_sweep.h"

namespace mdsx {
namespace batch {
namespace detail {

template <int P, bool TRUNC, int RW>
cudaError_t launch_one(const BatchArgs& a, cudaStream_t st) {
    constexpr int smem = BatchShape<P, RW>::kSmemBytes;
    cudaError_t e =
        cudaFuncSetAttribute(batch_sweep_kernel<P, TRUNC, RW>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    batch_sweep_kernel<P, TRUNC, RW><<<a.grid, kThreads, smem, st>>>(a);
    return cudaGetLastError();
}

template <int P, bool TRUNC, int RW>
cudaError_t occupancy_one(int* ctas, size_t* local_bytes) {
    constexpr int smem = BatchShape<P, RW>::kSmemBytes;
    cudaError_t e =
        cudaFuncSetAttribute(batch_sweep_kernel<P, TRUNC, RW>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    cudaFuncAttributes attr{};
    e = cudaFuncGetAttributes(&attr, batch_sweep_kernel<P, TRUNC, RW>);
    if (e != cudaSuccess) return e;
    *local_bytes = attr.localSizeBytes;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas, batch_sweep_kernel<P, TRUNC, RW>, kThreads, smem);
}

template <int P, bool TRUNC, int RW>
cudaError_t launch_queue_one(const QueueArgs& a, int grid, cudaStream_t st) {
    constexpr int smem = QueueShape<P, RW>::kSmemBytes;
    cudaError_t e =
        cudaFuncSetAttribute(batch_queue_kernel<P, TRUNC, RW>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    batch_queue_kernel<P, TRUNC, RW><<<grid, kThreads, smem, st>>>(a);
    return cudaGetLastError();
}

template <int P, bool TRUNC, int RW>
cudaError_t occupancy_queue_one(int* ctas) {
    constexpr int smem = QueueShape<P, RW>::kSmemBytes;
    cudaError_t e =
        cudaFuncSetAttribute(batch_queue_kernel<P, TRUNC, RW>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas, batch_queue_kernel<P, TRUNC, RW>, kThreads, smem);
}

template <int P, int RW>
cudaError_t launch_queue_p(bool trunc, const QueueArgs& a, int grid, cudaStream_t st) {
    return trunc ? launch_queue_one<P, true, RW>(a, grid, st) : launch_queue_one<P, false, RW>(a, grid, st);
}
template <int P, int RW>
cudaError_t occupancy_queue_p(bool trunc, int* ctas) {
    return trunc ? occupancy_queue_one<P, true, RW>(ctas) : occupancy_queue_one<P, false, RW>(ctas);
}

template <int P, int RW>
cudaError_t launch_p(bool trunc, const BatchArgs& a, cudaStream_t st) {
    return trunc ? launch_one<P, true, RW>(a, st) : launch_one<P, false, RW>(a, st);
}
template <int P, int RW>
cudaError_t occupancy_p(bool trunc, int* ctas, size_t* local_bytes) {
    return trunc ? occupancy_one<P, true, RW>(ctas, local_bytes) : occupancy_one<P, false, RW>(ctas, local_bytes);
}

}  // namespace detail
}  // namespace batch
}  // namespace mdsx

// Cases of one P: rows per warp 1 (always), 2 (P <= 8), 4 (P <= 4).
#define MDSX_BATCH_CASE(P)                                                                              \
    case P:                                                                                            \
        if (rw == 1) return detail::FN<P, 1>(ARGS);                                                    \
        if constexpr (P <= 8) {                                                                        \
            if (rw == 2) return detail::FN<P, 2>(ARGS);                                                \
        }                                                                                              \
        if constexpr (P <= 4) {                                                                        \
            if (rw == 4) return detail::FN<P, 4>(ARGS);                                                \
        }                                                                                              \
        return cudaErrorInvalidValue;
