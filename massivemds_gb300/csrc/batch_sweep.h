// Host interface of the batched sweep kernels (batch_sweep_lo.cu: P 1..4,
// batch_sweep_hi.cu: P 5..10; two translation units so they build in parallel).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

#include "batch_kernel.cuh"
#include "batch_pairs.cuh"
#include "batch_queue.cuh"

namespace mdsx {
namespace batch {

// Rows per warp built for P: {1, 2, 4} for P <= 4, {1, 2} for P <= 8, {1} above.
bool rw_built(int p, int rw);
// (schedule, rows per warp) built for P: rw_built for schedules 0 and 1; schedule 2 with 4 and P <= kPairMaxP.
bool shape_built(int p, int schedule, int rw);
// Dynamic shared memory of one CTA.
int smem_bytes(int p, int rw);
// Resident CTAs per SM and local (spill) bytes per thread of the kernel.
cudaError_t occupancy(int p, bool trunc, int rw, int* ctas_per_sm, size_t* local_bytes);
cudaError_t launch(int p, bool trunc, int rw, const BatchArgs& a, cudaStream_t st);

// Row-block queue schedule (batch_queue.cuh).
cudaError_t occupancy_queue(int p, bool trunc, int rw, int* ctas_per_sm);
cudaError_t launch_queue(int p, bool trunc, int rw, const QueueArgs& a, int grid, cudaStream_t st);

// Unordered-pair schedule (batch_pairs.cuh, batch_sweep_pairs.cu): P <= kPairMaxP.
cudaError_t occupancy_pairs(int p, bool trunc, int* ctas_per_sm);
// The sweep (grid CTAs) and its finish kernel (finish_blocks blocks) as a programmatic dependent.
cudaError_t launch_pairs(int p, bool trunc, const BatchPairArgs& a, int grid, int finish_blocks, cudaStream_t st);

#define MDSX_BATCH_DECLARE(R)                                                                  \
    cudaError_t occupancy_##R(int p, bool trunc, int rw, int* ctas_per_sm, size_t* local_bytes); \
    cudaError_t launch_##R(int p, bool trunc, int rw, const BatchArgs& a, cudaStream_t st);      \
    cudaError_t occupancy_queue_##R(int p, bool trunc, int rw, int* ctas_per_sm);                 \
    cudaError_t launch_queue_##R(int p, bool trunc, int rw, const QueueArgs& a, int grid, cudaStream_t st);
MDSX_BATCH_DECLARE(lo)
MDSX_BATCH_DECLARE(hi)
#undef MDSX_BATCH_DECLARE

}  // namespace batch
}  // namespace mdsx
