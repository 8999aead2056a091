// Batched sweep kernels for P = 1..4 (see batch_kernel.cuh).
#include "batch_dispatch.cuh"

namespace mdsx {
namespace batch {

cudaError_t launch_lo(int p, bool trunc, int rw, const BatchArgs& a, cudaStream_t st) {
#define FN launch_p
#define ARGS trunc, a, st
    switch (p) {
        MDSX_BATCH_CASE(1)
        MDSX_BATCH_CASE(2)
        MDSX_BATCH_CASE(3)
        MDSX_BATCH_CASE(4)
        default: return cudaErrorInvalidValue;
    }
#undef FN
#undef ARGS
}

cudaError_t occupancy_lo(int p, bool trunc, int rw, int* ctas_per_sm, size_t* local_bytes) {
#define FN occupancy_p
#define ARGS trunc, ctas_per_sm, local_bytes
    switch (p) {
        MDSX_BATCH_CASE(1)
        MDSX_BATCH_CASE(2)
        MDSX_BATCH_CASE(3)
        MDSX_BATCH_CASE(4)
        default: return cudaErrorInvalidValue;
    }
#undef FN
#undef ARGS
}

cudaError_t launch_queue_lo(int p, bool trunc, int rw, const QueueArgs& a, int grid, cudaStream_t st) {
#define FN launch_queue_p
#define ARGS trunc, a, grid, st
    switch (p) {
        MDSX_BATCH_CASE(1)
        MDSX_BATCH_CASE(2)
        MDSX_BATCH_CASE(3)
        MDSX_BATCH_CASE(4)
        default: return cudaErrorInvalidValue;
    }
#undef FN
#undef ARGS
}

cudaError_t occupancy_queue_lo(int p, bool trunc, int rw, int* ctas_per_sm) {
#define FN occupancy_queue_p
#define ARGS trunc, ctas_per_sm
    switch (p) {
        MDSX_BATCH_CASE(1)
        MDSX_BATCH_CASE(2)
        MDSX_BATCH_CASE(3)
        MDSX_BATCH_CASE(4)
        default: return cudaErrorInvalidValue;
    }
#undef FN
#undef ARGS
}

}  // namespace batch
}  // namespace mdsx
