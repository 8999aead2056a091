// Compile-time dispatch from (P, truncation) to the sweep kernel instances of one
// precision mode. Included once per precision translation unit.
#pragma once

#include "sweep.h"

namespace mdsx {
namespace detail {

template <typename C, typename S, int P, bool TRUNC>
cudaError_t launch_one(int grid, const CUtensorMap& td, const CUtensorMap& tx, const SweepArgs& args,
                       cudaStream_t stream) {
    using Shape = SweepShape<C, S, P>;
    auto kernel = sweep_kernel<C, S, P, TRUNC>;
    static bool attr_set = false;  // one engine thread at a time; idempotent if raced
    if (!attr_set) {
        cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, Shape::kSmemBytes);
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    kernel<<<grid, kThreads, Shape::kSmemBytes, stream>>>(td, tx, args);
    return cudaGetLastError();
}

template <typename C, typename S, int P, bool TRUNC>
cudaError_t occupancy_one(int* ctas) {
    using Shape = SweepShape<C, S, P>;
    auto kernel = sweep_kernel<C, S, P, TRUNC>;
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, Shape::kSmemBytes);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas, kernel, kThreads, Shape::kSmemBytes);
}

template <typename C, typename S, int P>
void shape_one(KernelShape* out) {
    using Shape = SweepShape<C, S, P>;
    out->rw = Shape::RW;
    out->rb = Shape::RB;
    out->smem_bytes = Shape::kSmemBytes;
    out->delta_elem_bytes = (int)sizeof(S);
    out->x_elem_bytes = (int)sizeof(C);
}

// Calls F::template run<P>() for the runtime p in [1, MDSX_MAX_DIMENSION].
template <typename F>
auto dispatch_p(int p, F&& f) -> decltype(f.template run<1>()) {
    switch (p) {
        case 1: return f.template run<1>();
        case 2: return f.template run<2>();
        case 3: return f.template run<3>();
        case 4: return f.template run<4>();
        case 5: return f.template run<5>();
        case 6: return f.template run<6>();
        case 7: return f.template run<7>();
        case 8: return f.template run<8>();
        case 9: return f.template run<9>();
        case 10: return f.template run<10>();
        default: return decltype(f.template run<1>())();
    }
}

template <typename C, typename S>
struct LaunchF {
    bool trunc;
    int grid;
    const CUtensorMap& td;
    const CUtensorMap& tx;
    const SweepArgs& args;
    cudaStream_t stream;
    template <int P>
    cudaError_t run() const {
        return trunc ? launch_one<C, S, P, true>(grid, td, tx, args, stream)
                     : launch_one<C, S, P, false>(grid, td, tx, args, stream);
    }
};

template <typename C, typename S>
struct OccF {
    bool trunc;
    int* ctas;
    template <int P>
    cudaError_t run() const {
        return trunc ? occupancy_one<C, S, P, true>(ctas) : occupancy_one<C, S, P, false>(ctas);
    }
};

template <typename C, typename S>
struct ShapeF {
    KernelShape* out;
    template <int P>
    bool run() const {
        shape_one<C, S, P>(out);
        return true;
    }
};

}  // namespace detail
}  // namespace mdsx

#define MDSX_DEFINE_MODE(NAME, C, S)                                                                         \
    namespace mdsx {                                                                                         \
    bool sweep_shape_##NAME(int p, KernelShape* out) {                                                       \
        if (p < 1 || p > 10) return false;                                                                   \
        return detail::dispatch_p(p, detail::ShapeF<C, S>{out});                                             \
    }                                                                                                        \
    cudaError_t sweep_occupancy_##NAME(int p, bool trunc, int* ctas) {                                       \
        if (p < 1 || p > 10) return cudaErrorInvalidValue;                                                   \
        return detail::dispatch_p(p, detail::OccF<C, S>{trunc, ctas});                                       \
    }                                                                                                        \
    cudaError_t sweep_launch_##NAME(int p, bool trunc, int grid, const CUtensorMap& td, const CUtensorMap& tx, \
                                    const SweepArgs& args, cudaStream_t stream) {                            \
        if (p < 1 || p > 10) return cudaErrorInvalidValue;                                                   \
        return detail::dispatch_p(p, detail::LaunchF<C, S>{trunc, grid, td, tx, args, stream});              \
    }                                                                                                        \
    }
