// Host-side fault injection for the tests of the failure paths.
//
// The reference has none: it asserts or exits on errors. Here every C-ABI call
// returns a status, and these hooks let a test make one chosen host-side call
// fail -- a device allocation, a pinned host allocation, or the enqueue of a
// sweep kernel -- without touching the GPU: the failing call is not made at
// all, and the hook returns the error the runtime would have returned
// (cudaErrorMemoryAllocation, or cudaErrorLaunchOutOfResources, which is not
// sticky), so the context stays usable. Armed through mdsx_inject_fault
// (include/mdsx.h); one-shot: a hook disarms itself when it fires.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

namespace mdsx {

enum class FaultSite : int { kNone = 0, kDeviceAlloc = 1, kHostAlloc = 2, kLaunch = 3 };

// True when the armed fault of `site` fires now (and disarms it).
bool fault_fires(FaultSite site);

inline cudaError_t device_malloc(void** p, size_t bytes) {
    if (fault_fires(FaultSite::kDeviceAlloc)) {
        *p = nullptr;
        return cudaErrorMemoryAllocation;
    }
    return cudaMalloc(p, bytes);
}
template <typename T>
inline cudaError_t device_malloc(T** p, size_t bytes) {
    return device_malloc(reinterpret_cast<void**>(p), bytes);
}

inline cudaError_t host_malloc(void** p, size_t bytes) {
    if (fault_fires(FaultSite::kHostAlloc)) {
        *p = nullptr;
        return cudaErrorMemoryAllocation;
    }
    return cudaMallocHost(p, bytes);
}
template <typename T>
inline cudaError_t host_malloc(T** p, size_t bytes) {
    return host_malloc(reinterpret_cast<void**>(p), bytes);
}

// cudaSuccess, or the injected launch failure; called just before a sweep's launch.
inline cudaError_t launch_fault() {
    return fault_fires(FaultSite::kLaunch) ? cudaErrorLaunchOutOfResources : cudaSuccess;
}

}  // namespace mdsx
