// Self-tests. (1) The FP64 pair-math helpers (rcp_f64, rsqrt_f64,
// normal_cdf_pdf_f64) evaluated on the device for host-chosen inputs, which a
// test compares with correctly rounded host values.
// (2) The bounded device waits every kernel of this library uses
// (ptx.cuh, mbar_wait_bounded): a one-thread kernel waits on a shared-memory
// mbarrier that nothing arrives at, with a short limit, and must give up,
// record the timeout in an error word and return, leaving the context usable.
// The wait ends by its limit; no fault, trap or endless loop is involved.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/mdsx.h"
#include "ptx.cuh"
#include "sweep_kernel.cuh"

namespace {

__global__ void bounded_wait_probe(int* err, unsigned long long limit_ns, int* completed) {
    __shared__ uint64_t bar;
    mdsx::mbar_init(&bar, 1);
    mdsx::fence_mbar_init();
    // phase 0 never completes: no thread arrives
    const bool ok = mdsx::mbar_wait_bounded(&bar, 0u, err, mdsx::kDevTimeoutFull, limit_ns);
    *completed = ok ? 1 : 0;
}

__global__ void math_f64_probe(const double* __restrict__ x, size_t n, double* __restrict__ out) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        double cdf, pdf;
        mdsx::normal_cdf_pdf_f64(x[i], cdf, pdf);
        out[4 * i + 0] = mdsx::rcp_f64(x[i]);
        out[4 * i + 1] = mdsx::rsqrt_f64(x[i]);
        out[4 * i + 2] = cdf;
        out[4 * i + 3] = pdf;
    }
}

}  // namespace

extern "C" int mdsx_selftest_math_f64(const double* x, size_t n, double* out, int device) {
    if (!x || !out || n == 0 || n > ((size_t)1 << 24)) return MDSX_EINVAL;
    int prev = -1;
    cudaGetDevice(&prev);
    if (device >= 0 && cudaSetDevice(device) != cudaSuccess) return MDSX_ECUDA;
    double *dx = nullptr, *dout = nullptr;
    int rc = MDSX_OK;
    if (cudaMalloc(&dx, n * sizeof(double)) != cudaSuccess || cudaMalloc(&dout, 4 * n * sizeof(double)) != cudaSuccess)
        rc = MDSX_ENOMEM;
    if (!rc && cudaMemcpy(dx, x, n * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) rc = MDSX_ECUDA;
    if (!rc) {
        const unsigned grid = (unsigned)((n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024);
        math_f64_probe<<<grid, 256>>>(dx, n, dout);
        if (cudaGetLastError() != cudaSuccess ||
            cudaMemcpy(out, dout, 4 * n * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = MDSX_ECUDA;
    }
    cudaFree(dx);
    cudaFree(dout);
    if (prev >= 0) cudaSetDevice(prev);
    return rc;
}

extern "C" int mdsx_selftest_bounded_wait(double limit_seconds, int device, int* device_code) {
    if (!device_code || !(limit_seconds > 0.0) || limit_seconds > 10.0) return MDSX_EINVAL;
    int prev = -1;
    cudaGetDevice(&prev);
    if (device >= 0 && cudaSetDevice(device) != cudaSuccess) return MDSX_ECUDA;
    int* d = nullptr;
    int h[2] = {0, 0};
    int rc = MDSX_OK;
    if (cudaMalloc(&d, 2 * sizeof(int)) != cudaSuccess) rc = MDSX_ENOMEM;
    if (!rc && cudaMemset(d, 0, 2 * sizeof(int)) != cudaSuccess) rc = MDSX_ECUDA;
    if (!rc) {
        bounded_wait_probe<<<1, 1>>>(d, (unsigned long long)(limit_seconds * 1e9), d + 1);
        if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess ||
            cudaMemcpy(h, d, 2 * sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = MDSX_ECUDA;
    }
    cudaFree(d);
    if (prev >= 0) cudaSetDevice(prev);
    if (rc) return rc;
    *device_code = h[0];
    // the wait must have given up (not completed) and recorded the timeout
    return (h[1] == 0 && h[0] == mdsx::kDevTimeoutFull) ? MDSX_ETIMEOUT : MDSX_ECUDA;
}
