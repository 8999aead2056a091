// Layout kernels: locations into the SoA compute layout, delta rows into the
// padded storage layout (the NaN-preserving double -> float conversion of
// src/MemoryManagement.hpp:45-56 in MassiveMDS), and the per-row NaN marks the
// sweep uses to pick its masked path.
#include <cstdint>

#include "sweep.h"

namespace mdsx {
namespace {

// An 8-byte slot holding a double as the double-float pair (hi, lo), low word
// first: the location and delta layout of the double-float pair math. A NaN is
// stored as a float NaN in hi and 0x7ff80000 in lo, which is a NaN both as a
// float and as the high word of a double, so the slot reads as NaN to the pair
// math (hi) and to the FP64 NaN-row scan (mark_nan_rows) alike.
struct DDSlot {
    float hi, lo;
    DDSlot() = default;
    __device__ explicit DDSlot(double v) {
        if (isnan(v)) {
            hi = __int_as_float(0x7fc00000);
            lo = __int_as_float(0x7ff80000);
            return;
        }
        hi = (float)v;
        lo = isfinite(hi) ? (float)(v - (double)hi) : 0.0f;
    }
};
static_assert(sizeof(DDSlot) == 8, "a double-float slot is 8 bytes");

template <typename C>
__global__ void convert_locations_kernel(const double* __restrict__ src, int n, int p, C* __restrict__ dst, int x_ld) {
    const long long total = (long long)p * x_ld;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const int q = (int)(idx / x_ld);
        const int i = (int)(idx - (long long)q * x_ld);
        dst[idx] = i < n ? (C)src[(long long)i * p + q] : C(0);
    }
}

template <typename C>
__global__ void set_one_location_kernel(const double* __restrict__ src, int index, int p, C* __restrict__ dst,
                                        int x_ld) {
    const int q = threadIdx.x;
    if (q < p) dst[(long long)q * x_ld + index] = (C)src[q];
}

template <typename T>
__global__ void convert_delta_rows_kernel(const double* __restrict__ src, long long rows, int n, T* __restrict__ dst,
                                          long long ld) {
    const long long total = rows * n;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const long long r = idx / n;
        const long long c = idx - r * n;
        dst[r * ld + c] = (T)src[idx];  // NaN converts to NaN
    }
}

__global__ void copy_delta_rows_f32_kernel(const float* __restrict__ src, long long rows, int n, float* __restrict__ dst,
                                           long long ld) {
    const long long total = rows * n;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const long long r = idx / n;
        const long long c = idx - r * n;
        dst[r * ld + c] = src[idx];
    }
}

// One warp per row.
template <typename T>
__global__ void mark_nan_rows_kernel(const T* __restrict__ delta, int rows, int cols, long long ld,
                                     int* __restrict__ row_nan, int rows_padded) {
    const int warps = (gridDim.x * blockDim.x) >> 5;
    const int lane = threadIdx.x & 31;
    for (int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < rows_padded; row += warps) {
        int bad = 0;
        if (row < rows) {
            const T* r = delta + (long long)row * ld;
            for (int c = lane; c < cols; c += 32) bad |= (r[c] != r[c]);
            bad = __any_sync(0xffffffffu, bad);
        } else {
            bad = 1;
        }
        if (lane == 0) row_nan[row] = bad;
    }
}

__global__ void mark_padding_rows_kernel(int n, int* __restrict__ row_nan, int rows_padded) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < rows_padded; i += gridDim.x * blockDim.x)
        row_nan[i] = i >= n ? 1 : 0;
}

template <typename T>
__global__ void write_flag_row_kernel(const int* __restrict__ row_nan, int n, int rows_padded,
                                      T* __restrict__ flags, int x_ld) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < x_ld; j += gridDim.x * blockDim.x)
        flags[j] = (j >= n || (j < rows_padded && row_nan[j] != 0)) ? T(1) : T(0);
}

int grid_for(long long work, int threads) {
    long long blocks = (work + threads - 1) / threads;
    if (blocks < 1) blocks = 1;
    if (blocks > 4096) blocks = 4096;
    return (int)blocks;
}

}  // namespace

cudaError_t convert_locations(const double* src, int n, int p, void* dst, int x_ld, bool to_f32, cudaStream_t s) {
    const int grid = grid_for((long long)p * x_ld, 256);
    if (to_f32)
        convert_locations_kernel<float><<<grid, 256, 0, s>>>(src, n, p, static_cast<float*>(dst), x_ld);
    else
        convert_locations_kernel<double><<<grid, 256, 0, s>>>(src, n, p, static_cast<double*>(dst), x_ld);
    return cudaGetLastError();
}

cudaError_t set_one_location(const double* src, int index, int p, void* dst, int x_ld, bool to_f32, cudaStream_t s) {
    if (to_f32)
        set_one_location_kernel<float><<<1, 32, 0, s>>>(src, index, p, static_cast<float*>(dst), x_ld);
    else
        set_one_location_kernel<double><<<1, 32, 0, s>>>(src, index, p, static_cast<double*>(dst), x_ld);
    return cudaGetLastError();
}

cudaError_t convert_locations_dd(const double* src, int n, int p, void* dst, int x_ld, cudaStream_t s) {
    const int grid = grid_for((long long)p * x_ld, 256);
    convert_locations_kernel<DDSlot><<<grid, 256, 0, s>>>(src, n, p, static_cast<DDSlot*>(dst), x_ld);
    return cudaGetLastError();
}

cudaError_t set_one_location_dd(const double* src, int index, int p, void* dst, int x_ld, cudaStream_t s) {
    set_one_location_kernel<DDSlot><<<1, 32, 0, s>>>(src, index, p, static_cast<DDSlot*>(dst), x_ld);
    return cudaGetLastError();
}

cudaError_t convert_delta_rows_dd(const double* src, long long rows, int n, void* dst, long long ld, cudaStream_t s) {
    convert_delta_rows_kernel<DDSlot><<<grid_for(rows * n, 256), 256, 0, s>>>(src, rows, n, static_cast<DDSlot*>(dst),
                                                                              ld);
    return cudaGetLastError();
}

cudaError_t convert_delta_rows(const double* src, long long rows, int n, void* dst, long long ld, bool to_f32,
                               cudaStream_t s) {
    const int grid = grid_for(rows * n, 256);
    if (to_f32)
        convert_delta_rows_kernel<float><<<grid, 256, 0, s>>>(src, rows, n, static_cast<float*>(dst), ld);
    else
        convert_delta_rows_kernel<double><<<grid, 256, 0, s>>>(src, rows, n, static_cast<double*>(dst), ld);
    return cudaGetLastError();
}

cudaError_t copy_delta_rows_f32(const float* src, long long rows, int n, float* dst, long long ld, cudaStream_t s) {
    copy_delta_rows_f32_kernel<<<grid_for(rows * n, 256), 256, 0, s>>>(src, rows, n, dst, ld);
    return cudaGetLastError();
}

cudaError_t mark_nan_rows_block(const void* delta, bool is_f32, int rows, int cols, long long ld, int* row_nan,
                                int rows_padded, cudaStream_t s) {
    const int grid = grid_for((long long)rows_padded * 32, 256);
    if (is_f32)
        mark_nan_rows_kernel<float><<<grid, 256, 0, s>>>(static_cast<const float*>(delta), rows, cols, ld, row_nan,
                                                         rows_padded);
    else
        mark_nan_rows_kernel<double><<<grid, 256, 0, s>>>(static_cast<const double*>(delta), rows, cols, ld, row_nan,
                                                          rows_padded);
    return cudaGetLastError();
}

cudaError_t mark_nan_rows(const void* delta, bool is_f32, int n, long long ld, int* row_nan, int rows_padded,
                          cudaStream_t s) {
    return mark_nan_rows_block(delta, is_f32, n, n, ld, row_nan, rows_padded, s);
}

cudaError_t mark_padding_rows(int n, int* row_nan, int rows_padded, cudaStream_t s) {
    mark_padding_rows_kernel<<<grid_for(rows_padded, 256), 256, 0, s>>>(n, row_nan, rows_padded);
    return cudaGetLastError();
}

cudaError_t write_flag_row(const int* row_nan, int n, int rows_padded, void* flags, bool is_f32, int x_ld,
                           cudaStream_t s) {
    if (is_f32)
        write_flag_row_kernel<float><<<grid_for(x_ld, 256), 256, 0, s>>>(row_nan, n, rows_padded,
                                                                          static_cast<float*>(flags), x_ld);
    else
        write_flag_row_kernel<double><<<grid_for(x_ld, 256), 256, 0, s>>>(row_nan, n, rows_padded,
                                                                           static_cast<double*>(flags), x_ld);
    return cudaGetLastError();
}

}  // namespace mdsx
