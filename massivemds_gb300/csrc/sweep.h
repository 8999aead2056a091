// Host-side interface of the sweep kernels (implemented in sweep_f32.cu,
// sweep_f64.cu, sweep_f64s32.cu; one translation unit per precision mode so the
// build compiles them in parallel).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <string>

#include "sweep_kernel.cuh"

namespace mdsx {

enum class Mode : int {
    kF32 = 0,          // FP32 pairs, FP32-stored delta, FP64 reductions
    kF64 = 1,          // FP64 pairs, FP64-stored delta
    kF64DeltaF32 = 2,  // FP64 pairs, FP32-stored delta
};

struct KernelShape {
    int rw;                // rows per consumer warp
    int rb;                // rows per tile (8 * rw)
    int smem_bytes;        // dynamic shared memory per CTA
    int delta_elem_bytes;  // 4 or 8
    int x_elem_bytes;      // 4 or 8
};

// Shape of the sweep kernel for (mode, P); false if P is not built.
bool sweep_shape(Mode mode, int p, KernelShape* out);

// Resident CTAs per SM of the sweep kernel for (mode, P, trunc).
cudaError_t sweep_occupancy(Mode mode, int p, bool trunc, int* ctas_per_sm);

// Launches one fused sweep.
cudaError_t sweep_launch(Mode mode, int p, bool trunc, int grid, const CUtensorMap& tmap_delta,
                         const CUtensorMap& tmap_x, const SweepArgs& args, cudaStream_t stream);

// Per-precision entry points behind the three functions above.
#define MDSX_DECLARE_MODE(NAME)                                                                          \
    bool sweep_shape_##NAME(int p, KernelShape* out);                                                  \
    cudaError_t sweep_occupancy_##NAME(int p, bool trunc, int* ctas_per_sm);                           \
    cudaError_t sweep_launch_##NAME(int p, bool trunc, int grid, const CUtensorMap& tmap_delta,       \
                                    const CUtensorMap& tmap_x, const SweepArgs& args, cudaStream_t stream);
MDSX_DECLARE_MODE(f32)
MDSX_DECLARE_MODE(f64)
MDSX_DECLARE_MODE(f64s32)
#undef MDSX_DECLARE_MODE

// Unordered-pair schedule (sweep_pairs.cu, pair_kernel.cuh).
struct PairArgs;
struct PairMaps {
    CUtensorMap a;   // delta, box 128 columns x 32 rows
    CUtensorMap b;   // delta, box 128 bytes (32 FP32 or 16 FP64 columns) x 128 rows, 128-byte swizzle
    CUtensorMap xi;  // locations + flag row, box 32 columns x (P + 1) rows
    CUtensorMap xj;  // the same, box 128 columns x (P + 1) rows
};
// Built for every precision mode with P <= kPairMaxP.
bool pair_built(Mode mode, int p);
// dd: double-float pair math over the FP64 modes' storage (mode kF64DeltaF32:
// FP32 delta; kF64: delta and locations as (hi, lo) float pairs in 8-byte slots).
cudaError_t pair_occupancy(int p, bool trunc, Mode mode, int* ctas_per_sm, bool dd = false);
// Enqueues the pair sweep and its finish kernel (two launches).
cudaError_t pair_launch(int p, bool trunc, Mode mode, const PairMaps& maps, const PairArgs& args,
                        cudaStream_t stream, bool dd = false);
// The double-float instances (sweep_pairs_dd.cu), P <= kPairMaxP64.
cudaError_t pair_occupancy_dd(int p, bool trunc, bool delta_f32, int* ctas_per_sm);
cudaError_t pair_launch_dd(int p, bool trunc, bool delta_f32, const PairMaps& maps, const PairArgs& args,
                           cudaStream_t stream);
// flags[j] = 1 for j >= n or a NaN in row j of delta (row_nan), else 0, for j < x_ld,
// in the location type (float or double).
cudaError_t write_flag_row(const int* row_nan, int n, int rows_padded, void* flags, bool is_f32, int x_ld,
                           cudaStream_t s);

// Sets the message mdsx_last_error(NULL) returns on this thread (engine.cu).
void set_global_error(const std::string& msg);

// Preprocessing kernels (prep.cu).
// Row-major double locations [n][p] -> SoA [p][x_ld] in the compute type; columns >= n zeroed.
cudaError_t convert_locations(const double* src, int n, int p, void* dst, int x_ld, bool to_f32, cudaStream_t s);
// One location (p doubles at src) into column `index` of the SoA array.
cudaError_t set_one_location(const double* src, int index, int p, void* dst, int x_ld, bool to_f32, cudaStream_t s);
// rows [row0, row0+rows) of a row-major double matrix with n columns -> rows of a
// matrix with leading dimension ld in float (NaN kept) or double.
// The double-float layout: each double as (hi, lo) floats in its 8-byte slot
// (NaN in both words), for the double-float pair math.
cudaError_t convert_locations_dd(const double* src, int n, int p, void* dst, int x_ld, cudaStream_t s);
cudaError_t set_one_location_dd(const double* src, int index, int p, void* dst, int x_ld, cudaStream_t s);
cudaError_t convert_delta_rows_dd(const double* src, long long rows, int n, void* dst, long long ld, cudaStream_t s);
cudaError_t convert_delta_rows(const double* src, long long rows, int n, void* dst, long long ld, bool to_f32,
                               cudaStream_t s);
// Same from float rows into float storage.
cudaError_t copy_delta_rows_f32(const float* src, long long rows, int n, float* dst, long long ld, cudaStream_t s);
// row_nan[i] = 1 if row i (< n) has a NaN in columns [0, n); rows in [n, rows_padded) get 1.
cudaError_t mark_nan_rows(const void* delta, bool is_f32, int n, long long ld, int* row_nan, int rows_padded,
                          cudaStream_t s);
// The same over a block of `rows` rows of `cols` columns (a row partition of delta).
cudaError_t mark_nan_rows_block(const void* delta, bool is_f32, int rows, int cols, long long ld, int* row_nan,
                                int rows_padded, cudaStream_t s);
// row_nan[i] = 0 for rows < n and 1 for rows in [n, rows_padded), without reading delta.
cudaError_t mark_padding_rows(int n, int* row_nan, int rows_padded, cudaStream_t s);

}  // namespace mdsx
