// Engine state shared by the translation units of libmdsx.so (engine.cu, hmc.cu).
// Not part of the public ABI.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <string>

#include "../../include/mdsx.h"
#include "pair_kernel.cuh"
#include "sweep.h"

using mdsx::KernelShape;
using mdsx::Mode;
using mdsx::SweepArgs;

struct mdsx_engine {
    int p = 0, n = 0;
    // Rows of delta this engine holds and sweeps: [row_begin, row_begin + rows).
    // The whole matrix (row_begin 0, rows N) unless made by mdsx_create_rows.
    int row_begin = 0, rows = 0;
    long flags = 0;
    int device = 0;
    bool trunc = false;
    Mode mode = Mode::kF64;
    bool delta_f32 = false, x_f32 = false;
    // Double-float pair math (MDSX_FLAG_DOUBLE_FLOAT): storage as the FP64 mode
    // `mode`, with FP64 delta and the locations held as (hi, lo) float pairs in
    // their 8-byte slots; unordered-pair schedule only.
    bool dd = false;
    float* d_normal_table = nullptr;       // normal_dd_table (double-float pair math, truncation)
    double* d_normal_table_f64 = nullptr;  // normal_f64_table (FP64 pair math, truncation)

    cudaStream_t own_stream = nullptr;
    cudaEvent_t h2d_done = nullptr;  // recorded after the copy of a caller's host locations
    cudaStream_t stream = nullptr;
    int sm_count = 0;

    KernelShape shape{};
    int n_row_blocks = 0, rows_padded = 0, steps_per_row = 0, grid = 0, max_slots = 0;
    long long n_units = 0;

    void* d_delta = nullptr;
    long long ld = 0;
    void* d_x[2] = {nullptr, nullptr};
    int x_ld = 0;
    int xcur = 0;
    double* d_xin = nullptr;
    double* d_grad[2] = {nullptr, nullptr};
    int gcur = 0;
    double* d_out = nullptr;  // [0] r2, [1] logPhi, [2] sumOfIncrements, [3] error word (int)
    void* d_gpart = nullptr;
    double* d_lpart = nullptr;
    double* d_lrow = nullptr;
    unsigned* d_counts = nullptr;  // [n_row_blocks] + [1]
    int* d_row_nan = nullptr;
    double* h_out = nullptr;  // pinned mirror of d_out
    // Small problems only (null otherwise): pinned staging of a caller's host
    // locations (N*P doubles), so that updateLocations returns without waiting
    // for the device (h2d_done marks the end of the last copy out of it), and a
    // pinned mirror of the gradient (rows*P doubles), brought to the host in the
    // same wait as the sums so that getLogLikelihoodGradient needs no second one.
    double* h_xstage = nullptr;
    double* h_grad = nullptr;
    bool h_grad_valid = false;  // h_grad holds d_grad[gcur] as of the last sweep_and_read

    CUtensorMap tmap_delta{};
    CUtensorMap tmap_x[2]{};

    // Unordered-pair schedule (P <= 6, every precision mode): plan, scratch, tensor maps per location buffer.
    int schedule = MDSX_SWEEP_ROWS;
    bool pairs_built = false;
    int pair_nb = 0, pair_nc = 0, pair_grid = 0, pair_max_slots = 0;
    long long pair_units = 0;
    void* d_rowpart = nullptr;  // float (FP32 math) or double (FP64 math)
    void* d_colpart = nullptr;
    double* d_plpart = nullptr;
    long long* d_pair_begin = nullptr;  // [pair_grid + 1]
    int* d_pair_jfirst = nullptr;       // [pair_nb]
    int* d_pair_jslots = nullptr;       // [pair_nb]
    mdsx::PairMaps pair_maps[2]{};

    bool data_set = false;
    double tau = 0.0, stored_tau = 0.0;
    bool sum_known = false;
    double sum_r2 = 0.0, sum_log = 0.0;  // last computed (ordered-pair, unscaled) sums
    double stored_sum_r2 = 0.0, stored_sum_log = 0.0;
    bool grad_known = false, stored_grad_known = false;
    int last_launches = 0;
    std::string last_error;
};

namespace mdsx {
namespace internal {

int fail(mdsx_engine* e, int code, const std::string& msg);
int cuda_fail(mdsx_engine* e, cudaError_t err, const char* what);

#define MDSX_CUDA(e, call)                                              \
    do {                                                                \
        cudaError_t _err = (call);                                      \
        if (_err != cudaSuccess) return mdsx::internal::cuda_fail(e, _err, #call); \
    } while (0)

struct DeviceGuard {
    int prev = -1;
    bool changed = false;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) == cudaSuccess && prev != dev) changed = cudaSetDevice(dev) == cudaSuccess;
    }
    ~DeviceGuard() {
        if (changed) cudaSetDevice(prev);
    }
};

// Enqueues one fused sweep at the current state (no synchronisation).
int enqueue_sweep(mdsx_engine* e);
int enqueue_sweep_leapfrog(mdsx_engine* e, const mdsx::PairLeapfrog& lf);
// Runs a sweep and reads its sums back; sum and gradient become known.
int sweep_and_read(mdsx_engine* e);
// getSumOfIncrements() from the cached sums and the current precision.
double sum_of_increments(const mdsx_engine* e);

}  // namespace internal
}  // namespace mdsx
