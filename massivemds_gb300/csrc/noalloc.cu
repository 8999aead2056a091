// Allocation-free entry point: the FP32 fused sweep with its scratch in a
// file-scope device array instead of cudaMalloc'd buffers.
//
// Who needs it: callers that must not allocate device memory themselves or
// through this library -- hosts whose GPU memory is owned by another
// allocator (a JVM or R process sharing the device with a framework that has
// reserved it), and sampler loops that cannot afford cudaMalloc/cudaFree in
// their inner loop (both can fail at run time and synchronise the device).
// They pass device buffers for delta, the locations and both outputs; every
// intermediate lives in g_noalloc_scratch below.
//
// Rules of use:
//  - The array takes kNoAllocScratchBytes on each device where this file's
//    module is loaded: under CUDA's default lazy module loading, the devices
//    where the entry point has been called; with CUDA_MODULE_LOADING=EAGER,
//    every device the process uses. It is held until the process exits.
//  - Every call resolves the array's device address with
//    cudaGetSymbolAddress in the caller's current device and context, so a
//    context created after cudaDeviceReset, or a non-primary context made
//    current by the caller, gets its own module's copy.
//  - The call is synchronous: it returns after the results are in the
//    caller's buffers and the kernel's status word has been read back.
//  - All calls share the one array and it keeps the previous call's contents;
//    each call clears the counters and the error word it needs at zero. Calls
//    whose work overlaps on the GPU (other streams, other host threads) race
//    on the scratch: serialise them.
//  - Sizes whose scratch does not fit are rejected with MDSX_EINVAL.
//
// Delta is read once per call when it holds no NaN: the sweep first runs with
// only the padding rows marked (no scan of delta for missing pairs); a NaN
// pair on the kernel's unmasked path then makes the sum NaN, and only in that
// case are the NaN rows marked by a scan and the sweep run again.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>

#include "../../include/mdsx.h"
#include "normal_rational.h"
#include "sweep.h"

namespace {

constexpr size_t kNoAllocScratchBytes = MDSX_NOALLOC_SCRATCH_BYTES;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

int noalloc_fail(int code, const std::string& msg) {
    mdsx::set_global_error(msg);  // read back with mdsx_last_error(NULL)
    return code;
}

int noalloc_cuda_fail(cudaError_t err, const char* what) {
    return noalloc_fail(MDSX_ECUDA, std::string(what) + ": " + cudaGetErrorString(err));
}

#define NOALLOC_CUDA(call)                                      \
    do {                                                        \
        cudaError_t _err = (call);                              \
        if (_err != cudaSuccess) return noalloc_cuda_fail(_err, #call); \
    } while (0)

// Device address of g_noalloc_scratch in the current context.
int scratch_address(void** out) {
    void* ptr = nullptr;
    cudaError_t err = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (err != cudaSuccess) return noalloc_cuda_fail(err, "cudaGetSymbolAddress(g_noalloc_scratch)");
    *out = ptr;
    return MDSX_OK;
}

size_t align256(size_t v) { return (v + 255) & ~size_t(255); }

// One launch for a call's preparation: zero the sums, the error word and the
// counters; mark the padding rows (>= N) for the masked path and clear the
// others; convert the locations to the FP32 SoA layout [P][x_ld].
__global__ void noalloc_prepare_kernel(double* __restrict__ out, unsigned* __restrict__ counts, int n_counts,
                                       int* __restrict__ row_nan, int n, int rows_padded,
                                       const double* __restrict__ locations, int p, float* __restrict__ x, int x_ld) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t0 < 4) out[t0] = 0.0;
    for (long long i = t0; i < n_counts; i += stride) counts[i] = 0u;
    for (long long i = t0; i < rows_padded; i += stride) row_nan[i] = i >= n ? 1 : 0;
    const long long total = (long long)p * x_ld;
    for (long long idx = t0; idx < total; idx += stride) {
        const int q = (int)(idx / x_ld);
        const int i = (int)(idx - (long long)q * x_ld);
        x[idx] = i < n ? (float)locations[(long long)i * p + q] : 0.0f;
    }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_tiled() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void* ptr = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(ptr);
    }
    return fn;
}

int tmap_f32(CUtensorMap* map, const void* base, long long cols, long long rows, long long ld, unsigned box_cols,
             unsigned box_rows) {
    auto fn = encode_tiled();
    if (!fn) return noalloc_fail(MDSX_ECUDA, "cuTensorMapEncodeTiled unavailable from the driver");
    cuuint64_t gdim[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t gstride[1] = {(cuuint64_t)(ld * 4)};
    cuuint32_t box[2] = {box_cols, box_rows};
    cuuint32_t estride[2] = {1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(base), gdim, gstride, box, estride,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return noalloc_fail(MDSX_ECUDA, "cuTensorMapEncodeTiled failed");
    return MDSX_OK;
}

// The plan of the last call on this thread: a sampler calls the sweep again and
// again with the same problem, and the occupancy query, the CTA-slot count (a
// pass over every row block) and the two tensor-map encodings then need not be
// redone. Everything is keyed by what it depends on; the scratch address is
// still resolved on every call.
struct NoallocPlan {
    int device = -1, p = -1, trunc = -1, ctas = 0, sms = 0;  // occupancy of the sweep kernel
    int n = -1, grid = 0, max_slots = 0;                      // CTA slots per row block
    const void* delta = nullptr;                              // tensor maps
    long long delta_ld = -1;
    const void* x = nullptr;
    CUtensorMap tmap_delta{}, tmap_x{};
};
thread_local NoallocPlan t_plan;

}  // namespace

extern "C" {

int mdsx_sweep_f32_noalloc(const float* d_delta, long long delta_ld, const double* d_locations, int location_count,
                           int embedding_dimension, double precision, int truncation, double* d_sum_of_increments,
                           double* d_gradient, void* stream_handle) {
    const int n = location_count, p = embedding_dimension;
    if (!d_delta || !d_locations || !d_sum_of_increments || !d_gradient)
        return noalloc_fail(MDSX_EINVAL, "a device pointer is NULL");
    if (p < 1 || p > MDSX_MAX_DIMENSION) return noalloc_fail(MDSX_EINVAL, "embeddingDimension outside 1..MDSX_MAX_DIMENSION");
    if (n < 1) return noalloc_fail(MDSX_EINVAL, "locationCount must be >= 1");
    if (n > MDSX_NOALLOC_MAX_LOCATIONS)
        return noalloc_fail(MDSX_EINVAL, "locationCount above MDSX_NOALLOC_MAX_LOCATIONS for the allocation-free sweep");
    if (delta_ld < n || delta_ld % 4 != 0)
        return noalloc_fail(MDSX_EINVAL, "delta_ld must be >= locationCount and a multiple of 4 floats");
    if (reinterpret_cast<uintptr_t>(d_delta) % 16 != 0) return noalloc_fail(MDSX_EINVAL, "delta must be 16-byte aligned");
    if (!(precision > 0.0) || !std::isfinite(precision)) return noalloc_fail(MDSX_EINVAL, "precision must be finite and > 0");
    cudaStream_t stream = static_cast<cudaStream_t>(stream_handle);

    int device = 0;
    NOALLOC_CUDA(cudaGetDevice(&device));
    void* base = nullptr;
    int rc = scratch_address(&base);
    if (rc) return rc;

    // Same tile plan as the engine's FP32 mode.
    mdsx::KernelShape shape{};
    if (!mdsx::sweep_shape(mdsx::Mode::kF32, p, &shape)) return noalloc_fail(MDSX_EUNSUPPORTED, "dimension not built");
    NoallocPlan& plan = t_plan;
    const int trunc_key = truncation != 0;
    if (plan.device != device || plan.p != p || plan.trunc != trunc_key) {
        plan = NoallocPlan{};
        NOALLOC_CUDA(mdsx::sweep_occupancy(mdsx::Mode::kF32, p, truncation != 0, &plan.ctas));
        NOALLOC_CUDA(cudaDeviceGetAttribute(&plan.sms, cudaDevAttrMultiProcessorCount, device));
        plan.device = device;
        plan.p = p;
        plan.trunc = trunc_key;
    }
    const int rb = shape.rb;
    const int n_row_blocks = (n + rb - 1) / rb;
    const int rows_padded = n_row_blocks * rb;
    const int steps_per_row = (n + mdsx::kStepCols - 1) / mdsx::kStepCols;
    const long long n_units = (long long)n_row_blocks * steps_per_row;
    const int grid = (int)std::min<long long>(n_units, (long long)plan.sms * std::max(plan.ctas, 1));
    if (plan.n != n || plan.grid != grid) {
        int max_slots = 1;
        for (int b = 0; b < n_row_blocks; ++b) {
            const long long u0 = (long long)b * steps_per_row, u1 = u0 + steps_per_row - 1;
            max_slots =
                std::max(max_slots, mdsx::cta_of_unit(u1, n_units, grid) - mdsx::cta_of_unit(u0, n_units, grid) + 1);
        }
        plan.n = n;
        plan.grid = grid;
        plan.max_slots = max_slots;
        plan.delta = nullptr;  // the tensor maps depend on n
        plan.x = nullptr;
    }
    const int max_slots = plan.max_slots;
    const int x_ld = (int)std::max<long long>((n + mdsx::kStepCols - 1) / mdsx::kStepCols * mdsx::kStepCols, rows_padded);

    // Carve the scratch: [out: 4 doubles][counters][row marks][x SoA][gpart][lpart][lrow]
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t at = off;
        off = align256(off + bytes);
        return static_cast<unsigned char*>(base) + at;
    };
    double* out = reinterpret_cast<double*>(take(4 * sizeof(double)));
    unsigned* counts = reinterpret_cast<unsigned*>(take(((size_t)n_row_blocks + 1) * sizeof(unsigned)));
    int* row_nan = reinterpret_cast<int*>(take((size_t)rows_padded * sizeof(int)));
    float* x = reinterpret_cast<float*>(take((size_t)p * x_ld * sizeof(float)));
    float* gpart = reinterpret_cast<float*>(take((size_t)n_row_blocks * max_slots * rb * p * sizeof(float)));
    double* lpart =
        reinterpret_cast<double*>(take((size_t)n_row_blocks * max_slots * mdsx::kConsumerWarps * 2 * sizeof(double)));
    double* lrow = reinterpret_cast<double*>(take((size_t)n_row_blocks * 2 * sizeof(double)));
    if (off > kNoAllocScratchBytes)
        return noalloc_fail(MDSX_EINVAL, "problem needs " + std::to_string(off) + " bytes of scratch; the allocation-free "
                            "sweep has " + std::to_string(kNoAllocScratchBytes));

    // First pass: only the padding rows (>= N) take the masked path.
    {
        const long long work = std::max<long long>((long long)p * x_ld, rows_padded);
        const int blocks = (int)std::min<long long>((work + 255) / 256, 1024);
        noalloc_prepare_kernel<<<blocks, 256, 0, stream>>>(out, counts, n_row_blocks + 1, row_nan, n, rows_padded,
                                                           d_locations, p, x, x_ld);
        NOALLOC_CUDA(cudaGetLastError());
    }

    if (plan.delta != d_delta || plan.delta_ld != delta_ld) {
        plan.delta = nullptr;
        rc = tmap_f32(&plan.tmap_delta, d_delta, n, n, delta_ld, mdsx::kStepCols, rb);
        if (rc) return rc;
        plan.delta = d_delta;
        plan.delta_ld = delta_ld;
    }
    if (plan.x != x) {
        rc = tmap_f32(&plan.tmap_x, x, n, p, x_ld, mdsx::kStepCols, p);
        if (rc) return rc;
        plan.x = x;
    }
    const CUtensorMap& tmap_delta = plan.tmap_delta;
    const CUtensorMap& tmap_x = plan.tmap_x;

    mdsx::SweepArgs a{};
    a.n = n;
    a.row_offset = 0;
    a.rows = n;
    a.n_row_blocks = n_row_blocks;
    a.steps_per_row = steps_per_row;
    a.grid = grid;
    a.n_units = n_units;
    a.max_slots = max_slots;
    a.rows_padded = rows_padded;
    a.x_ld = x_ld;
    a.x = x;
    a.row_nan = row_nan;
    const double tau = precision, s = std::sqrt(tau);
    a.tau = tau;
    a.sqrt_tau = s;
    a.k_e = (float)(-0.5 * tau * 1.4426950408889634074);
    a.log2_k2 = (float)std::log2(1.0 / std::sqrt(2.0 * M_PI * tau));
    a.tp0 = (float)(mdsx::kTailP0 / tau);
    a.tp1 = (float)(mdsx::kTailP1 / s);
    a.tp2 = (float)mdsx::kTailP2;
    a.ts0 = (float)(mdsx::kTailS0 / (s * s * s));
    a.ts1 = (float)(mdsx::kTailS1 / (s * s));
    a.ts2 = (float)(mdsx::kTailS2 / s);
    a.gpart = gpart;
    a.lpart = lpart;
    a.lrow = lrow;
    a.rb_count = counts;
    a.done_count = counts + n_row_blocks;
    a.grad_out = d_gradient;
    a.sums_out = out;
    a.truncation = truncation ? 1 : 0;
    a.err = reinterpret_cast<int*>(out + 3);
    a.sum_copy = d_sum_of_increments;  // the last CTA writes the caller's sum itself
    // Counters, sums and the error word start at zero on each pass (the
    // preparation kernel clears them for the first).
    double host_out[4];
    for (int pass = 0; pass < 2; ++pass) {
        if (pass == 1) {  // the second pass starts from zero again
            NOALLOC_CUDA(cudaMemsetAsync(out, 0, 4 * sizeof(double), stream));
            NOALLOC_CUDA(cudaMemsetAsync(counts, 0, ((size_t)n_row_blocks + 1) * sizeof(unsigned), stream));
        }
        NOALLOC_CUDA(mdsx::sweep_launch(mdsx::Mode::kF32, p, truncation != 0, grid, tmap_delta, tmap_x, a, stream));
        // the status and the sum to the host, then one synchronisation
        NOALLOC_CUDA(cudaMemcpyAsync(host_out, out, sizeof(host_out), cudaMemcpyDeviceToHost, stream));
        NOALLOC_CUDA(cudaStreamSynchronize(stream));
        int dev_err = 0;
        std::memcpy(&dev_err, &host_out[3], sizeof(int));
        if (dev_err != 0) return noalloc_fail(MDSX_ETIMEOUT, "a bounded device wait in the sweep kernel timed out");
        // A finite sum: no NaN pair reached the unmasked path. Otherwise mark
        // the rows holding a NaN and sweep again (NaN locations stay NaN).
        if (!std::isnan(host_out[2]) || pass == 1) break;
        NOALLOC_CUDA(mdsx::mark_nan_rows(d_delta, true, n, delta_ld, row_nan, rows_padded, stream));
    }
    return MDSX_OK;
}

}  // extern "C"
