// The CUDA engine behind the C ABI in include/mdsx.h.
//
// State machine of the MassiveMDS CPU engine (src/NewMultiDimensionalScaling.hpp),
// restated for device-resident data:
//   updateLocations  -> locations dirty (sum and gradient unknown)       (:134-166)
//   setParameters    -> tau; with truncation both results dirty         (:262-274)
//   getSumOfIncrements / getLogLikelihoodGradient -> one fused sweep if the
//                       result is unknown; the sweep yields both results (:193-203, :281-302)
//   storeState       -> copy locations, keep sums, tau (and the gradient) (:205-217)
//   restoreState     -> swap locations back, restore sums as known, tau   (:234-255)
//   acceptState      -> nothing to do for whole-matrix updates            (:226-232)
//   makeDirty        -> both results unknown                             (:276-279)
// Device layout: delta row-major [N][ld] (ld = N rounded up to 16 bytes),
// locations SoA [P][x_ld] in the compute precision (two buffers: current and
// stored), gradient [N][P] double (two buffers), scratch sized by the tile plan.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/mdsx.h"
#include "normal_rational.h"
#include "pair_kernel.cuh"
#include "pair_plan.h"
#include "engine_internal.h"
#include "sweep.h"
#include "fault.h"



namespace mdsx {
namespace internal {

thread_local std::string g_create_error;

// Small problems (N * P doubles up to this size) go through pinned host
// copies on the host-API path: updateLocations stages the caller's locations
// and returns without a wait, and every host-API sweep brings the gradient to
// the host with its sums, so that getLogLikelihoodGradient after
// getLogLikelihood costs no second wait. Above it, a host memcpy of the
// locations or the gradient costs more than the wait it saves (measured on
// GB300 with a Grace host: N = 1000, P = 2 gains 9 %; N = 20 000 loses 7 %).
constexpr size_t kHostMirrorMaxBytes = size_t(64) << 10;

int fail(mdsx_engine* e, int code, const std::string& msg) {
    if (e)
        e->last_error = msg;
    else
        g_create_error = msg;
    return code;
}

int cuda_fail(mdsx_engine* e, cudaError_t err, const char* what) {
    std::string msg = std::string(what) + ": " + cudaGetErrorString(err);
    return fail(e, err == cudaErrorMemoryAllocation ? MDSX_ENOMEM : MDSX_ECUDA, msg);
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

long long round_up(long long v, long long m) { return (v + m - 1) / m * m; }

int make_tmap_2d(mdsx_engine* e, CUtensorMap* map, void* base, bool f32, long long cols, long long rows,
                 long long ld_elems, unsigned box_cols, unsigned box_rows,
                 CUtensorMapSwizzle swizzle = CU_TENSOR_MAP_SWIZZLE_NONE) {
    auto fn = encode_tiled();
    if (!fn) return fail(e, MDSX_ECUDA, "cuTensorMapEncodeTiled unavailable from the driver");
    const int elem = f32 ? 4 : 8;
    cuuint64_t gdim[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t gstride[1] = {(cuuint64_t)(ld_elems * elem)};
    cuuint32_t box[2] = {box_cols, box_rows};
    cuuint32_t estride[2] = {1, 1};
    CUresult r = fn(map, f32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, base, gdim,
                    gstride, box, estride, CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        char buf[128];
        snprintf(buf, sizeof buf, "cuTensorMapEncodeTiled failed (CUresult %d)", (int)r);
        return fail(e, MDSX_ECUDA, buf);
    }
    return MDSX_OK;
}

void free_all(mdsx_engine* e) {
    cudaFree(e->d_delta);
    cudaFree(e->d_x[0]);
    cudaFree(e->d_x[1]);
    cudaFree(e->d_xin);
    cudaFree(e->d_grad[0]);
    cudaFree(e->d_grad[1]);
    cudaFree(e->d_out);
    cudaFree(e->d_gpart);
    cudaFree(e->d_lpart);
    cudaFree(e->d_lrow);
    cudaFree(e->d_counts);
    cudaFree(e->d_row_nan);
    cudaFree(e->d_rowpart);
    cudaFree(e->d_colpart);
    cudaFree(e->d_plpart);
    cudaFree(e->d_pair_begin);
    cudaFree(e->d_pair_jfirst);
    cudaFree(e->d_pair_jslots);
    cudaFree(e->d_normal_table);
    cudaFree(e->d_normal_table_f64);
    if (e->h_out) cudaFreeHost(e->h_out);
    if (e->h_xstage) cudaFreeHost(e->h_xstage);
    if (e->h_grad) cudaFreeHost(e->h_grad);
    if (e->h2d_done) cudaEventDestroy(e->h2d_done);
    if (e->own_stream) cudaStreamDestroy(e->own_stream);
}

// Unordered-pair schedule: units (J, I), I >= 4J, split evenly over
// G <= U CTAs; scratch for row, column and likelihood partials; tensor maps of
// delta (plain and 128-byte swizzled boxes) and of both location buffers.
int plan_pairs(mdsx_engine* e) {
    int ctas = 0;
    const bool f64 = !e->x_f32;
    MDSX_CUDA(e, mdsx::pair_occupancy(e->p, e->trunc, e->mode, &ctas, e->dd));
    if (ctas < 1) return fail(e, MDSX_ECUDA, "pair sweep kernel cannot be resident on this device");
    e->pair_nb = (e->n + mdsx::kPairCols - 1) / mdsx::kPairCols;
    e->pair_nc = (e->n + mdsx::kPairRows - 1) / mdsx::kPairRows;
    e->pair_units = mdsx::pair_units_before(e->pair_nb, e->pair_nc);
    const mdsx::PairPlan plan = mdsx::pair_plan({e->n}, (long long)e->sm_count * ctas);
    const mdsx::PairInstancePlan& q = plan.inst[0];
    e->pair_grid = plan.grid;
    e->pair_max_slots = q.max_slots;
    const int G = plan.grid;
    const std::vector<long long>& begin = plan.cta_begin;
    const std::vector<int>& jfirst = q.j_first;
    const std::vector<int>& jslots = q.j_slots;
    MDSX_CUDA(e, mdsx::device_malloc(&e->d_pair_begin, (size_t)(G + 1) * sizeof(long long)));
    MDSX_CUDA(e, mdsx::device_malloc(&e->d_pair_jfirst, (size_t)e->pair_nb * sizeof(int)));
    MDSX_CUDA(e, mdsx::device_malloc(&e->d_pair_jslots, (size_t)e->pair_nb * sizeof(int)));
    MDSX_CUDA(e, cudaMemcpy(e->d_pair_begin, begin.data(), (size_t)(G + 1) * sizeof(long long),
                            cudaMemcpyHostToDevice));
    MDSX_CUDA(e, cudaMemcpy(e->d_pair_jfirst, jfirst.data(), (size_t)e->pair_nb * sizeof(int), cudaMemcpyHostToDevice));
    MDSX_CUDA(e, cudaMemcpy(e->d_pair_jslots, jslots.data(), (size_t)e->pair_nb * sizeof(int), cudaMemcpyHostToDevice));
    const size_t part_bytes = f64 ? sizeof(double) : sizeof(float);
    MDSX_CUDA(e, mdsx::device_malloc(&e->d_rowpart, (size_t)e->pair_units * mdsx::kPairRows * e->p * part_bytes));
    MDSX_CUDA(e, mdsx::device_malloc(&e->d_colpart, (size_t)e->pair_nb * e->pair_max_slots * mdsx::kPairWarps * e->p *
                                               mdsx::kPairCols * part_bytes));
    MDSX_CUDA(e, mdsx::device_malloc(&e->d_plpart, (size_t)e->pair_grid * mdsx::kPairWarps * 2 * sizeof(double)));
    for (int b = 0; b < 2; ++b) {
        mdsx::PairMaps& m = e->pair_maps[b];
        int rc = make_tmap_2d(e, &m.a, e->d_delta, e->delta_f32, e->n, e->n, e->ld, mdsx::kPairCols,
                              mdsx::kPairRows);
        if (!rc)
            rc = make_tmap_2d(e, &m.b, e->d_delta, e->delta_f32, e->n, e->n, e->ld, e->delta_f32 ? 32 : 16,
                              mdsx::kPairCols, CU_TENSOR_MAP_SWIZZLE_128B);
        // the location maps span x_ld columns, so the flags of rows >= N are read from memory (1), not filled
        if (!rc)
            rc = make_tmap_2d(e, &m.xi, e->d_x[b], e->x_f32, e->x_ld, e->p + 1, e->x_ld, mdsx::kPairRows, e->p + 1);
        if (!rc)
            rc = make_tmap_2d(e, &m.xj, e->d_x[b], e->x_f32, e->x_ld, e->p + 1, e->x_ld, mdsx::kPairCols, e->p + 1);
        if (rc) return rc;
    }
    return MDSX_OK;
}

// The normal-tail tables on the host, computed once per process (the series
// coefficients take long-double erfc, exp and log1p, which are slow where long
// double is a software type) and copied to each engine that needs them.
const std::vector<double>& normal_f64_table_host() {
    static const std::vector<double> table = [] {
        std::vector<double> t(mdsx::kNormalF64Doubles);
        mdsx::normal_f64_table(t.data());
        return t;
    }();
    return table;
}
const std::vector<float>& normal_dd_table_host() {
    static const std::vector<float> table = [] {
        std::vector<float> t(mdsx::kNormalDDFloats);
        mdsx::normal_dd_table(t.data());
        return t;
    }();
    return table;
}

int plan_and_allocate(mdsx_engine* e) {
    if (!mdsx::sweep_shape(e->mode, e->p, &e->shape))
        return fail(e, MDSX_EUNSUPPORTED, "embedding dimension not built (1..MDSX_MAX_DIMENSION)");
    int ctas = 0;
    MDSX_CUDA(e, mdsx::sweep_occupancy(e->mode, e->p, e->trunc, &ctas));
    if (ctas < 1) return fail(e, MDSX_ECUDA, "sweep kernel cannot be resident on this device");
    const int rb = e->shape.rb;
    e->n_row_blocks = (e->rows + rb - 1) / rb;
    e->rows_padded = e->n_row_blocks * rb;
    // Stream-K partition: U = row blocks x 128-column stages, split evenly
    // over G <= U CTAs (so no CTA has an empty range).
    e->steps_per_row = (e->n + mdsx::kStepCols - 1) / mdsx::kStepCols;
    e->n_units = (long long)e->n_row_blocks * e->steps_per_row;
    const long long grid_max = (long long)e->sm_count * ctas;
    e->grid = (int)std::min<long long>(e->n_units, grid_max);
    e->max_slots = 1;
    for (int rb = 0; rb < e->n_row_blocks; ++rb) {
        const long long u0 = (long long)rb * e->steps_per_row, u1 = u0 + e->steps_per_row - 1;
        const int slots = mdsx::cta_of_unit(u1, e->n_units, e->grid) - mdsx::cta_of_unit(u0, e->n_units, e->grid) + 1;
        e->max_slots = std::max(e->max_slots, slots);
    }

    const int delta_elem = e->shape.delta_elem_bytes;
    e->ld = round_up(e->n, 16 / delta_elem);
    e->x_ld = (int)std::max<long long>(round_up(e->n, mdsx::kStepCols), (long long)e->row_begin + e->rows_padded);
    // P location rows and one flag row (read by the unordered-pair schedule)
    const size_t x_bytes = (size_t)(e->p + 1) * e->x_ld * e->shape.x_elem_bytes;
    const size_t acc_bytes = e->x_f32 ? 4 : 8;

    MDSX_CUDA(e, mdsx::device_malloc(&e->d_delta, (size_t)e->rows * e->ld * delta_elem));
    MDSX_CUDA(e, mdsx::device_malloc(&e->d_x[0], x_bytes));
    MDSX_CUDA(e, mdsx::device_malloc(&e->d_x[1], x_bytes));
    MDSX_CUDA(e, cudaMemsetAsync(e->d_x[0], 0, x_bytes, e->stream));
    MDSX_CUDA(e, cudaMemsetAsync(e->d_x[1], 0, x_bytes, e->stream));
    MDSX_CUDA(e, mdsx::device_malloc(&e->d_xin, (size_t)e->n * e->p * sizeof(double)));
    MDSX_CUDA(e, mdsx::device_malloc(&e->d_grad[0], (size_t)e->rows * e->p * sizeof(double)));
    MDSX_CUDA(e, mdsx::device_malloc(&e->d_grad[1], (size_t)e->rows * e->p * sizeof(double)));
    MDSX_CUDA(e, mdsx::device_malloc(&e->d_out, 4 * sizeof(double)));
    MDSX_CUDA(e, cudaMemsetAsync(e->d_out, 0, 4 * sizeof(double), e->stream));
    MDSX_CUDA(e, mdsx::device_malloc(&e->d_gpart, (size_t)e->n_row_blocks * e->max_slots * rb * e->p * acc_bytes));
    MDSX_CUDA(e, mdsx::device_malloc(&e->d_lpart,
                            (size_t)e->n_row_blocks * e->max_slots * mdsx::kConsumerWarps * 2 * sizeof(double)));
    MDSX_CUDA(e, mdsx::device_malloc(&e->d_lrow, (size_t)e->n_row_blocks * 2 * sizeof(double)));
    MDSX_CUDA(e, mdsx::device_malloc(&e->d_counts, ((size_t)e->n_row_blocks + 1) * sizeof(unsigned)));
    MDSX_CUDA(e, cudaMemsetAsync(e->d_counts, 0, ((size_t)e->n_row_blocks + 1) * sizeof(unsigned), e->stream));
    MDSX_CUDA(e, mdsx::device_malloc(&e->d_row_nan, (size_t)e->rows_padded * sizeof(int)));
    MDSX_CUDA(e, cudaMemsetAsync(e->d_row_nan, 0, (size_t)e->rows_padded * sizeof(int), e->stream));
    MDSX_CUDA(e, mdsx::host_malloc(&e->h_out, 4 * sizeof(double)));
    if ((size_t)e->n * e->p * sizeof(double) <= kHostMirrorMaxBytes) {
        MDSX_CUDA(e, mdsx::host_malloc(&e->h_xstage, (size_t)e->n * e->p * sizeof(double)));
        MDSX_CUDA(e, mdsx::host_malloc(&e->h_grad, (size_t)e->rows * e->p * sizeof(double)));
    }

    int rc = make_tmap_2d(e, &e->tmap_delta, e->d_delta, e->delta_f32, e->n, e->rows, e->ld, mdsx::kStepCols, rb);
    if (rc) return rc;
    for (int b = 0; b < 2; ++b) {
        rc = make_tmap_2d(e, &e->tmap_x[b], e->d_x[b], e->x_f32, e->n, e->p, e->x_ld, mdsx::kStepCols, e->p);
        if (rc) return rc;
    }
    // The unordered-pair schedule needs both delta_ij and delta_ji: whole-matrix engines only.
    if (mdsx::pair_built(e->mode, e->p) && e->rows == e->n) {
        rc = plan_pairs(e);
        if (rc) return rc;
        // Measured on GB300: with truncation the pair math dominates and sharing it between
        // (i, j) and (j, i) wins by 17-29 % in FP32 (N = 5 000 .. 50 000, P = 1 .. 4); without it
        // the FP32 row-block sweep is already at the memory bound and its single kernel is
        // faster. FP64 is bound by the FP64 pipe either way: pairs win by 1.4x untruncated and
        // 1.8x truncated (N = 20 000, P = 2).
        if (e->trunc || e->mode != Mode::kF32) e->schedule = MDSX_SWEEP_PAIRS;
    }
    // the FP64 math's normal-tail table (pair and row-block schedules)
    if (!e->dd && e->mode != Mode::kF32 && e->trunc) {
        const std::vector<double>& table = normal_f64_table_host();
        MDSX_CUDA(e, mdsx::device_malloc(&e->d_normal_table_f64, table.size() * sizeof(double)));
        MDSX_CUDA(e, cudaMemcpy(e->d_normal_table_f64, table.data(), table.size() * sizeof(double),
                                cudaMemcpyHostToDevice));
    }
    if (e->dd) {
        if (e->schedule != MDSX_SWEEP_PAIRS)
            return fail(e, MDSX_EUNSUPPORTED,
                        "double-float pair math runs on the unordered-pair schedule only (P <= 6, whole matrix)");
        if (e->trunc) {
            const std::vector<float>& table = normal_dd_table_host();
            MDSX_CUDA(e, mdsx::device_malloc(&e->d_normal_table, table.size() * sizeof(float)));
            MDSX_CUDA(e, cudaMemcpy(e->d_normal_table, table.data(), table.size() * sizeof(float),
                                    cudaMemcpyHostToDevice));
        }
    }
    MDSX_CUDA(e, cudaStreamSynchronize(e->stream));
    return MDSX_OK;
}

// Caller locations (device, row-major N x P doubles) into the current SoA buffer.
cudaError_t locations_to_soa(mdsx_engine* e, const double* d_src) {
    return e->dd ? mdsx::convert_locations_dd(d_src, e->n, e->p, e->d_x[e->xcur], e->x_ld, e->stream)
                 : mdsx::convert_locations(d_src, e->n, e->p, e->d_x[e->xcur], e->x_ld, e->x_f32, e->stream);
}

// Flag row (row P) of both location buffers from the NaN-row marks.
cudaError_t write_flags(mdsx_engine* e) {
    if (e->rows != e->n) return cudaSuccess;  // the flag row serves the unordered-pair schedule only
    const size_t elem = e->x_f32 ? sizeof(float) : sizeof(double);
    for (int b = 0; b < 2; ++b) {
        cudaError_t err = mdsx::write_flag_row(e->d_row_nan, e->n, e->rows_padded,
                                               static_cast<char*>(e->d_x[b]) + (size_t)e->p * e->x_ld * elem,
                                               e->x_f32, e->x_ld, e->stream);
        if (err != cudaSuccess) return err;
    }
    return cudaSuccess;
}

// Clears the error word and self-resetting counters after a failed sweep.
void reset_scratch(mdsx_engine* e) {
    cudaMemsetAsync(e->d_counts, 0, ((size_t)e->n_row_blocks + 1) * sizeof(unsigned), e->stream);
    cudaMemsetAsync(e->d_out, 0, 4 * sizeof(double), e->stream);
    cudaStreamSynchronize(e->stream);
}

SweepArgs make_args(mdsx_engine* e) {
    SweepArgs a{};
    a.n = e->n;
    a.row_offset = e->row_begin;
    a.rows = e->rows;
    a.n_row_blocks = e->n_row_blocks;
    a.steps_per_row = e->steps_per_row;
    a.grid = e->grid;
    a.n_units = e->n_units;
    a.max_slots = e->max_slots;
    a.rows_padded = e->rows_padded;
    a.x_ld = e->x_ld;
    a.x = e->d_x[e->xcur];
    a.row_nan = e->d_row_nan;
    const double tau = e->tau, s = std::sqrt(tau);
    a.tau = tau;
    a.sqrt_tau = s;
    // FP32 constants, in terms of d (z = s * d):
    //   E'   = exp(-tau d^2 / 2) / sqrt(2 pi tau) = 2^(d^2 k_e + log2_k2)
    //   1/Phi = S(d) / (S(d) - E' P(d)),  S monic cubic, P quadratic
    a.k_e = (float)(-0.5 * tau * 1.4426950408889634074);
    a.log2_k2 = (float)std::log2(1.0 / std::sqrt(2.0 * M_PI * tau));
    a.tp0 = (float)(mdsx::kTailP0 / tau);
    a.tp1 = (float)(mdsx::kTailP1 / s);
    a.tp2 = (float)mdsx::kTailP2;
    a.ts0 = (float)(mdsx::kTailS0 / (s * s * s));
    a.ts1 = (float)(mdsx::kTailS1 / (s * s));
    a.ts2 = (float)(mdsx::kTailS2 / s);
    a.gpart = e->d_gpart;
    a.lpart = e->d_lpart;
    a.lrow = e->d_lrow;
    a.rb_count = e->d_counts;
    a.done_count = e->d_counts + e->n_row_blocks;
    a.grad_out = e->d_grad[e->gcur];
    a.sums_out = e->d_out;
    a.truncation = e->trunc ? 1 : 0;
    a.err = reinterpret_cast<int*>(e->d_out + 3);
    a.normal_table_f64 = e->d_normal_table_f64;
    return a;
}

// Arguments of the unordered-pair sweep at the engine's current state.
mdsx::PairArgs make_pair_args(mdsx_engine* e) {
    const SweepArgs a = make_args(e);
    mdsx::PairArgs pa{};
    pa.n = e->n;
    pa.nb = e->pair_nb;
    pa.nc = e->pair_nc;
    pa.grid = e->pair_grid;
    pa.max_slots = e->pair_max_slots;
    pa.truncation = a.truncation;
    pa.n_units = e->pair_units;
    pa.k_e = a.k_e;
    pa.log2_k2 = a.log2_k2;
    pa.tp0 = a.tp0;
    pa.tp1 = a.tp1;
    pa.tp2 = a.tp2;
    pa.ts0 = a.ts0;
    pa.ts1 = a.ts1;
    pa.ts2 = a.ts2;
    pa.tau = a.tau;
    pa.sqrt_tau = a.sqrt_tau;
    pa.rowpart = e->d_rowpart;
    pa.colpart = e->d_colpart;
    pa.lpart = e->d_plpart;
    pa.cta_begin = e->d_pair_begin;
    pa.j_first_cta = e->d_pair_jfirst;
    pa.j_slots = e->d_pair_jslots;
    pa.grad_out = a.grad_out;
    pa.sums_out = a.sums_out;
    pa.err = a.err;
    pa.normal_table = e->d_normal_table;
    pa.normal_table_f64 = e->d_normal_table_f64;
    return pa;
}

// Enqueues one fused sweep; does not synchronise.
int enqueue_sweep(mdsx_engine* e) {
    if (!e->data_set) return fail(e, MDSX_ESTATE, "setPairwiseData has not been called");
    if (!(e->tau > 0.0)) return fail(e, MDSX_ESTATE, "precision (setParameters) not set");
    e->h_grad_valid = false;
    MDSX_CUDA(e, mdsx::launch_fault());
    if (e->schedule == MDSX_SWEEP_PAIRS) {
        const mdsx::PairArgs pa = make_pair_args(e);
        MDSX_CUDA(e, mdsx::pair_launch(e->p, e->trunc, e->mode, e->pair_maps[e->xcur], pa, e->stream, e->dd));
        e->last_launches = 2;
        return MDSX_OK;
    }
    SweepArgs a = make_args(e);
    MDSX_CUDA(e, mdsx::sweep_launch(e->mode, e->p, e->trunc, e->grid, e->tmap_delta, e->tmap_x[e->xcur], a,
                                    e->stream));
    e->last_launches = 1;
    return MDSX_OK;
}

// Enqueues one fused sweep whose finish kernel also applies the leapfrog step
// `lf` (unordered-pair schedule only; MDSX_EUNSUPPORTED otherwise, and the
// caller runs its own kick/drift after enqueue_sweep).
int enqueue_sweep_leapfrog(mdsx_engine* e, const mdsx::PairLeapfrog& lf) {
    if (!e->data_set) return fail(e, MDSX_ESTATE, "setPairwiseData has not been called");
    if (!(e->tau > 0.0)) return fail(e, MDSX_ESTATE, "precision (setParameters) not set");
    if (e->schedule != MDSX_SWEEP_PAIRS) return MDSX_EUNSUPPORTED;
    e->h_grad_valid = false;
    MDSX_CUDA(e, mdsx::launch_fault());
    mdsx::PairArgs pa = make_pair_args(e);
    pa.leapfrog = 1;
    pa.leap = lf;
    MDSX_CUDA(e, mdsx::pair_launch(e->p, e->trunc, e->mode, e->pair_maps[e->xcur], pa, e->stream, e->dd));
    e->last_launches = 2;
    return MDSX_OK;
}

// Runs a sweep and brings its sums to the host; both results become known.
int sweep_and_read(mdsx_engine* e) {
    int rc = enqueue_sweep(e);
    if (rc) return rc;
    MDSX_CUDA(e, cudaMemcpyAsync(e->h_out, e->d_out, 4 * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
    if (e->h_grad)
        MDSX_CUDA(e, cudaMemcpyAsync(e->h_grad, e->d_grad[e->gcur], (size_t)e->rows * e->p * sizeof(double),
                                     cudaMemcpyDeviceToHost, e->stream));
    MDSX_CUDA(e, cudaStreamSynchronize(e->stream));
    int dev_err = 0;
    std::memcpy(&dev_err, &e->h_out[3], sizeof(int));
    if (dev_err != 0) {
        reset_scratch(e);
        e->sum_known = e->grad_known = false;
        return fail(e, MDSX_ETIMEOUT, "a bounded device wait in the sweep kernel timed out");
    }
    e->sum_r2 = e->h_out[0];
    e->sum_log = e->h_out[1];
    e->sum_known = true;
    e->grad_known = true;
    e->h_grad_valid = e->h_grad != nullptr;
    return MDSX_OK;
}

double sum_of_increments(const mdsx_engine* e) {
    // src/NewMultiDimensionalScaling.hpp:198-202 with the total halved at :554-557.
    const double half_r2 = 0.5 * e->sum_r2;
    if (e->trunc) return 0.5 * e->tau * half_r2 + 0.5 * e->sum_log;
    return 0.5 * e->tau * half_r2;
}

}  // namespace internal
}  // namespace mdsx

using namespace mdsx::internal;

extern "C" {

const char* mdsx_version(void) { return "mdsx 0.1 (sm_103a)"; }

int mdsx_create_rows(int embedding_dimension, int location_count, long flags, int device, int row_begin, int row_end,
                     mdsx_engine** out) {
    if (!out) return fail(nullptr, MDSX_EINVAL, "out is NULL");
    *out = nullptr;
    if (embedding_dimension < 1) return fail(nullptr, MDSX_EINVAL, "embeddingDimension must be >= 1");
    if (embedding_dimension > MDSX_MAX_DIMENSION)
        return fail(nullptr, MDSX_EUNSUPPORTED, "embeddingDimension above MDSX_MAX_DIMENSION");
    if (location_count < 1) return fail(nullptr, MDSX_EINVAL, "locationCount must be >= 1");
    if (location_count > (1 << 20)) return fail(nullptr, MDSX_EINVAL, "locationCount above 2^20");
    if (row_begin < 0 || row_end > location_count || row_begin >= row_end)
        return fail(nullptr, MDSX_EINVAL, "row range must satisfy 0 <= row_begin < row_end <= locationCount");
    if ((flags & MDSX_FLAG_DOUBLE_FLOAT) && (flags & MDSX_FLAG_FLOAT))
        return fail(nullptr, MDSX_EINVAL, "MDSX_FLAG_DOUBLE_FLOAT and MDSX_FLAG_FLOAT exclude each other");
    int count = 0;
    cudaError_t err = cudaGetDeviceCount(&count);
    if (err != cudaSuccess || count == 0)
        return fail(nullptr, MDSX_ECUDA, std::string("no CUDA device: ") + cudaGetErrorString(err));
    if (device < 0) {
        if (cudaGetDevice(&device) != cudaSuccess) device = 0;
    }
    if (device >= count) return fail(nullptr, MDSX_EINVAL, "device index out of range");

    auto* e = new mdsx_engine;
    e->p = embedding_dimension;
    e->n = location_count;
    e->row_begin = row_begin;
    e->rows = row_end - row_begin;
    e->flags = flags;
    e->device = device;
    e->trunc = (flags & MDSX_FLAG_LEFT_TRUNCATION) != 0;
    e->dd = (flags & MDSX_FLAG_DOUBLE_FLOAT) != 0;
    if (flags & MDSX_FLAG_FLOAT) {
        e->mode = Mode::kF32;
        e->delta_f32 = e->x_f32 = true;
    } else if (flags & MDSX_FLAG_DELTA_F32) {
        e->mode = Mode::kF64DeltaF32;
        e->delta_f32 = true;
    } else {
        e->mode = Mode::kF64;
    }
    DeviceGuard guard(device);
    int rc = MDSX_OK;
    if ((err = cudaDeviceGetAttribute(&e->sm_count, cudaDevAttrMultiProcessorCount, device)) != cudaSuccess)
        rc = cuda_fail(e, err, "cudaDeviceGetAttribute");
    if (!rc && (err = cudaStreamCreateWithFlags(&e->own_stream, cudaStreamNonBlocking)) != cudaSuccess)
        rc = cuda_fail(e, err, "cudaStreamCreate");
    if (!rc && (err = cudaEventCreateWithFlags(&e->h2d_done, cudaEventDisableTiming)) != cudaSuccess)
        rc = cuda_fail(e, err, "cudaEventCreate");
    if (!rc) {
        e->stream = e->own_stream;
        rc = plan_and_allocate(e);
    }
    if (rc) {
        g_create_error = e->last_error;
        free_all(e);
        delete e;
        return rc;
    }
    *out = e;
    return MDSX_OK;
}

int mdsx_create(int embedding_dimension, int location_count, long flags, int device, mdsx_engine** out) {
    return mdsx_create_rows(embedding_dimension, location_count, flags, device, 0, location_count, out);
}

int mdsx_get_row_range(const mdsx_engine* e, int* row_begin, int* row_end) {
    if (!e || !row_begin || !row_end) return MDSX_EINVAL;
    *row_begin = e->row_begin;
    *row_end = e->row_begin + e->rows;
    return MDSX_OK;
}

int mdsx_destroy(mdsx_engine* e) {
    if (!e) return MDSX_EINVAL;
    {
        DeviceGuard guard(e->device);
        if (e->stream) cudaStreamSynchronize(e->stream);
        free_all(e);
    }
    delete e;
    return MDSX_OK;
}

const char* mdsx_last_error(const mdsx_engine* e) {
    return e ? e->last_error.c_str() : g_create_error.c_str();
}

int mdsx_update_locations(mdsx_engine* e, int index, const double* x, size_t length) {
    if (!e) return MDSX_EINVAL;
    if (!x) return fail(e, MDSX_EINVAL, "locations pointer is NULL");
    DeviceGuard guard(e->device);
    if (index == -1) {
        if (length != (size_t)e->n * e->p) return fail(e, MDSX_EINVAL, "updateLocations(-1): length != N*P");
    } else {
        if (index < 0 || index >= e->n) return fail(e, MDSX_EINVAL, "updateLocations: index out of range");
        if (length != (size_t)e->p) return fail(e, MDSX_EINVAL, "updateLocations(i): length != P");
    }
    // The caller may reuse its buffer as soon as we return. Small problems stage
    // it in pinned memory and wait only for the previous copy out of the staging
    // (normally long done); larger ones copy from the caller's buffer and wait
    // for that copy. Either way the conversion runs on, ahead of the caller's
    // next call.
    const double* src = x;
    if (e->h_xstage) {
        MDSX_CUDA(e, cudaEventSynchronize(e->h2d_done));
        std::memcpy(e->h_xstage, x, length * sizeof(double));
        src = e->h_xstage;
    }
    MDSX_CUDA(e, cudaMemcpyAsync(e->d_xin, src, length * sizeof(double), cudaMemcpyHostToDevice, e->stream));
    MDSX_CUDA(e, cudaEventRecord(e->h2d_done, e->stream));
    if (index == -1)
        MDSX_CUDA(e, locations_to_soa(e, e->d_xin));
    else
        MDSX_CUDA(e, e->dd ? mdsx::set_one_location_dd(e->d_xin, index, e->p, e->d_x[e->xcur], e->x_ld, e->stream)
                           : mdsx::set_one_location(e->d_xin, index, e->p, e->d_x[e->xcur], e->x_ld, e->x_f32,
                                                    e->stream));
    if (!e->h_xstage) MDSX_CUDA(e, cudaEventSynchronize(e->h2d_done));
    e->sum_known = false;
    e->grad_known = false;
    return MDSX_OK;
}

int mdsx_get_sum_of_increments(mdsx_engine* e, double* out) {
    if (!e) return MDSX_EINVAL;
    if (!out) return fail(e, MDSX_EINVAL, "out is NULL");
    DeviceGuard guard(e->device);
    if (!e->sum_known) {
        int rc = sweep_and_read(e);
        if (rc) return rc;
    }
    *out = sum_of_increments(e);
    return MDSX_OK;
}

int mdsx_get_log_likelihood_gradient(mdsx_engine* e, double* out, size_t length) {
    if (!e) return MDSX_EINVAL;
    if (!out) return fail(e, MDSX_EINVAL, "out is NULL");
    if (length != (size_t)e->rows * e->p)
        return fail(e, MDSX_EINVAL, "getLogLikelihoodGradient: length != N*P (rows*P for a row range)");
    DeviceGuard guard(e->device);
    if (!e->grad_known) {
        int rc = sweep_and_read(e);
        if (rc) return rc;
    }
    if (e->h_grad_valid) {
        std::memcpy(out, e->h_grad, length * sizeof(double));
        return MDSX_OK;
    }
    MDSX_CUDA(e, cudaMemcpyAsync(out, e->d_grad[e->gcur], length * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
    MDSX_CUDA(e, cudaStreamSynchronize(e->stream));
    return MDSX_OK;
}

int mdsx_store_state(mdsx_engine* e) {
    if (!e) return MDSX_EINVAL;
    DeviceGuard guard(e->device);
    const int other = 1 - e->xcur;
    const size_t x_bytes = (size_t)e->p * e->x_ld * e->shape.x_elem_bytes;
    MDSX_CUDA(e, cudaMemcpyAsync(e->d_x[other], e->d_x[e->xcur], x_bytes, cudaMemcpyDeviceToDevice, e->stream));
    e->stored_grad_known = e->grad_known;
    e->h_grad_valid = false;
    if (e->grad_known)
        MDSX_CUDA(e, cudaMemcpyAsync(e->d_grad[1 - e->gcur], e->d_grad[e->gcur],
                                     (size_t)e->rows * e->p * sizeof(double), cudaMemcpyDeviceToDevice, e->stream));
    e->stored_sum_r2 = e->sum_r2;
    e->stored_sum_log = e->sum_log;
    e->stored_tau = e->tau;
    return MDSX_OK;
}

int mdsx_restore_state(mdsx_engine* e) {
    if (!e) return MDSX_EINVAL;
    // As the reference: the stored sum comes back and counts as known.
    e->sum_r2 = e->stored_sum_r2;
    e->sum_log = e->stored_sum_log;
    e->sum_known = true;
    e->tau = e->stored_tau;
    e->xcur = 1 - e->xcur;
    e->gcur = 1 - e->gcur;
    e->grad_known = e->stored_grad_known;
    e->h_grad_valid = false;
    return MDSX_OK;
}

int mdsx_accept_state(mdsx_engine* e) { return e ? MDSX_OK : MDSX_EINVAL; }

int mdsx_set_pairwise_data(mdsx_engine* e, const double* data, size_t length) {
    if (!e) return MDSX_EINVAL;
    if (!data) return fail(e, MDSX_EINVAL, "data pointer is NULL");
    if (length != (size_t)e->rows * e->n)
        return fail(e, MDSX_EINVAL, "setPairwiseData: length != N*N (rows*N for a row range)");
    DeviceGuard guard(e->device);
    if (!e->delta_f32 && !e->dd && e->ld == e->n) {
        MDSX_CUDA(e, cudaMemcpyAsync(e->d_delta, data, length * sizeof(double), cudaMemcpyHostToDevice, e->stream));
    } else {
        // Stage rows of doubles on the device and convert/pad them in place.
        const long long chunk_elems = 16LL << 20;  // 128 MB of doubles
        const long long rows_per_chunk = std::max(1LL, chunk_elems / e->n);
        double* staging = nullptr;
        MDSX_CUDA(e, mdsx::device_malloc(&staging, (size_t)std::min<long long>(rows_per_chunk, e->rows) * e->n * sizeof(double)));
        const int elem = e->delta_f32 ? 4 : 8;
        for (long long r0 = 0; r0 < e->rows; r0 += rows_per_chunk) {
            const long long rows = std::min<long long>(rows_per_chunk, e->rows - r0);
            cudaError_t err = cudaMemcpyAsync(staging, data + r0 * e->n, (size_t)(rows * e->n) * sizeof(double),
                                              cudaMemcpyHostToDevice, e->stream);
            void* dst = static_cast<char*>(e->d_delta) + (size_t)(r0 * e->ld) * elem;
            if (err == cudaSuccess)
                err = e->dd && !e->delta_f32
                          ? mdsx::convert_delta_rows_dd(staging, rows, e->n, dst, e->ld, e->stream)
                          : mdsx::convert_delta_rows(staging, rows, e->n, dst, e->ld, e->delta_f32, e->stream);
            if (err == cudaSuccess) err = cudaStreamSynchronize(e->stream);
            if (err != cudaSuccess) {
                cudaFree(staging);
                return cuda_fail(e, err, "setPairwiseData staging");
            }
        }
        cudaFree(staging);
    }
    MDSX_CUDA(e, mdsx::mark_nan_rows_block(e->d_delta, e->delta_f32, e->rows, e->n, e->ld, e->d_row_nan,
                                           e->rows_padded, e->stream));
    MDSX_CUDA(e, write_flags(e));
    MDSX_CUDA(e, cudaStreamSynchronize(e->stream));
    e->data_set = true;
    e->sum_known = e->grad_known = false;
    return MDSX_OK;
}

int mdsx_set_pairwise_data_f32(mdsx_engine* e, const float* data, size_t length) {
    if (!e) return MDSX_EINVAL;
    if (!data) return fail(e, MDSX_EINVAL, "data pointer is NULL");
    if (length != (size_t)e->rows * e->n)
        return fail(e, MDSX_EINVAL, "setPairwiseData: length != N*N (rows*N for a row range)");
    DeviceGuard guard(e->device);
    if (e->delta_f32) {
        MDSX_CUDA(e, cudaMemcpy2DAsync(e->d_delta, (size_t)e->ld * sizeof(float), data, (size_t)e->n * sizeof(float),
                                       (size_t)e->n * sizeof(float), (size_t)e->rows, cudaMemcpyHostToDevice,
                                       e->stream));
        MDSX_CUDA(e, mdsx::mark_nan_rows_block(e->d_delta, true, e->rows, e->n, e->ld, e->d_row_nan, e->rows_padded,
                                               e->stream));
        MDSX_CUDA(e, write_flags(e));
        MDSX_CUDA(e, cudaStreamSynchronize(e->stream));
        e->data_set = true;
        e->sum_known = e->grad_known = false;
        return MDSX_OK;
    }
    // FP64 storage: widen on the host.
    std::vector<double> wide(length);
    for (size_t k = 0; k < length; ++k) wide[k] = (double)data[k];
    return mdsx_set_pairwise_data(e, wide.data(), length);
}

int mdsx_set_parameters(mdsx_engine* e, const double* data, size_t length) {
    if (!e) return MDSX_EINVAL;
    if (!data) return fail(e, MDSX_EINVAL, "data pointer is NULL");
    if (length != 1) return fail(e, MDSX_EINVAL, "setParameters: length != 1 (precision only)");
    if (!(data[0] > 0.0) || !std::isfinite(data[0]))
        return fail(e, MDSX_EINVAL, "setParameters: precision must be finite and > 0");
    if (data[0] == e->tau) return MDSX_OK;
    e->tau = data[0];
    // The gradient scales with tau; with truncation the sum depends on it too.
    // (Without truncation the cached sum is kept unscaled, as the reference does.)
    e->grad_known = false;
    if (e->trunc) e->sum_known = false;
    return MDSX_OK;
}

int mdsx_make_dirty(mdsx_engine* e) {
    if (!e) return MDSX_EINVAL;
    e->sum_known = false;
    e->grad_known = false;
    return MDSX_OK;
}

int mdsx_get_internal_dimension(mdsx_engine* e, int* out) {
    if (!e || !out) return MDSX_EINVAL;
    *out = e->p;
    return MDSX_OK;
}

int mdsx_get_log_likelihood(mdsx_engine* e, double* out) {
    if (!e) return MDSX_EINVAL;
    if (!out) return fail(e, MDSX_EINVAL, "out is NULL");
    double s = 0.0;
    int rc = mdsx_get_sum_of_increments(e, &s);
    if (rc) return rc;
    // R/mds.R:24-28; a row range carries its rows' share of the N(N-1)/2 observations.
    const double observation_count = (double)e->rows * (double)(e->n - 1) / 2.0;
    *out = 0.5 * (std::log(e->tau) - std::log(2.0 * M_PI)) * observation_count - s;
    return MDSX_OK;
}

int mdsx_set_stream(mdsx_engine* e, void* stream) {
    if (!e) return MDSX_EINVAL;
    DeviceGuard guard(e->device);
    MDSX_CUDA(e, cudaStreamSynchronize(e->stream));
    e->stream = stream ? static_cast<cudaStream_t>(stream) : e->own_stream;
    return MDSX_OK;
}

int mdsx_update_locations_device(mdsx_engine* e, const double* d_x, size_t length) {
    if (!e) return MDSX_EINVAL;
    if (!d_x) return fail(e, MDSX_EINVAL, "locations pointer is NULL");
    if (length != (size_t)e->n * e->p) return fail(e, MDSX_EINVAL, "length != N*P");
    DeviceGuard guard(e->device);
    MDSX_CUDA(e, locations_to_soa(e, d_x));
    e->sum_known = false;
    e->grad_known = false;
    return MDSX_OK;
}

int mdsx_evaluate_device(mdsx_engine* e, double* d_sum, double* d_gradient) {
    if (!e) return MDSX_EINVAL;
    DeviceGuard guard(e->device);
    int rc = enqueue_sweep(e);
    if (rc) return rc;
    const int launches = e->last_launches;
    if (d_sum)
        MDSX_CUDA(e, cudaMemcpyAsync(d_sum, e->d_out + 2, sizeof(double), cudaMemcpyDeviceToDevice, e->stream));
    if (d_gradient)
        MDSX_CUDA(e, cudaMemcpyAsync(d_gradient, e->d_grad[e->gcur], (size_t)e->rows * e->p * sizeof(double),
                                     cudaMemcpyDeviceToDevice, e->stream));
    e->last_launches = launches;
    // Results live on the device; the host-side cache is refreshed lazily.
    e->sum_known = false;
    e->grad_known = true;
    return MDSX_OK;
}

int mdsx_set_sweep_schedule(mdsx_engine* e, int schedule) {
    if (!e) return MDSX_EINVAL;
    if (schedule != MDSX_SWEEP_ROWS && schedule != MDSX_SWEEP_PAIRS)
        return fail(e, MDSX_EINVAL, "unknown sweep schedule");
    if (schedule == MDSX_SWEEP_PAIRS && e->rows != e->n)
        return fail(e, MDSX_EUNSUPPORTED, "the unordered-pair schedule needs an engine over the whole matrix");
    if (schedule == MDSX_SWEEP_PAIRS && !e->d_rowpart)
        return fail(e, MDSX_EUNSUPPORTED, "the unordered-pair schedule is built for P <= 6 only");
    if (schedule == MDSX_SWEEP_ROWS && e->dd)
        return fail(e, MDSX_EUNSUPPORTED, "double-float pair math runs on the unordered-pair schedule only");
    if (schedule != e->schedule) {
        e->schedule = schedule;
        e->sum_known = e->grad_known = false;
    }
    return MDSX_OK;
}

int mdsx_get_sweep_schedule(mdsx_engine* e, int* out) {
    if (!e || !out) return MDSX_EINVAL;
    *out = e->schedule;
    return MDSX_OK;
}

int mdsx_last_launch_count(mdsx_engine* e, int* out) {
    if (!e || !out) return MDSX_EINVAL;
    *out = e->last_launches;
    return MDSX_OK;
}

}  // extern "C"

// Dispatch of the three precision modes.
namespace mdsx {
void set_global_error(const std::string& msg) { g_create_error = msg; }

bool sweep_shape(Mode mode, int p, KernelShape* out) {
    switch (mode) {
        case Mode::kF32: return sweep_shape_f32(p, out);
        case Mode::kF64: return sweep_shape_f64(p, out);
        case Mode::kF64DeltaF32: return sweep_shape_f64s32(p, out);
    }
    return false;
}
cudaError_t sweep_occupancy(Mode mode, int p, bool trunc, int* ctas) {
    switch (mode) {
        case Mode::kF32: return sweep_occupancy_f32(p, trunc, ctas);
        case Mode::kF64: return sweep_occupancy_f64(p, trunc, ctas);
        case Mode::kF64DeltaF32: return sweep_occupancy_f64s32(p, trunc, ctas);
    }
    return cudaErrorInvalidValue;
}
cudaError_t sweep_launch(Mode mode, int p, bool trunc, int grid, const CUtensorMap& td, const CUtensorMap& tx,
                         const SweepArgs& args, cudaStream_t stream) {
    switch (mode) {
        case Mode::kF32: return sweep_launch_f32(p, trunc, grid, td, tx, args, stream);
        case Mode::kF64: return sweep_launch_f64(p, trunc, grid, td, tx, args, stream);
        case Mode::kF64DeltaF32: return sweep_launch_f64s32(p, trunc, grid, td, tx, args, stream);
    }
    return cudaErrorInvalidValue;
}
}  // namespace mdsx
