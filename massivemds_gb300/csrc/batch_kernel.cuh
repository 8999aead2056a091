// Batched fused sweep: many independent MDS instances of one embedding
// dimension P in one persistent launch (no counterpart in the reference, which
// keeps one engine per instance, src/jni/dr_inference_multidimensionalscaling_
// NativeMDSSingleton.cpp:10-20).
//
// The work list is the concatenation of every instance's units (row block x
// 128-column stage, the single-instance kernel's unit), instance k owning the
// global units [unit_begin_k, unit_begin_k + R_k S_k). CTAs take contiguous
// stream-K ranges of the global list, so instances of uneven N share the
// machine without per-instance launches or tails. Per-instance state (tensor
// maps, precision constants, scratch, outputs) lives in a device array of
// BatchInstance descriptors; a CTA walks its range with an instance cursor.
// Pair arithmetic, the FP32 compensated accumulation and the deterministic
// last-arriver publication are those of sweep_kernel.cuh, with per-instance
// counters; the rows per warp (RW) are a template parameter chosen by the
// autotuner (batch.cu).
#pragma once

#include <cuda.h>

#include <climits>

#include "sweep_kernel.cuh"

namespace mdsx {
namespace batch {

struct BatchInstance {  // CUtensorMap members keep it 64-byte aligned (TMA requirement)
    CUtensorMap tmap_delta;  // delta [N][ld] FP32, box 128 x RB
    CUtensorMap tmap_x;      // SoA locations [P][x_ld] FP32, box 128 x P
    long long unit_begin;    // first global unit
    int n, n_row_blocks, steps_per_row, max_slots;
    int x_ld, truncation;
    const float* x;          // SoA locations
    const int* row_nan;      // [rows_padded]
    float k_e, log2_k2, tp0, tp1, tp2, ts0, ts1, ts2;
    double tau;
    float* gpart;            // [R][max_slots][RB][P]
    double* lpart;           // [R][max_slots][warps][2]
    double* lrow;            // [R][2]
    unsigned* rb_count;      // [R]
    unsigned* done_count;    // [1]
    double* grad_out;        // [N][P]
    double* sums_out;        // [4]: sum r^2, sum log Phi, getSumOfIncrements(), error word
};

struct BatchArgs {
    const BatchInstance* inst;
    int count;
    long long n_units;
    int grid;
    int* err;
};

template <int P, int RW>
struct BatchShape {
    static constexpr int RB = RW * kConsumerWarps;
    static constexpr int kDeltaBytes = RB * kStepCols * 4;
    static constexpr int kXBytes = P * kStepCols * 4;
    static constexpr int kStageBytes = kDeltaBytes + kXBytes;
    static constexpr int kSmemBytes = kStages * kStageBytes + 2 * kStages * 8 + 128;
};

// Instance holding global unit u, searching forward from k.
__device__ __forceinline__ int advance_instance(const BatchInstance* inst, int count, int k, long long u) {
    while (k + 1 < count && __ldg(&inst[k + 1].unit_begin) <= u) ++k;
    return k;
}

// First instance whose range can hold u (binary search on unit_begin).
__device__ __forceinline__ int find_instance(const BatchInstance* inst, int count, long long u) {
    int lo = 0, hi = count - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(&inst[mid].unit_begin) <= u)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

template <int P, bool TRUNC, int RW>
__global__ void __launch_bounds__(kThreads, MDSX_F32_MIN_CTAS) batch_sweep_kernel(const BatchArgs a) {
    using Shape = BatchShape<P, RW>;
    constexpr int RB = Shape::RB;

    extern __shared__ unsigned char smem_raw[];
    unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) &
                                                           ~uintptr_t(127));
    float* sdelta = reinterpret_cast<float*>(smem);
    float* sx = reinterpret_cast<float*>(smem + kStages * Shape::kDeltaBytes);
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + kStages * Shape::kStageBytes);
    uint64_t* empty = full + kStages;

    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const long long u_begin = cta_unit_begin(blockIdx.x, a.n_units, a.grid);
    const long long u_end = cta_unit_begin(blockIdx.x + 1, a.n_units, a.grid);

    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], kConsumerWarps);
        }
        fence_mbar_init();
    }
    __syncthreads();

    if (warp == kConsumerWarps) {
        // ------------------------------------------------------ producer warp
        if (lane == 0) {
            int stage = 0;
            uint32_t phase = 0;
            long long issued = 0;
            // Instance fields live in registers and are reloaded only when the
            // range crosses into the next instance; (rb, st) advance by one
            // unit at a time, so a unit costs no memory access or division.
            int k = find_instance(a.inst, a.count, u_begin);
            const BatchInstance* in = a.inst + k;
            long long next_begin = k + 1 < a.count ? __ldg(&a.inst[k + 1].unit_begin) : LLONG_MAX;
            int S_ = in->steps_per_row;
            long long lu = u_begin - in->unit_begin;
            int rb = (int)(lu / S_);
            int st = (int)(lu - (long long)rb * S_);
            prefetch_tensormap(&in->tmap_delta);
            prefetch_tensormap(&in->tmap_x);
            for (long long u = u_begin; u < u_end; ++u) {
                if (u >= next_begin) {  // first unit of the next instance(s)
                    k = advance_instance(a.inst, a.count, k, u);
                    in = a.inst + k;
                    next_begin = k + 1 < a.count ? __ldg(&a.inst[k + 1].unit_begin) : LLONG_MAX;
                    S_ = in->steps_per_row;
                    rb = 0;
                    st = 0;
                    prefetch_tensormap(&in->tmap_delta);
                    prefetch_tensormap(&in->tmap_x);
                }
                if (!mbar_wait_bounded(&empty[stage], phase ^ 1u, a.err, kDevTimeoutEmpty)) break;
                mbar_arrive_expect_tx(&full[stage], Shape::kStageBytes);
                tma_load_2d(sdelta + stage * (RB * kStepCols), &in->tmap_delta, st * kStepCols, rb * RB, &full[stage]);
                tma_load_2d(sx + stage * (P * kStepCols), &in->tmap_x, st * kStepCols, 0, &full[stage]);
                ++issued;
                if (++stage == kStages) {
                    stage = 0;
                    phase ^= 1u;
                }
                if (++st == S_) {
                    st = 0;
                    ++rb;
                }
            }
            // Do not leave while copies issued by this thread may still be in flight.
            const int pending = issued < kStages ? (int)issued : kStages;
            for (int j = 0; j < pending; ++j) {
                if (--stage < 0) {
                    stage = kStages - 1;
                    phase ^= 1u;
                }
                mbar_wait_time_only(&full[stage], phase);
            }
        }
        return;
    }

    // -------------------------------------------------------- consumer warps
    int stage = 0;
    uint32_t phase = 0;
    int k = find_instance(a.inst, a.count, u_begin);
    long long next_begin = k + 1 < a.count ? __ldg(&a.inst[k + 1].unit_begin) : LLONG_MAX;
    for (long long u = u_begin; u < u_end;) {
        if (u >= next_begin) {
            k = advance_instance(a.inst, a.count, k, u);
            next_begin = k + 1 < a.count ? __ldg(&a.inst[k + 1].unit_begin) : LLONG_MAX;
        }
        const BatchInstance* in = a.inst + k;
        const int S_ = in->steps_per_row;
        const int n = in->n;
        const long long lu = u - in->unit_begin;
        const int rb = (int)(lu / S_);
        const int st0 = (int)(lu - (long long)rb * S_);
        const long long rb_first = in->unit_begin + (long long)rb * S_;  // global units of row block rb
        const long long rb_end = rb_first + S_;
        const long long seg_end = u_end < rb_end ? u_end : rb_end;
        const int steps = (int)(seg_end - u);
        const int first_cta = cta_of_unit(rb_first, a.n_units, a.grid);
        const int n_slots = cta_of_unit(rb_end - 1, a.n_units, a.grid) - first_cta + 1;
        const int slot = blockIdx.x - first_cta;
        u = seg_end;
        const int row0 = rb * RB + warp * RW;
        const PairConstsF32 kc{pk(-1.f, -1.f),           pk(in->k_e, in->k_e), pk(in->log2_k2, in->log2_k2),
                               pk(-in->tp0, -in->tp0),   pk(-in->tp1, -in->tp1), pk(-in->tp2, -in->tp2),
                               pk(in->ts0, in->ts0),     pk(in->ts1, in->ts1), pk(in->ts2, in->ts2)};

        f2 xi2[RW][P];
        bool rows_clean = true;
#pragma unroll
        for (int r = 0; r < RW; ++r) {
            const int i = row0 + r;
            rows_clean &= (in->row_nan[i] == 0);
#pragma unroll
            for (int q = 0; q < P; ++q) {
                const float v = in->x[(size_t)q * in->x_ld + i];
                xi2[r][q] = pk(v, v);
            }
        }
        f2 g2[RW][P], r2p = pk(0.f, 0.f), prodp = pk(1.f, 1.f);
#pragma unroll
        for (int r = 0; r < RW; ++r)
#pragma unroll
            for (int q = 0; q < P; ++q) g2[r][q] = pk(0.f, 0.f);
        float r2_hi = 0.f, r2_lo = 0.f, log2_sum = 0.f;

        bool alive = true;
        for (int s = 0; s < steps; ++s) {
            if (!mbar_wait_bounded(&full[stage], phase, a.err, kDevTimeoutFull)) {
                alive = false;
                break;
            }
            const int j0 = (st0 + s) * kStepCols;
            const bool masked = !rows_clean || (j0 + kStepCols > n) || (j0 < row0 + RW && row0 < j0 + kStepCols);
            const float* dtile = sdelta + stage * (RB * kStepCols) + (warp * RW) * kStepCols + 4 * lane;
            const float* xtile = sx + stage * (P * kStepCols) + 4 * lane;
            if (masked)
                stage_f32<P, TRUNC, true, RW>(dtile, xtile, xi2, row0, j0, n, n, lane, kc, g2, r2p, prodp);
            else
                stage_f32<P, TRUNC, false, RW>(dtile, xtile, xi2, row0, j0, n, n, lane, kc, g2, r2p, prodp);
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[stage]);
            if (++stage == kStages) {
                stage = 0;
                phase ^= 1u;
            }
            if ((s + 1) % (kLogFoldPairs / (2 * RW)) == 0 || s + 1 == steps) {
                if (TRUNC) {
                    float lo, hi;
                    upk(prodp, lo, hi);
                    log2_sum += lg2_approx(lo) + lg2_approx(hi);
                    prodp = pk(1.f, 1.f);
                }
                const float step_sum = sum2(r2p);
                r2p = pk(0.f, 0.f);
                float hi, e;
                two_sum(r2_hi, step_sum, hi, e);
                r2_hi = hi;
                r2_lo += e;
            }
        }
        if (!alive) return;

        // ---- publish this warp's partials into the CTA's slot of row block rb
        const size_t slot_base = (size_t)rb * in->max_slots + slot;
        {
            constexpr int K = RW * P;
            using TS = TransposeShape<K>;
            float gv[K];
#pragma unroll
            for (int r = 0; r < RW; ++r)
#pragma unroll
                for (int q = 0; q < P; ++q) gv[r * P + q] = sum2(g2[r][q]);
            warp_transpose_reduce<K>(gv, lane);
            const int idx = lane >> TS::kLaneShift;
            if ((lane & ((1 << TS::kLaneShift) - 1)) == 0 && idx < K)
                in->gpart[(slot_base * RB + warp * RW) * P + idx] = gv[0];
        }
        {
            float lv[3] = {r2_hi, r2_lo, log2_sum};
            warp_transpose_reduce<3>(lv, lane);
            const float t_hi = __shfl_sync(0xffffffffu, lv[0], 0);
            const float t_lo = __shfl_sync(0xffffffffu, lv[0], 8);
            const float t_lg = __shfl_sync(0xffffffffu, lv[0], 16);
            if (lane == 0) {
                in->lpart[(slot_base * kConsumerWarps + warp) * 2 + 0] = (double)t_hi + (double)t_lo;
                in->lpart[(slot_base * kConsumerWarps + warp) * 2 + 1] = -0.69314718055994530942 * (double)t_lg;
            }
        }
        __syncwarp();
        unsigned prev = 0;
        if (lane == 0) {
            fence_acq_rel_gpu();
            prev = atomicAdd(&in->rb_count[rb], 1u);
        }
        prev = __shfl_sync(0xffffffffu, prev, 0);
        if (prev != (unsigned)(kConsumerWarps * n_slots - 1)) continue;

        // ---- this warp completed row block rb of instance k
        __threadfence();
        for (int idx = lane; idx < RB * P; idx += 32) {
            const int rr = idx / P;
            const int q = idx - rr * P;
            double sum = 0.0;
            for (int j = 0; j < n_slots; ++j)
                sum += (double)__ldcg(&in->gpart[(((size_t)rb * in->max_slots + j) * RB + rr) * P + q]);
            const int row = rb * RB + rr;
            if (row < n) in->grad_out[(size_t)row * P + q] = -in->tau * sum;
        }
        double br2 = 0.0, blog = 0.0;
        for (int idx = lane; idx < n_slots * kConsumerWarps; idx += 32) {
            const size_t base = ((size_t)rb * in->max_slots * kConsumerWarps + idx) * 2;
            br2 += __ldcg(&in->lpart[base]);
            blog += __ldcg(&in->lpart[base + 1]);
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            br2 += __shfl_xor_sync(0xffffffffu, br2, off);
            blog += __shfl_xor_sync(0xffffffffu, blog, off);
        }
        if (lane == 0) {
            in->lrow[2 * rb] = br2;
            in->lrow[2 * rb + 1] = blog;
            in->rb_count[rb] = 0u;
        }
        __syncwarp();
        if (lane == 0) {
            fence_acq_rel_gpu();
            prev = atomicAdd(in->done_count, 1u);
        }
        prev = __shfl_sync(0xffffffffu, prev, 0);
        if (prev != (unsigned)(in->n_row_blocks - 1)) continue;

        // ---- last row block of instance k: its likelihood sums in a fixed order
        __threadfence();
        double tr2 = 0.0, tlog = 0.0;
        for (int j = lane; j < in->n_row_blocks; j += 32) {
            tr2 += __ldcg(&in->lrow[2 * j]);
            tlog += __ldcg(&in->lrow[2 * j + 1]);
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            tr2 += __shfl_xor_sync(0xffffffffu, tr2, off);
            tlog += __shfl_xor_sync(0xffffffffu, tlog, off);
        }
        if (lane == 0) {
            in->sums_out[0] = tr2;
            in->sums_out[1] = tlog;
            // src/NewMultiDimensionalScaling.hpp:198-202 and :554-557
            in->sums_out[2] =
                in->truncation ? 0.5 * (0.5 * in->tau * tr2 + tlog) : 0.5 * in->tau * (0.5 * tr2);
            *in->done_count = 0u;
        }
    }
}

}  // namespace batch
}  // namespace mdsx
