// Batched fused sweep, row-block queue schedule (the batched engine's second
// schedule; batch_kernel.cuh holds the stream-K one).
//
// Work item = one row block (RB rows x all N columns) of one instance. CTAs
// take items from a global counter (items ordered largest instance first), so
// a CTA owns every column of its row block: each consumer warp finishes its RW
// rows and writes their gradient directly, with no cross-CTA partials. The
// producer lane streams the row block's 128-column stages through the TMA
// ring with per-stage metadata {instance, row block, stage} in shared memory;
// the first stage of a row block also brings the block's own locations and
// their missing-row flags (row P of the SoA location array) with the same
// transaction. An end marker (a stage arrival without data) stops the
// consumers. Likelihood: one (sum r^2, sum log Phi) pair per warp and row block;
// the CTA's warps count a finished row block in shared memory and the last of
// them counts it once in the instance's global counter; the warp that completes
// an instance sums its partials in a fixed order. Results do not depend on
// which CTA took which item: bitwise deterministic.
#pragma once

#include <cuda.h>

#include <climits>

#include "sweep_kernel.cuh"

namespace mdsx {
namespace batch {

struct QueueInstance {     // device descriptor; CUtensorMap members keep it 64-byte aligned
    CUtensorMap tmap_delta;  // delta [N][ld] FP32, box 128 x RB
    CUtensorMap tmap_x;      // SoA [P + 1][x_ld] FP32 (row P: 1 for rows with a NaN), box 128 x (P + 1)
    int n, n_row_blocks, steps_per_row, truncation;
    long long item_begin;    // first queue item (row block 0) of this instance
    float k_e, log2_k2, tp0, tp1, tp2, ts0, ts1, ts2;
    double tau;
    double* lpart;           // [n_row_blocks][warps][2]
    unsigned* done_count;    // [1] row blocks finished
    double* grad_out;        // [N][P]
    double* sums_out;        // [4]
};

struct QueueArgs {
    const QueueInstance* inst;
    int count;
    long long n_items;
    unsigned long long* next;  // queue counter, zero at launch
    int* err;
};

template <int P, int RW>
struct QueueShape {
    static constexpr int RB = RW * kConsumerWarps;
    static constexpr int kDeltaBytes = RB * kStepCols * 4;
    static constexpr int kXBytes = (P + 1) * kStepCols * 4;     // x_j tile (with the flag row)
    static constexpr int kRowsBytes = (P + 1) * kStepCols * 4;  // the row block's own locations
    static constexpr int kSlotBytes = kDeltaBytes + kXBytes + kRowsBytes;
    static constexpr int kSmemBytes = kStages * (kSlotBytes + 16) + 2 * kStages * 8 + 8 * 4 + 128;
};

__device__ __forceinline__ int queue_find_instance(const QueueInstance* inst, int count, long long item) {
    int lo = 0, hi = count - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(&inst[mid].item_begin) <= item)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

template <int P, bool TRUNC, int RW>
__global__ void __launch_bounds__(kThreads, MDSX_F32_MIN_CTAS) batch_queue_kernel(const QueueArgs a) {
    using Shape = QueueShape<P, RW>;
    constexpr int RB = Shape::RB;
    extern __shared__ unsigned char smem_raw[];
    unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) &
                                                           ~uintptr_t(127));
    // slot s: [delta RB x 128][x (P+1) x 128][rows (P+1) x 128]; then metadata, barriers, counters
    int4* meta = reinterpret_cast<int4*>(smem + kStages * Shape::kSlotBytes);
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + kStages * (Shape::kSlotBytes + 16));
    uint64_t* empty = full + kStages;
    // Warps of this CTA that finished the CTA's j-th row block, in slot j % 8: a
    // warp can run at most kStages (< 8) row blocks ahead of the slowest one.
    unsigned* rb_warps = reinterpret_cast<unsigned*>(empty + kStages);
    auto slot_delta = [&](int s) { return reinterpret_cast<float*>(smem + s * Shape::kSlotBytes); };
    auto slot_x = [&](int s) { return reinterpret_cast<float*>(smem + s * Shape::kSlotBytes + Shape::kDeltaBytes); };
    auto slot_rows = [&](int s) {
        return reinterpret_cast<float*>(smem + s * Shape::kSlotBytes + Shape::kDeltaBytes + Shape::kXBytes);
    };

    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], kConsumerWarps);
        }
        for (int j = 0; j < 8; ++j) rb_warps[j] = 0u;
        fence_mbar_init();
    }
    __syncthreads();

    if (warp == kConsumerWarps) {
        // ------------------------------------------------------ producer warp
        if (lane == 0) {
            int stage = 0;
            uint32_t phase = 0;
            long long issued = 0;
            bool ok = true;
            while (ok) {
                const long long item = (long long)atomicAdd(a.next, 1ull);
                if (item >= a.n_items) break;
                const int k = queue_find_instance(a.inst, a.count, item);
                const QueueInstance* in = a.inst + k;
                const int rb = (int)(item - in->item_begin);
                const int S_ = in->steps_per_row;
                prefetch_tensormap(&in->tmap_delta);
                prefetch_tensormap(&in->tmap_x);
                for (int st = 0; st < S_; ++st) {
                    if (!mbar_wait_bounded(&empty[stage], phase ^ 1u, a.err, kDevTimeoutEmpty)) {
                        ok = false;
                        break;
                    }
                    meta[stage] = make_int4(k, rb, st, 0);
                    const uint32_t bytes = Shape::kDeltaBytes + Shape::kXBytes + (st == 0 ? Shape::kRowsBytes : 0);
                    mbar_arrive_expect_tx(&full[stage], bytes);
                    tma_load_2d(slot_delta(stage), &in->tmap_delta, st * kStepCols, rb * RB, &full[stage]);
                    tma_load_2d(slot_x(stage), &in->tmap_x, st * kStepCols, 0, &full[stage]);
                    if (st == 0) tma_load_2d(slot_rows(stage), &in->tmap_x, rb * RB, 0, &full[stage]);
                    ++issued;
                    if (++stage == kStages) {
                        stage = 0;
                        phase ^= 1u;
                    }
                }
            }
            // end marker: a stage that completes without data
            bool ended = false;
            if (ok && mbar_wait_bounded(&empty[stage], phase ^ 1u, a.err, kDevTimeoutEmpty)) {
                meta[stage] = make_int4(-1, 0, 0, 0);
                mbar_arrive(&full[stage]);
                ended = true;
            }
            // Let this thread's copies land before the CTA can exit: the last
            // stages issued, walking back from the end-marker slot. That slot's
            // earlier data stage was released by every consumer before the
            // marker went in (and its barrier has moved on), so it is skipped.
            int s = stage;
            uint32_t ph = phase;
            const int window = ended ? kStages - 1 : kStages;
            const int pending = issued < window ? (int)issued : window;
            for (int j = 0; j < pending; ++j) {
                if (--s < 0) {
                    s = kStages - 1;
                    ph ^= 1u;
                }
                mbar_wait_time_only(&full[s], ph);
            }
        }
        return;
    }

    // -------------------------------------------------------- consumer warps
    int stage = 0;
    uint32_t phase = 0;
    f2 xi2[RW][P], g2[RW][P], r2p = pk(0.f, 0.f), prodp = pk(1.f, 1.f);
    float r2_hi = 0.f, r2_lo = 0.f, log2_sum = 0.f;
    bool rows_clean = true;
    int row0 = 0, fold = 0, n = 0, steps_per_row = 0;
    unsigned rb_seq = 0;  // row blocks of this CTA finished by this warp
    PairConstsF32 kc{};
    for (;;) {
        if (!mbar_wait_bounded(&full[stage], phase, a.err, kDevTimeoutFull)) return;
        const int4 m = meta[stage];
        if (m.x < 0) return;  // end marker
        const int k = m.x, rb = m.y, st = m.z;
        const QueueInstance* in = a.inst + k;
        if (st == 0) {
            // a new row block: this warp's rows, their flags and the instance constants
            n = in->n;
            steps_per_row = in->steps_per_row;
            row0 = rb * RB + warp * RW;
            const float* rows = slot_rows(stage);
            rows_clean = row0 + RW <= n;
#pragma unroll
            for (int r = 0; r < RW; ++r) {
                const int c = warp * RW + r;  // column within the 128-wide rows tile
                rows_clean &= rows[P * kStepCols + c] == 0.0f;
#pragma unroll
                for (int q = 0; q < P; ++q) {
                    const float v = rows[q * kStepCols + c];
                    xi2[r][q] = pk(v, v);
                    g2[r][q] = pk(0.f, 0.f);
                }
            }
            kc = PairConstsF32{pk(-1.f, -1.f),         pk(in->k_e, in->k_e), pk(in->log2_k2, in->log2_k2),
                               pk(-in->tp0, -in->tp0), pk(-in->tp1, -in->tp1), pk(-in->tp2, -in->tp2),
                               pk(in->ts0, in->ts0),   pk(in->ts1, in->ts1), pk(in->ts2, in->ts2)};
            r2p = pk(0.f, 0.f);
            prodp = pk(1.f, 1.f);
            r2_hi = r2_lo = log2_sum = 0.f;
            fold = 0;
        }
        const int j0 = st * kStepCols;
        const bool masked = !rows_clean || (j0 + kStepCols > n) || (j0 < row0 + RW && row0 < j0 + kStepCols);
        const float* dtile = slot_delta(stage) + (warp * RW) * kStepCols + 4 * lane;
        const float* xtile = slot_x(stage) + 4 * lane;
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
        const bool last = st + 1 == steps_per_row;
        if (++fold == kLogFoldPairs / (2 * RW) || last) {
            fold = 0;
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
        if (!last) continue;

        // ---- row block rb of instance k done: gradient rows, likelihood partial
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
            if ((lane & ((1 << TS::kLaneShift) - 1)) == 0 && idx < K) {
                const int row = row0 + idx / P;
                if (row < n) in->grad_out[(size_t)row * P + idx % P] = -in->tau * (double)gv[0];
            }
        }
        {
            float lv[3] = {r2_hi, r2_lo, log2_sum};
            warp_transpose_reduce<3>(lv, lane);
            const float t_hi = __shfl_sync(0xffffffffu, lv[0], 0);
            const float t_lo = __shfl_sync(0xffffffffu, lv[0], 8);
            const float t_lg = __shfl_sync(0xffffffffu, lv[0], 16);
            if (lane == 0) {
                in->lpart[((size_t)rb * kConsumerWarps + warp) * 2 + 0] = (double)t_hi + (double)t_lo;
                in->lpart[((size_t)rb * kConsumerWarps + warp) * 2 + 1] = -0.69314718055994530942 * (double)t_lg;
            }
        }
        // The last of the CTA's 8 warps to finish this row block counts it once
        // in the instance's global counter (one contended atomic per row block).
        __syncwarp();
        unsigned done = 0;
        if (lane == 0) {
            fence_acq_rel_gpu();
            unsigned* slot = &rb_warps[rb_seq & 7u];
            if (atomicAdd(slot, 1u) == kConsumerWarps - 1) {
                atomicExch(slot, 0u);
                done = atomicAdd(in->done_count, 1u) + 1u;  // row blocks done, this one included
            }
        }
        ++rb_seq;
        done = __shfl_sync(0xffffffffu, done, 0);
        if (done != (unsigned)in->n_row_blocks) continue;

        // ---- last row block of instance k: its likelihood sums in a fixed order
        __threadfence();
        double tr2 = 0.0, tlog = 0.0;
        for (int j = lane; j < in->n_row_blocks * kConsumerWarps; j += 32) {
            tr2 += __ldcg(&in->lpart[2 * (size_t)j]);
            tlog += __ldcg(&in->lpart[2 * (size_t)j + 1]);
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
            in->sums_out[2] = in->truncation ? 0.5 * (0.5 * in->tau * tr2 + tlog) : 0.5 * in->tau * (0.5 * tr2);
            *in->done_count = 0u;
        }
    }
}

}  // namespace batch
}  // namespace mdsx
