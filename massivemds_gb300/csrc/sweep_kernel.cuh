// The fused MDS likelihood + gradient sweep (the engine's hot path).
//
// One pass over the N x N dissimilarity matrix delta computes, for every ordered
// pair (i, j) that is not missing (i == j or delta_ij NaN, as in
// src/NewMultiDimensionalScaling.hpp:402-410 of MassiveMDS):
//   d_ij   = ||x_i - x_j||                           (src/Distance.hpp:78-88)
//   r_ij   = delta_ij - d_ij
//   lik:   r_ij^2 and, with truncation, logPhi(d_ij sqrt(tau))   (:508-514)
//   grad:  g_i += [r_ij - phi(z)/(Phi(z) sqrt(tau))] / d_ij * (x_i - x_j)   (:421-461)
// and reduces sum_ij r^2, sum_ij logPhi and tau * g_i.
//
// Work decomposition. delta rows are grouped in row blocks of RB = 8*RW rows;
// each row block's columns are cut into chunks of chunk_steps stages of 128
// columns. A tile is (row block, chunk). Persistent CTAs walk tiles
// blockIdx.x, blockIdx.x + gridDim.x, ... Each CTA has one producer warp that
// streams [RB x 128] delta boxes and [P x 128] location boxes into a kStages
// shared-memory ring with TMA (cp.async.bulk.tensor.2d), and 8 consumer warps;
// consumer warp w owns rows w*RW .. w*RW+RW-1 of the box, each lane 4
// consecutive columns (128-bit shared loads).
//
// Reductions are deterministic. Each warp writes its per-tile partials (gradient
// rows, and the pair of likelihood sums) to scratch; the warp that completes a
// row block (an atomic counter per row block; no thread ever waits on another
// CTA) sums that row block's partials in chunk order, and the warp that
// completes the last row block sums the row-block likelihood partials in a
// fixed order. Counters reset themselves for the next launch.
//
// FP32 mode: pair arithmetic in FP32 with MUFU rsqrt/ex2/rcp; Phi from the
// rational tail fit in normal_rational.h (one ex2 shared by Phi and phi, one rcp
// giving 1/Phi); logPhi summed as log2 of running products of 1/Phi (one lg2
// per 64 pairs); r^2 sums compensated with TwoSum; per-tile partials promoted to
// FP64 for every reduction above the warp. FP64 mode: pair arithmetic in FP64
// with CUDA's double sqrt/erfc/exp/log.
#pragma once

#include <cstdint>
#include <cuda.h>

#include "ptx.cuh"

namespace mdsx {

constexpr int kConsumerWarps = 8;
constexpr int kThreads = (kConsumerWarps + 1) * 32;  // + 1 producer warp
constexpr int kStepCols = 128;                       // columns per stage: 32 lanes x 4
constexpr int kStages = 4;
constexpr int kLogFoldPairs = 64;                    // product of <= 64 factors in [1, 2] cannot overflow

struct SweepArgs {
    int n;             // locations N
    int n_row_blocks;  // ceil(N / RB)
    int n_chunks;      // column chunks per row block
    int chunk_steps;   // stages per chunk
    int n_tiles;       // n_row_blocks * n_chunks
    int rows_padded;   // n_row_blocks * RB
    int x_ld;          // row stride of the SoA location array [P][x_ld]
    const void* x;     // SoA locations (compute type)
    const int* row_nan;  // [rows_padded]; nonzero: row has a NaN, or row >= N
    // FP32 pair constants (d-space): E' = 2^(d^2 k_e + log2_k2) = exp(-tau d^2/2)/sqrt(2 pi tau)
    float k_e, log2_k2;
    float tp0, tp1, tp2, ts0, ts1, ts2;  // 1/Phi = S(d) / (S(d) - E' P(d))
    double tau, sqrt_tau;
    // scratch
    void* gpart;         // [n_chunks][rows_padded][P] partial gradients (accumulator type)
    double* lpart;       // [n_tiles][kConsumerWarps][2] per-warp likelihood partials
    double* lrow;        // [n_row_blocks][2]
    unsigned* rb_count;  // [n_row_blocks] completions per row block
    unsigned* done_count;  // [1] completed row blocks
    // outputs
    double* grad_out;  // [N][P] = tau * sum_j ..., row-major
    double* sums_out;  // [0] = sum of r^2, [1] = sum of logPhi, over ordered non-missing pairs,
                       // [2] = getSumOfIncrements() of those sums
    int truncation;
    int* err;
};

template <typename C, int P>
struct RowsPerWarp {
    static constexpr int value = sizeof(C) == 4 ? (P <= 4 ? 4 : (P <= 6 ? 2 : 1)) : (P <= 3 ? 2 : 1);
};

template <typename C, typename S, int P>
struct SweepShape {
    static constexpr int RW = RowsPerWarp<C, P>::value;
    static constexpr int RB = RW * kConsumerWarps;
    static constexpr int kDeltaBytes = RB * kStepCols * (int)sizeof(S);
    static constexpr int kXBytes = P * kStepCols * (int)sizeof(C);
    static constexpr int kStageBytes = kDeltaBytes + kXBytes;
    static constexpr int kSmemBytes = kStages * kStageBytes + 2 * kStages * 8 + 128;  // + barriers + alignment slack
};

// ---------------------------------------------------------------- pair math

struct PairConstsF32 {
    float k_e, log2_k2, tp0, tp1, tp2, ts0, ts1, ts2;
};

// One ordered pair in FP32. Accumulates r^2 into r2, the factor 1/Phi into prod,
// and v * rs * (x_i - x_j) into g (tau applied at finalisation).
template <int P, bool TRUNC, bool MASKED>
__device__ __forceinline__ void pair_f32(const float (&xi)[P], const float (&xj)[P][4], int c, float delta,
                                         bool valid, const PairConstsF32& k, float (&g)[P], float& r2,
                                         float& prod) {
    float dx[P];
#pragma unroll
    for (int q = 0; q < P; ++q) dx[q] = xi[q] - xj[q][c];
    float d2 = dx[0] * dx[0];
#pragma unroll
    for (int q = 1; q < P; ++q) d2 = fmaf(dx[q], dx[q], d2);
    const float rs = rsqrt_approx(d2);
    const float d = d2 * rs;
    float res = delta - d;
    if (MASKED) res = valid ? res : 0.0f;
    r2 = fmaf(res, res, r2);
    float cc;
    if (TRUNC) {
        const float e = ex2_approx(fmaf(d2, k.k_e, k.log2_k2));
        const float pp = fmaf(fmaf(k.tp2, d, k.tp1), d, k.tp0);
        const float ss = fmaf(fmaf(d + k.ts2, d, k.ts1), d, k.ts0);
        const float aa = fmaf(-e, pp, ss);
        float iphi = ss * rcp_approx(aa);
        if (MASKED) iphi = valid ? iphi : 1.0f;
        prod *= iphi;
        cc = fmaf(-e, iphi, res) * rs;
    } else {
        cc = res * rs;
    }
    if (MASKED) cc = valid ? cc : 0.0f;
#pragma unroll
    for (int q = 0; q < P; ++q) g[q] = fmaf(cc, dx[q], g[q]);
}

// One ordered pair in FP64 (CUDA double sqrt/erfc/exp/log).
template <int P, bool TRUNC, bool MASKED>
__device__ __forceinline__ void pair_f64(const double (&xi)[P], const double (&xj)[P][4], int c, double delta,
                                         bool valid, double tau, double sqrt_tau, double (&g)[P], double& r2,
                                         double& lsum) {
    double dx[P];
#pragma unroll
    for (int q = 0; q < P; ++q) dx[q] = xi[q] - xj[q][c];
    double d2 = dx[0] * dx[0];
#pragma unroll
    for (int q = 1; q < P; ++q) d2 = fma(dx[q], dx[q], d2);
    if (MASKED && !valid) return;
    const double d = sqrt(d2);
    double res = delta - d;
    r2 = fma(res, res, r2);
    if (TRUNC) {
        const double z = d * sqrt_tau;
        const double cdf = 0.5 * erfc(-z * 0.70710678118654752440);
        lsum += log(cdf);
        const double pdf = 0.39894228040143267794 * exp(-0.5 * z * z);
        res -= pdf / (cdf * sqrt_tau);
    }
    const double cc = res / d;
#pragma unroll
    for (int q = 0; q < P; ++q) g[q] = fma(cc, dx[q], g[q]);
}

// --------------------------------------------------------------- the kernel

template <typename C, typename S, int P, bool TRUNC>
__global__ void __launch_bounds__(kThreads, sizeof(C) == 4 ? 2 : 1)
    sweep_kernel(const __grid_constant__ CUtensorMap tmap_delta, const __grid_constant__ CUtensorMap tmap_x,
                 const SweepArgs a) {
    using Shape = SweepShape<C, S, P>;
    constexpr int RW = Shape::RW;
    constexpr int RB = Shape::RB;
    constexpr bool F32 = sizeof(C) == 4;
    using Acc = C;  // accumulator type of gradient partials

    extern __shared__ unsigned char smem_raw[];
    unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) &
                                                           ~uintptr_t(127));
    S* sdelta = reinterpret_cast<S*>(smem);
    C* sx = reinterpret_cast<C*>(smem + kStages * Shape::kDeltaBytes);
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + kStages * Shape::kStageBytes);
    uint64_t* empty = full + kStages;

    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;

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
            prefetch_tensormap(&tmap_delta);
            prefetch_tensormap(&tmap_x);
            int stage = 0;
            uint32_t phase = 0;
            long issued = 0;
            bool ok = true;
            for (int t = blockIdx.x; ok && t < a.n_tiles; t += gridDim.x) {
                const int rb = t / a.n_chunks;
                const int cb = t - rb * a.n_chunks;
                const int col0 = cb * a.chunk_steps * kStepCols;
                const int steps = min(a.chunk_steps, (a.n - col0 + kStepCols - 1) / kStepCols);
                for (int s = 0; s < steps; ++s) {
                    if (!mbar_wait_bounded(&empty[stage], phase ^ 1u, a.err, kDevTimeoutEmpty)) {
                        ok = false;
                        break;
                    }
                    mbar_arrive_expect_tx(&full[stage], Shape::kStageBytes);
                    tma_load_2d(sdelta + stage * (RB * kStepCols), &tmap_delta, col0 + s * kStepCols, rb * RB,
                                &full[stage]);
                    tma_load_2d(sx + stage * (P * kStepCols), &tmap_x, col0 + s * kStepCols, 0, &full[stage]);
                    ++issued;
                    if (++stage == kStages) {
                        stage = 0;
                        phase ^= 1u;
                    }
                }
            }
            // Do not leave while copies issued by this thread may still be in
            // flight: wait (bounded) for the last min(issued, kStages) stages.
            const int pending = issued < kStages ? (int)issued : kStages;
            for (int k = 0; k < pending; ++k) {
                if (--stage < 0) {
                    stage = kStages - 1;
                    phase ^= 1u;
                }
                // phase now holds the parity that stage's latest fill completes.
                mbar_wait_bounded(&full[stage], phase, a.err, kDevTimeoutFull);
            }
        }
        return;
    }

    // -------------------------------------------------------- consumer warps
    const C* xg = static_cast<const C*>(a.x);
    Acc* gpart = static_cast<Acc*>(a.gpart);
    int stage = 0;
    uint32_t phase = 0;
    PairConstsF32 kc{a.k_e, a.log2_k2, a.tp0, a.tp1, a.tp2, a.ts0, a.ts1, a.ts2};
    constexpr int kFoldSteps = F32 ? (kLogFoldPairs / (RW * 4) > 0 ? kLogFoldPairs / (RW * 4) : 1) : 1 << 30;

    for (int t = blockIdx.x; t < a.n_tiles; t += gridDim.x) {
        const int rb = t / a.n_chunks;
        const int cb = t - rb * a.n_chunks;
        const int col0 = cb * a.chunk_steps * kStepCols;
        const int steps = min(a.chunk_steps, (a.n - col0 + kStepCols - 1) / kStepCols);
        const int row0 = rb * RB + warp * RW;

        C xi[RW][P];
        bool rows_clean = true;
#pragma unroll
        for (int r = 0; r < RW; ++r) {
            const int i = row0 + r;
            rows_clean &= (a.row_nan[i] == 0);
#pragma unroll
            for (int q = 0; q < P; ++q) xi[r][q] = xg[(size_t)q * a.x_ld + i];
        }

        C g[RW][P];
#pragma unroll
        for (int r = 0; r < RW; ++r)
#pragma unroll
            for (int q = 0; q < P; ++q) g[r][q] = C(0);
        // likelihood accumulators
        float r2_step = 0.f, r2_hi = 0.f, r2_lo = 0.f, prod = 1.f, log2_sum = 0.f;  // FP32 mode
        double r2_d = 0.0, lsum_d = 0.0;                                               // FP64 mode

        bool alive = true;
        for (int s = 0; s < steps; ++s) {
            if (!mbar_wait_bounded(&full[stage], phase, a.err, kDevTimeoutFull)) {
                alive = false;
                break;
            }
            const int j0 = col0 + s * kStepCols;
            const bool masked = !rows_clean || (j0 + kStepCols > a.n) || (j0 < row0 + RW && row0 < j0 + kStepCols);
            const S* dtile = sdelta + stage * (RB * kStepCols) + (warp * RW) * kStepCols + 4 * lane;
            const C* xtile = sx + stage * (P * kStepCols) + 4 * lane;

            C xj[P][4];
#pragma unroll
            for (int q = 0; q < P; ++q) {
                if constexpr (F32) {
                    const float4 v = *reinterpret_cast<const float4*>(xtile + q * kStepCols);
                    xj[q][0] = v.x; xj[q][1] = v.y; xj[q][2] = v.z; xj[q][3] = v.w;
                } else {
                    const double2 v0 = *reinterpret_cast<const double2*>(xtile + q * kStepCols);
                    const double2 v1 = *reinterpret_cast<const double2*>(xtile + q * kStepCols + 2);
                    xj[q][0] = v0.x; xj[q][1] = v0.y; xj[q][2] = v1.x; xj[q][3] = v1.y;
                }
            }
#pragma unroll
            for (int r = 0; r < RW; ++r) {
                S dl[4];
                if constexpr (sizeof(S) == 4) {
                    const float4 v = *reinterpret_cast<const float4*>(dtile + r * kStepCols);
                    dl[0] = v.x; dl[1] = v.y; dl[2] = v.z; dl[3] = v.w;
                } else {
                    const double2 v0 = *reinterpret_cast<const double2*>(dtile + r * kStepCols);
                    const double2 v1 = *reinterpret_cast<const double2*>(dtile + r * kStepCols + 2);
                    dl[0] = v0.x; dl[1] = v0.y; dl[2] = v1.x; dl[3] = v1.y;
                }
                const int i = row0 + r;
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    const int j = j0 + 4 * lane + c;
                    if constexpr (F32) {
                        if (masked) {
                            const bool valid = (j < a.n) && (i != j) && (dl[c] == dl[c]) && (i < a.n);
                            pair_f32<P, TRUNC, true>(xi[r], xj, c, (float)dl[c], valid, kc, g[r], r2_step, prod);
                        } else {
                            pair_f32<P, TRUNC, false>(xi[r], xj, c, (float)dl[c], true, kc, g[r], r2_step, prod);
                        }
                    } else {
                        if (masked) {
                            const bool valid = (j < a.n) && (i != j) && (dl[c] == dl[c]) && (i < a.n);
                            pair_f64<P, TRUNC, true>(xi[r], xj, c, (double)dl[c], valid, a.tau, a.sqrt_tau, g[r],
                                                     r2_d, lsum_d);
                        } else {
                            pair_f64<P, TRUNC, false>(xi[r], xj, c, (double)dl[c], true, a.tau, a.sqrt_tau, g[r],
                                                      r2_d, lsum_d);
                        }
                    }
                }
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[stage]);
            if (++stage == kStages) {
                stage = 0;
                phase ^= 1u;
            }
            if constexpr (F32) {
                if ((s + 1) % kFoldSteps == 0 || s + 1 == steps) {
                    if (TRUNC) {
                        log2_sum += lg2_approx(prod);
                        prod = 1.f;
                    }
                    float hi, e;
                    two_sum(r2_hi, r2_step, hi, e);
                    r2_hi = hi;
                    r2_lo += e;
                    r2_step = 0.f;
                }
            }
        }
        if (!alive) return;

        // ---- epilogue: per-warp partials of this tile
#pragma unroll
        for (int r = 0; r < RW; ++r)
#pragma unroll
            for (int q = 0; q < P; ++q) {
                C v = g[r][q];
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
                g[r][q] = v;
            }
#pragma unroll
        for (int r = 0; r < RW; ++r)
#pragma unroll
            for (int q = 0; q < P; ++q)
                if (lane == r * P + q) gpart[((size_t)cb * a.rows_padded + row0 + r) * P + q] = g[r][q];

        double lr2, llog;
        if constexpr (F32) {
            lr2 = (double)r2_hi + (double)r2_lo;
            llog = -0.69314718055994530942 * (double)log2_sum;
        } else {
            lr2 = r2_d;
            llog = lsum_d;
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            lr2 += __shfl_xor_sync(0xffffffffu, lr2, off);
            llog += __shfl_xor_sync(0xffffffffu, llog, off);
        }
        if (lane == 0) {
            a.lpart[((size_t)t * kConsumerWarps + warp) * 2 + 0] = lr2;
            a.lpart[((size_t)t * kConsumerWarps + warp) * 2 + 1] = llog;
        }
        __threadfence();
        __syncwarp();
        unsigned prev = 0;
        if (lane == 0) prev = atomicAdd(&a.rb_count[rb], 1u);
        prev = __shfl_sync(0xffffffffu, prev, 0);
        if (prev != (unsigned)(kConsumerWarps * a.n_chunks - 1)) continue;

        // ---- this warp completed row block rb: finalise its gradient rows and likelihood
        __threadfence();
        for (int idx = lane; idx < RB * P; idx += 32) {
            const int row = rb * RB + idx / P;
            const int q = idx - (idx / P) * P;
            double sum = 0.0;
            for (int k = 0; k < a.n_chunks; ++k) sum += (double)__ldcg(&gpart[((size_t)k * a.rows_padded + row) * P + q]);
            if (row < a.n) a.grad_out[(size_t)row * P + q] = a.tau * sum;
        }
        double br2 = 0.0, blog = 0.0;
        for (int idx = lane; idx < a.n_chunks * kConsumerWarps; idx += 32) {
            const size_t base = ((size_t)rb * a.n_chunks * kConsumerWarps + idx) * 2;
            br2 += __ldcg(&a.lpart[base]);
            blog += __ldcg(&a.lpart[base + 1]);
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            br2 += __shfl_xor_sync(0xffffffffu, br2, off);
            blog += __shfl_xor_sync(0xffffffffu, blog, off);
        }
        if (lane == 0) {
            a.lrow[2 * rb] = br2;
            a.lrow[2 * rb + 1] = blog;
            a.rb_count[rb] = 0u;
        }
        __threadfence();
        __syncwarp();
        if (lane == 0) prev = atomicAdd(a.done_count, 1u);
        prev = __shfl_sync(0xffffffffu, prev, 0);
        if (prev != (unsigned)(a.n_row_blocks - 1)) continue;

        // ---- last row block: total likelihood sums in a fixed order
        __threadfence();
        double tr2 = 0.0, tlog = 0.0;
        for (int k = lane; k < a.n_row_blocks; k += 32) {
            tr2 += __ldcg(&a.lrow[2 * k]);
            tlog += __ldcg(&a.lrow[2 * k + 1]);
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            tr2 += __shfl_xor_sync(0xffffffffu, tr2, off);
            tlog += __shfl_xor_sync(0xffffffffu, tlog, off);
        }
        if (lane == 0) {
            a.sums_out[0] = tr2;
            a.sums_out[1] = tlog;
            // src/NewMultiDimensionalScaling.hpp:198-202 and :554-557: halve the
            // ordered-pair total; without truncation scale by 0.5 * tau.
            a.sums_out[2] = a.truncation ? 0.5 * (0.5 * a.tau * tr2 + tlog) : 0.5 * a.tau * (0.5 * tr2);
            *a.done_count = 0u;
        }
    }
}

}  // namespace mdsx
