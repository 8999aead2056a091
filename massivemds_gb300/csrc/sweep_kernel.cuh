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
// Work decomposition (stream-K). delta rows are grouped in row blocks of
// RB = 8*RW rows; a unit is one row block x one 128-column stage, units are
// numbered row-block-major (u = rb * S + step, S = ceil(N / 128)), and CTA c of
// G takes the contiguous range [c*U/G, (c+1)*U/G) of the U units, so every CTA
// gets the same work to within one stage. Within its range a CTA walks row-block
// segments; consumer warps keep their gradient rows in registers for a whole
// segment and publish only when the segment ends. Each CTA has one producer
// warp that streams [RB x 128] delta boxes and [P x 128] location boxes into a
// kStages shared-memory ring with TMA (cp.async.bulk.tensor.2d), and 8 consumer
// warps; consumer warp w owns rows w*RW .. w*RW+RW-1 of the box, each lane 4
// consecutive columns (128-bit shared loads).
//
// Reductions are deterministic. A row block is split between the consecutive
// CTAs whose ranges meet it; each warp writes its segment partials (gradient
// rows, and the pair of likelihood sums) to the slot of its CTA; the warp that
// completes a row block (an atomic counter per row block; no thread ever waits
// on another CTA) sums that row block's slots in CTA order, and the warp that
// completes the last row block sums the row-block likelihood partials in a
// fixed order. Counters reset themselves for the next launch.
//
// FP32 mode: pair arithmetic in FP32 with MUFU rsqrt/ex2/rcp; Phi from the
// rational tail fit in normal_rational.h (one ex2 shared by Phi and phi, one rcp
// giving 1/Phi); logPhi summed as log2 of running products of 1/Phi (one lg2
// per 64 pairs); r^2 sums compensated with TwoSum; per-tile partials promoted to
// FP64 for every reduction above the warp. FP64 mode: pair arithmetic in FP64
// with a Newton-refined rsqrt_f64, and log Phi and phi / Phi from the Taylor
// table of normal_dd.h (normal_f64, in shared memory); normal_cdf_pdf_f64 (our
// Mills-ratio fit with CUDA's exp) remains for the FP64 self-test.
#pragma once

#include <cstdint>
#include <cuda.h>

#include "normal_dd.h"
#include "normal_mills_f64.h"
#include "ptx.cuh"

namespace mdsx {

constexpr int kConsumerWarps = 8;
constexpr int kThreads = (kConsumerWarps + 1) * 32;  // + 1 producer warp
constexpr int kStepCols = 128;                       // columns per stage: 32 lanes x 4
#ifndef MDSX_STAGES
#define MDSX_STAGES 4
#endif
#ifndef MDSX_F32_MIN_CTAS
#define MDSX_F32_MIN_CTAS 2
#endif
constexpr int kStages = MDSX_STAGES;  // depth of the TMA ring
constexpr int kLogFoldPairs = 64;

struct SweepArgs {
    int n;               // locations N (the columns of delta)
    int row_offset;      // first row of delta this launch covers (a row partition; 0 for the whole matrix)
    int rows;            // rows covered: [row_offset, row_offset + rows); N for the whole matrix
    int n_row_blocks;    // ceil(rows / RB)
    int steps_per_row;   // S = ceil(N / 128): units per row block
    int grid;            // G: CTAs launched (<= U, so no CTA has an empty range)
    long long n_units;   // U = n_row_blocks * S
    int max_slots;       // most CTAs meeting one row block
    int rows_padded;     // n_row_blocks * RB
    int x_ld;            // row stride of the SoA location array [P][x_ld], >= row_offset + rows_padded
    const void* x;       // SoA locations (compute type)
    const int* row_nan;  // [rows_padded], by covered row; nonzero: row has a NaN, or lies past the covered rows
    // FP32 pair constants (d-space): E' = 2^(d^2 k_e + log2_k2) = exp(-tau d^2/2)/sqrt(2 pi tau)
    float k_e, log2_k2;
    float tp0, tp1, tp2, ts0, ts1, ts2;  // 1/Phi = S(d) / (S(d) - E' P(d))
    double tau, sqrt_tau;
    // scratch
    void* gpart;           // [n_row_blocks][max_slots][RB][P] partial gradients (accumulator type)
    double* lpart;         // [n_row_blocks][max_slots][kConsumerWarps][2] likelihood partials
    double* lrow;          // [n_row_blocks][2]
    unsigned* rb_count;    // [n_row_blocks] warp publications per row block
    unsigned* done_count;  // [1] completed row blocks
    // outputs
    double* grad_out;  // [rows][P] = tau * sum_j ..., row-major, covered rows only
    double* sums_out;  // [0] = sum of r^2, [1] = sum of logPhi, over ordered non-missing pairs,
                       // [2] = getSumOfIncrements() of those sums
    int truncation;
    int* err;
    const double* normal_table_f64;  // FP64 math with truncation: normal_f64_table (kNormalF64Doubles)
    double* sum_copy;                // optional: also receives getSumOfIncrements() (the caller's buffer)
};

// The FP64 normal-tail table in shared memory (a static array of the kernel
// that calls it; two doubles where the table is not used).
template <bool ENABLE>
__device__ __forceinline__ double* sweep_normal_table() {
    __shared__ __align__(16) double tab[ENABLE ? kNormalF64Doubles : 2];
    return tab;
}

// CTA whose unit range [c*U/G, (c+1)*U/G) holds unit u (requires G <= U).
__host__ __device__ inline int cta_of_unit(long long u, long long n_units, int grid) {
    return (int)(((u + 1) * (long long)grid - 1) / n_units);
}
__host__ __device__ inline long long cta_unit_begin(int c, long long n_units, int grid) {
    return (long long)c * n_units / grid;
}


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

// Packed FP32 (Blackwell f32x2): two pairs per instruction, the two adjacent
// columns 2h and 2h+1 of a lane's 4 columns. A pack is the 64-bit register
// pair the 128-bit shared loads of delta and x_j already deliver.
struct f2 {
    unsigned long long v;
};
__device__ __forceinline__ f2 pk(float a, float b) {
    f2 r;
    asm("mov.b64 %0, {%1,%2};" : "=l"(r.v) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void upk(f2 x, float& a, float& b) {
    asm("mov.b64 {%0,%1}, %2;" : "=f"(a), "=f"(b) : "l"(x.v));
}
__device__ __forceinline__ f2 ffma2(f2 a, f2 b, f2 c) {
    f2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d.v) : "l"(a.v), "l"(b.v), "l"(c.v));
    return d;
}
__device__ __forceinline__ f2 fmul2(f2 a, f2 b) {
    f2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d.v) : "l"(a.v), "l"(b.v));
    return d;
}
__device__ __forceinline__ f2 fadd2(f2 a, f2 b) {
    f2 d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d.v) : "l"(a.v), "l"(b.v));
    return d;
}
__device__ __forceinline__ f2 rsqrt2(f2 x) {
    float a, b;
    upk(x, a, b);
    return pk(rsqrt_approx(a), rsqrt_approx(b));
}
__device__ __forceinline__ f2 ex2_2(f2 x) {
    float a, b;
    upk(x, a, b);
    return pk(ex2_approx(a), ex2_approx(b));
}
__device__ __forceinline__ f2 rcp2(f2 x) {
    float a, b;
    upk(x, a, b);
    return pk(rcp_approx(a), rcp_approx(b));
}
__device__ __forceinline__ f2 sel2(bool k0, bool k1, f2 x, float fill) {
    float a, b;
    upk(x, a, b);
    return pk(k0 ? a : fill, k1 ? b : fill);
}
__device__ __forceinline__ float sum2(f2 x) {
    float a, b;
    upk(x, a, b);
    return a + b;
}

// Pair constants in d-space, each duplicated into a pack:
//   E'    = 2^(d^2 k_e + log2_k2) = exp(-tau d^2 / 2) / sqrt(2 pi tau)
//   1/Phi = S(d) / A,  A = S(d) - E' P(d),  S monic cubic (ts*), P quadratic (-P = ntp*)
//   tiny  = 1e-30, the start of the d^2 sum: d^2 is unchanged above ~1e-23, and
//           coincident points (d^2 = 0, i != j) get d ~ 1e-15 instead of 0 * inf =
//           NaN, so their likelihood term is the reference's (d = 0) and finite.
struct PairConstsF32 {
    f2 m1, k_e, log2_k2, ntp0, ntp1, ntp2, ts0, ts1, ts2;
    f2 tiny{0x0DA242600DA24260ull};  // (1e-30f, 1e-30f)
};

// Two ordered pairs (i, j), (i, j+1) in packed FP32. With r = delta - d,
// accumulates r^2 into r2, 1/Phi into prod and
//   -(r - phi(z) / (sqrt(tau) Phi(z))) / d * (x_i - x_j)
// into g: the negated gradient term (tau and the sign are applied at
// finalisation), which lets every negation fold into a coefficient.
template <int P, bool TRUNC, bool MASKED>
__device__ __forceinline__ void pair2_f32(const f2 (&xi)[P], const f2 (&xj)[P], f2 delta, bool v0, bool v1,
                                          const PairConstsF32& k, f2 (&g)[P], f2& r2, f2& prod) {
    f2 dx[P];
#pragma unroll
    for (int q = 0; q < P; ++q) dx[q] = ffma2(xj[q], k.m1, xi[q]);  // x_i - x_j
    f2 d2 = ffma2(dx[0], dx[0], k.tiny);
#pragma unroll
    for (int q = 1; q < P; ++q) d2 = ffma2(dx[q], dx[q], d2);
    const f2 rs = rsqrt2(d2);
    const f2 d = fmul2(d2, rs);
    f2 nres = ffma2(delta, k.m1, d);  // d - delta
    if (MASKED) nres = sel2(v0, v1, nres, 0.0f);
    r2 = ffma2(nres, nres, r2);
    f2 c;
    if (TRUNC) {
        const f2 e = ex2_2(ffma2(d2, k.k_e, k.log2_k2));
        const f2 npp = ffma2(ffma2(k.ntp2, d, k.ntp1), d, k.ntp0);           // -P(d)
        const f2 ss = ffma2(ffma2(fadd2(d, k.ts2), d, k.ts1), d, k.ts0);     // S(d)
        const f2 aa = ffma2(e, npp, ss);                                     // S - E' P
        f2 iphi = fmul2(ss, rcp2(aa));                                       // 1 / Phi
        if (MASKED) iphi = sel2(v0, v1, iphi, 1.0f);
        prod = fmul2(prod, iphi);
        c = fmul2(ffma2(e, iphi, nres), rs);
    } else {
        c = fmul2(nres, rs);
    }
    if (MASKED) c = sel2(v0, v1, c, 0.0f);
#pragma unroll
    for (int q = 0; q < P; ++q) g[q] = ffma2(c, dx[q], g[q]);
}

// Normal CDF and density at z >= 0 in FP64 with one exponential (the FP64
// helpers' self-test, mdsx_selftest_math_f64; the sweeps use normal_f64):
// Phi(z) = 1 - Q(z), Q(z) = phi(z) R(z) with R the Mills ratio from our rational
// fit (normal_mills_f64.h, evaluated at min(z, 8.5), where Q < 1e-17 beyond);
// the exponential of the density serves both. |Phi - Phi_exact| <= 1e-15.
__device__ __forceinline__ void normal_cdf_pdf_f64(double z, double& cdf, double& pdf) {
    pdf = 0.39894228040143267794 * exp(-0.5 * z * z);
    double num, den;
    mills_ratio_f64(fmin(z, kMillsClamp), num, den);
    cdf = 1.0 - pdf * num * rcp_f64(den);
}

// One ordered pair in FP64 (rsqrt_f64; log Phi and phi / Phi from the Taylor
// table of normal_f64, in shared memory): log Phi adds into the row's sum lsum.
template <int P, bool TRUNC, bool MASKED>
__device__ __forceinline__ void pair_f64(const double (&xi)[P], const double (&xj)[P][4], int c, double delta,
                                         bool valid, double sqrt_tau, double inv_sqrt_tau, const double* tab,
                                         double (&g)[P], double& r2, double& lsum) {
    double dx[P];
#pragma unroll
    for (int q = 0; q < P; ++q) dx[q] = xi[q] - xj[q][c];
    double d2 = dx[0] * dx[0];
#pragma unroll
    for (int q = 1; q < P; ++q) d2 = fma(dx[q], dx[q], d2);
    if (MASKED && !valid) return;
    // coincident points (d2 = 0): d = 0 as the reference's sqrt gives; rs is NaN,
    // so their gradient terms are NaN where the reference's divide by d = 0
    const double rs = rsqrt_f64(d2);
    const double d = d2 >= kMinNormalF64 ? d2 * rs : 0.0;
    double res = delta - d;
    r2 = fma(res, res, r2);
    double cc;
    if (TRUNC) {
        double lc, ratio;
        normal_f64(d * sqrt_tau, tab, lc, ratio);
        lsum += lc;
        cc = fma(-ratio, inv_sqrt_tau, res) * rs;  // (res - phi / (Phi sqrt_tau)) / d
    } else {
        cc = res * rs;
    }
#pragma unroll
    for (int q = 0; q < P; ++q) g[q] = fma(cc, dx[q], g[q]);
}

// One pipeline stage of one consumer warp: RW rows x 4 columns per lane, as
// 2*RW packed pairs of pairs. MASKED selects the path with the missing-pair /
// bounds mask; it is decided once per stage (warp-uniform), so the fast path
// carries no per-pair branch. Gradient accumulators are per row; one r^2 pack
// and one 1/Phi product pack per lane keep the register budget.
template <int P, bool TRUNC, bool MASKED, int RW>
__device__ __forceinline__ void stage_f32(const float* __restrict__ dtile, const float* __restrict__ xtile,
                                          const f2 (&xi)[RW][P], int i0, int j0, int n, int i_lim, int lane,
                                          const PairConstsF32& kc, f2 (&g)[RW][P], f2& r2, f2& prod) {
    f2 xj[2][P];
#pragma unroll
    for (int q = 0; q < P; ++q) {
        const ulonglong2 v = *reinterpret_cast<const ulonglong2*>(xtile + q * kStepCols);
        xj[0][q].v = v.x;
        xj[1][q].v = v.y;
    }
    f2 dl[RW][2];
#pragma unroll
    for (int r = 0; r < RW; ++r) {
        const ulonglong2 v = *reinterpret_cast<const ulonglong2*>(dtile + r * kStepCols);
        dl[r][0].v = v.x;
        dl[r][1].v = v.y;
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
#pragma unroll
        for (int r = 0; r < RW; ++r) {
            bool v0 = true, v1 = true;
            if (MASKED) {
                float a, b;
                upk(dl[r][h], a, b);
                const int i = i0 + r, j = j0 + 4 * lane + 2 * h;
                v0 = (j < n) && (i < i_lim) && (i != j) && (a == a);
                v1 = (j + 1 < n) && (i < i_lim) && (i != j + 1) && (b == b);
            }
            pair2_f32<P, TRUNC, MASKED>(xi[r], xj[h], dl[r][h], v0, v1, kc, g[r], r2, prod);
        }
    }
}

template <int P, bool TRUNC, bool MASKED, int RW, typename S>
__device__ __forceinline__ void stage_f64(const S* __restrict__ dtile, const double* __restrict__ xtile,
                                          const double (&xi)[RW][P], int i0, int j0, int n, int i_lim, int lane,
                                          double sqrt_tau, double inv_sqrt_tau, const double* tab,
                                          double (&g)[RW][P], double (&r2)[RW], double (&lsum)[RW]) {
    double xj[P][4];
#pragma unroll
    for (int q = 0; q < P; ++q) {
        const double2 v0 = *reinterpret_cast<const double2*>(xtile + q * kStepCols);
        const double2 v1 = *reinterpret_cast<const double2*>(xtile + q * kStepCols + 2);
        xj[q][0] = v0.x; xj[q][1] = v0.y; xj[q][2] = v1.x; xj[q][3] = v1.y;
    }
#pragma unroll
    for (int r = 0; r < RW; ++r) {
        double dl[4];
        if constexpr (sizeof(S) == 4) {
            const float4 v = *reinterpret_cast<const float4*>(dtile + r * kStepCols);
            dl[0] = v.x; dl[1] = v.y; dl[2] = v.z; dl[3] = v.w;
        } else {
            const double2 v0 = *reinterpret_cast<const double2*>(dtile + r * kStepCols);
            const double2 v1 = *reinterpret_cast<const double2*>(dtile + r * kStepCols + 2);
            dl[0] = v0.x; dl[1] = v0.y; dl[2] = v1.x; dl[3] = v1.y;
        }
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            bool valid = true;
            if (MASKED) {
                const int i = i0 + r, j = j0 + 4 * lane + c;
                valid = (j < n) && (i < i_lim) && (i != j) && (dl[c] == dl[c]);
            }
            pair_f64<P, TRUNC, MASKED>(xi[r], xj, c, dl[c], valid, sqrt_tau, inv_sqrt_tau, tab, g[r], r2[r],
                                       lsum[r]);
        }
    }
}

// Sums K values held by every lane over the 32 lanes of the warp with K2 - 1
// exchanges (K2 = K rounded up to a power of two, K2 <= 32) instead of 5 per
// value. Afterwards lane l holds the total of value index l >> (5 - log2 K2)
// in v[0]; lanes with l % (32/K2) == 0 are the writers. Fixed order:
// deterministic.
template <int K, typename T>
__device__ __forceinline__ void warp_transpose_reduce(T (&v)[K], int lane) {
    constexpr int K2 = K <= 1 ? 1 : K <= 2 ? 2 : K <= 4 ? 4 : K <= 8 ? 8 : K <= 16 ? 16 : 32;
    static_assert(K <= 32, "too many values");
    T w[K2];
#pragma unroll
    for (int k = 0; k < K2; ++k) w[k] = k < K ? v[k] : T(0);
    int o = 16;
#pragma unroll
    for (int cnt = K2; cnt > 1; cnt >>= 1, o >>= 1) {
        const bool upper = (lane & o) != 0;
#pragma unroll
        for (int k = 0; k < cnt / 2; ++k) {
            const T send = upper ? w[k] : w[k + cnt / 2];
            const T keep = upper ? w[k + cnt / 2] : w[k];
            w[k] = keep + __shfl_xor_sync(0xffffffffu, send, o);
        }
    }
#pragma unroll
    for (; o > 0; o >>= 1) w[0] += __shfl_xor_sync(0xffffffffu, w[0], o);
    v[0] = w[0];
}

template <int K>
struct TransposeShape {
    static constexpr int K2 = K <= 1 ? 1 : K <= 2 ? 2 : K <= 4 ? 4 : K <= 8 ? 8 : K <= 16 ? 16 : 32;
    static constexpr int kLog2 = K2 == 1 ? 0 : K2 == 2 ? 1 : K2 == 4 ? 2 : K2 == 8 ? 3 : K2 == 16 ? 4 : 5;
    static constexpr int kLaneShift = 5 - kLog2;  // value index = lane >> kLaneShift
};

__device__ __forceinline__ void fence_acq_rel_gpu() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }

// --------------------------------------------------------------- the kernel

template <typename C, typename S, int P, bool TRUNC>
__global__ void __launch_bounds__(kThreads, sizeof(C) == 4 ? MDSX_F32_MIN_CTAS : 1)
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
    const int S_ = a.steps_per_row;
    const long long u_begin = cta_unit_begin(blockIdx.x, a.n_units, a.grid);
    const long long u_end = cta_unit_begin(blockIdx.x + 1, a.n_units, a.grid);

    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], kConsumerWarps);
        }
        fence_mbar_init();
    }
    // FP64 math with truncation: the normal-tail table into shared memory
    double* tab = sweep_normal_table<!F32 && TRUNC>();
    if constexpr (!F32 && TRUNC) {
        const double2* src = reinterpret_cast<const double2*>(a.normal_table_f64);
        for (int k = threadIdx.x; k < kNormalF64Doubles / 2; k += blockDim.x)
            reinterpret_cast<double2*>(tab)[k] = __ldg(&src[k]);
    }
    __syncthreads();

    if (warp == kConsumerWarps) {
        // ------------------------------------------------------ producer warp
        if (lane == 0) {
            prefetch_tensormap(&tmap_delta);
            prefetch_tensormap(&tmap_x);
            int stage = 0;
            uint32_t phase = 0;
            long long issued = 0;
            for (long long u = u_begin; u < u_end; ++u) {
                const int rb = (int)(u / S_);
                const int st = (int)(u - (long long)rb * S_);
                if (!mbar_wait_bounded(&empty[stage], phase ^ 1u, a.err, kDevTimeoutEmpty)) break;
                mbar_arrive_expect_tx(&full[stage], Shape::kStageBytes);
                tma_load_2d(sdelta + stage * (RB * kStepCols), &tmap_delta, st * kStepCols, rb * RB, &full[stage]);
                tma_load_2d(sx + stage * (P * kStepCols), &tmap_x, st * kStepCols, 0, &full[stage]);
                ++issued;
                if (++stage == kStages) {
                    stage = 0;
                    phase ^= 1u;
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
                mbar_wait_time_only(&full[stage], phase);
            }
        }
        return;
    }

    // -------------------------------------------------------- consumer warps
    const C* xg = static_cast<const C*>(a.x);
    Acc* gpart = static_cast<Acc*>(a.gpart);
    int stage = 0;
    uint32_t phase = 0;
    const double inv_sqrt_tau = 1.0 / a.sqrt_tau;
    const PairConstsF32 kc{pk(-1.f, -1.f),         pk(a.k_e, a.k_e), pk(a.log2_k2, a.log2_k2),
                           pk(-a.tp0, -a.tp0),     pk(-a.tp1, -a.tp1), pk(-a.tp2, -a.tp2),
                           pk(a.ts0, a.ts0),       pk(a.ts1, a.ts1),   pk(a.ts2, a.ts2)};

    for (long long u = u_begin; u < u_end;) {
        // one row-block segment [u, seg_end) of this CTA's range
        const int rb = (int)(u / S_);
        const int st0 = (int)(u - (long long)rb * S_);
        const long long rb_end = (long long)(rb + 1) * S_;
        const long long seg_end = u_end < rb_end ? u_end : rb_end;
        const int steps = (int)(seg_end - u);
        const int first_cta = cta_of_unit((long long)rb * S_, a.n_units, a.grid);
        const int n_slots = cta_of_unit(rb_end - 1, a.n_units, a.grid) - first_cta + 1;
        const int slot = blockIdx.x - first_cta;
        u = seg_end;
        const int row0 = rb * RB + warp * RW;     // covered-row index (row marks, partials, output)
        const int grow0 = a.row_offset + row0;     // row of the whole matrix (diagonal, locations)
        const int i_lim = a.row_offset + a.rows;

        C xi[RW][P];
        f2 xi2[RW][P];  // FP32: (x_i, x_i) packs
        bool rows_clean = true;
#pragma unroll
        for (int r = 0; r < RW; ++r) {
            const int i = row0 + r;
            rows_clean &= (a.row_nan[i] == 0);
#pragma unroll
            for (int q = 0; q < P; ++q) {
                xi[r][q] = xg[(size_t)q * a.x_ld + a.row_offset + i];
                if constexpr (F32) xi2[r][q] = pk(xi[r][q], xi[r][q]);
            }
        }

        // FP64 accumulators: gradient, r^2 and logPhi sums per row, and the
        // running product of Phi between log folds.
        C g[RW][P];
        C r2[RW], acc2[RW];
        // FP32 accumulators (packs): negated gradient, r^2 per fold interval,
        // running product of 1/Phi; and the compensated segment sums.
        f2 g2[RW][P], r2p = pk(0.f, 0.f), prodp = pk(1.f, 1.f);
#pragma unroll
        for (int r = 0; r < RW; ++r) {
            r2[r] = C(0);
            acc2[r] = C(0);
#pragma unroll
            for (int q = 0; q < P; ++q) {
                g[r][q] = C(0);
                g2[r][q] = pk(0.f, 0.f);
            }
        }
        float r2_hi = 0.f, r2_lo = 0.f, log2_sum = 0.f;

        bool alive = true;
        for (int s = 0; s < steps; ++s) {
            if (!mbar_wait_bounded(&full[stage], phase, a.err, kDevTimeoutFull)) {
                alive = false;
                break;
            }
            const int j0 = (st0 + s) * kStepCols;
            const bool masked = !rows_clean || (j0 + kStepCols > a.n) || (j0 < grow0 + RW && grow0 < j0 + kStepCols);
            const S* dtile = sdelta + stage * (RB * kStepCols) + (warp * RW) * kStepCols + 4 * lane;
            const C* xtile = sx + stage * (P * kStepCols) + 4 * lane;
            if constexpr (F32) {
                if (masked)
                    stage_f32<P, TRUNC, true, RW>(dtile, xtile, xi2, grow0, j0, a.n, i_lim, lane, kc, g2, r2p, prodp);
                else
                    stage_f32<P, TRUNC, false, RW>(dtile, xtile, xi2, grow0, j0, a.n, i_lim, lane, kc, g2, r2p, prodp);
            } else {
                if (masked)
                    stage_f64<P, TRUNC, true, RW>(dtile, xtile, xi, grow0, j0, a.n, i_lim, lane, a.sqrt_tau,
                                                  inv_sqrt_tau, tab, g, r2, acc2);
                else
                    stage_f64<P, TRUNC, false, RW>(dtile, xtile, xi, grow0, j0, a.n, i_lim, lane, a.sqrt_tau,
                                                   inv_sqrt_tau, tab, g, r2, acc2);
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[stage]);
            if (++stage == kStages) {
                stage = 0;
                phase ^= 1u;
            }
            if constexpr (F32) {
                // Each half of the product pack gains 2*RW factors in [1, 2]
                // per stage; fold before 64 factors, and at the end of the segment.
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
        }
        if (!alive) return;

        // ---- publish this warp's segment partials into the CTA's slot of row block rb
        const size_t slot_base = (size_t)rb * a.max_slots + slot;
        {
            constexpr int K = RW * P;
            using TS = TransposeShape<K>;
            C gv[K];
#pragma unroll
            for (int r = 0; r < RW; ++r)
#pragma unroll
                for (int q = 0; q < P; ++q) {
                    if constexpr (F32)
                        gv[r * P + q] = sum2(g2[r][q]);
                    else
                        gv[r * P + q] = g[r][q];
                }
            warp_transpose_reduce<K>(gv, lane);
            const int idx = lane >> TS::kLaneShift;
            if ((lane & ((1 << TS::kLaneShift) - 1)) == 0 && idx < K)
                gpart[(slot_base * RB + warp * RW) * P + idx] = gv[0];
        }
        double lr2, llog;
        if constexpr (F32) {
            float lv[3] = {r2_hi, r2_lo, log2_sum};
            warp_transpose_reduce<3>(lv, lane);
            // lanes 0, 8, 16 hold the totals of r2_hi, r2_lo, log2_sum
            const float t_hi = __shfl_sync(0xffffffffu, lv[0], 0);
            const float t_lo = __shfl_sync(0xffffffffu, lv[0], 8);
            const float t_lg = __shfl_sync(0xffffffffu, lv[0], 16);
            lr2 = (double)t_hi + (double)t_lo;
            llog = -0.69314718055994530942 * (double)t_lg;
        } else {
            double lv[2] = {0.0, 0.0};
#pragma unroll
            for (int r = 0; r < RW; ++r) {
                lv[0] += r2[r];
                lv[1] += acc2[r];
            }
            warp_transpose_reduce<2>(lv, lane);
            lr2 = __shfl_sync(0xffffffffu, lv[0], 0);
            llog = __shfl_sync(0xffffffffu, lv[0], 16);
        }
        if (lane == 0) {
            a.lpart[(slot_base * kConsumerWarps + warp) * 2 + 0] = lr2;
            a.lpart[(slot_base * kConsumerWarps + warp) * 2 + 1] = llog;
        }
        // The warp barrier orders every lane's partial stores before lane 0's
        // release fence and counter increment.
        __syncwarp();
        unsigned prev = 0;
        if (lane == 0) {
            fence_acq_rel_gpu();
            prev = atomicAdd(&a.rb_count[rb], 1u);
        }
        prev = __shfl_sync(0xffffffffu, prev, 0);
        if (prev != (unsigned)(kConsumerWarps * n_slots - 1)) continue;

        // ---- this warp completed row block rb: finalise its gradient rows and likelihood
        __threadfence();
        for (int idx = lane; idx < RB * P; idx += 32) {
            const int rr = idx / P;
            const int q = idx - rr * P;
            double sum = 0.0;
            for (int k = 0; k < n_slots; ++k)
                sum += (double)__ldcg(&gpart[(((size_t)rb * a.max_slots + k) * RB + rr) * P + q]);
            const int row = rb * RB + rr;
            // FP32 partials hold the negated gradient terms.
            if (row < a.rows) a.grad_out[(size_t)row * P + q] = (F32 ? -a.tau : a.tau) * sum;
        }
        double br2 = 0.0, blog = 0.0;
        for (int idx = lane; idx < n_slots * kConsumerWarps; idx += 32) {
            const size_t base = ((size_t)rb * a.max_slots * kConsumerWarps + idx) * 2;
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
        __syncwarp();
        if (lane == 0) {
            fence_acq_rel_gpu();
            prev = atomicAdd(a.done_count, 1u);
        }
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
            if (a.sum_copy) *a.sum_copy = a.sums_out[2];
            *a.done_count = 0u;
        }
    }
}

}  // namespace mdsx
