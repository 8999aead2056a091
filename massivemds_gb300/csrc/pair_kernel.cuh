// The fused sweep over unordered pairs: FP32 pair math (FP32 mode), or FP64
// pair math over FP32-stored delta (DELTA_F32 mode) or FP64-stored delta
// (default mode), P <= kPairMaxP.
//
// d_ij = d_ji, so everything a pair needs apart from delta -- the distance,
// 1/d, Phi(d sqrt(tau)) and phi/Phi -- is computed once per unordered pair
// {i, j} and used for both ordered pairs (i, j) and (j, i), each with its own
// delta_ij and delta_ji. The reference sums run over ordered pairs and delta
// need not be symmetric (src/NewMultiDimensionalScaling.hpp:402-410 mask,
// :421-461 gradient, :508-514 likelihood); both directions keep their own
// residual, mask, likelihood term and gradient term. The N x N delta matrix is
// still read once, and the transcendental work per ordered pair halves.
//
// Work decomposition. Columns form blocks J of 128, rows chunks I of 32. A unit
// is one (J, I) with I at or below J's diagonal (I >= 4J): rows [32I, 32I+32) x
// columns [128J, 128J+128), pairs i > j only. Units are numbered
// column-block-major (J, then I = 4J .. nc-1) and CTA c of G takes a
// contiguous range of units whose modelled cost is 1/G of the total (stream-K;
// the host weights diagonal units and column-block starts, see
// pair_unit_cost). Per unit the CTA loads with TMA
//   A   = delta[I rows][J cols]   32 x 128, plain rows
//   B   = delta[J rows][I cols]   128 x 32, 128-byte swizzled (two boxes of 16
//                                 columns for FP64 delta)
//   x_I = P location rows + the flag row, 32 columns (compute type)
//   x_J = the same over J's 128 columns, with the first unit of each J
// into a ring of PairShape::kStages stages (mbarrier full/empty pairs). Lane 0
// of warp m % 8 issues unit m's copies between its own units (the batch
// kernel: lane 0 of warp 0 for every unit), so all 8 warps of a CTA compute and
// 2 CTAs of 256 threads fit an SM at 128 registers (P = 4, 6: one CTA per SM,
// pair_min_ctas).
//
// Consumer warp w owns rows 4w .. 4w+3 of the chunk and lane l the columns
// l, l+32, l+64, l+96 of the block. B gives a lane its four rows of column j
// with one 128-bit load of row j, conflict-free because the 128-byte swizzle
// spreads the 16-byte chunk w of rows j .. j+7 over all banks. The math policy
// (PairMathF32: f32x2 packs of two rows; PairMathF64: scalar FP64) does the
// pairs and keeps the likelihood sums.
//
// Accumulation. Column gradients (the (j, i) terms) stay in registers while the
// CTA walks the units of one J and are written per (J, CTA slot, warp) when J
// changes; row gradients (the (i, j) terms) are summed over the warp per unit
// and written per (unit, row). pair_finish_kernel sums both kinds of partials
// in a fixed order, and the per-warp likelihood partials, so results are
// bitwise reproducible from run to run. No thread waits on another CTA.
#pragma once

#include <cstdint>
#include <cuda.h>

#include <type_traits>

#include "dd.h"
#include "normal_dd.h"
#include "ptx.cuh"
#include "sweep_kernel.cuh"

namespace mdsx {

constexpr int kPairCols = 128;  // columns per block J: 32 lanes x 4
constexpr int kPairRows = 32;   // rows per chunk I: 8 warps x 4
constexpr int kPairWarps = 8;
constexpr int kPairThreads = kPairWarps * 32;
constexpr int kPairMaxP = 6;     // FP32 pair math: packs of two rows (PairMathF32), or of two columns (PairMathF32Cols) above MDSX_PAIR_ROWPACK_MAX_P
constexpr int kPairMaxP64 = 6;   // FP64 pair math (one CTA per SM, pair_min_ctas_of)
#ifndef MDSX_PAIR_F32_STAGES
#define MDSX_PAIR_F32_STAGES 3  // TMA ring depth of the FP32 pair kernels
#endif
#ifndef MDSX_PAIR_F32_CTAS
#define MDSX_PAIR_F32_CTAS 2  // CTAs per SM of the FP32 pair kernels with P = 1, 2, 3, 5
#endif
#ifndef MDSX_FINISH_THREADS
#define MDSX_FINISH_THREADS 256  // threads per block of the pair sweep's finish kernel (P > MDSX_FINISH_SMALL_P)
#endif
#ifndef MDSX_FINISH_THREADS_SMALL_P
#define MDSX_FINISH_THREADS_SMALL_P 128  // the same for P <= MDSX_FINISH_SMALL_P
#endif
#ifndef MDSX_FINISH_SMALL_P
#define MDSX_FINISH_SMALL_P 2
#endif
#ifndef MDSX_FINISH_THREADS_F64
#define MDSX_FINISH_THREADS_F64 512  // the same for FP64 partials, every P
#endif
#ifndef MDSX_FINISH_SPLIT_F64
#define MDSX_FINISH_SPLIT_F64 4  // FP64 partials: finish blocks per row chunk
#endif
#ifndef MDSX_FINISH_CHUNK
#define MDSX_FINISH_CHUNK 8  // row-partial loads in flight per finish thread
#endif
#ifndef MDSX_FINISH_COL_CHUNK
#define MDSX_FINISH_COL_CHUNK 8  // column-partial loads in flight per finish thread
#endif
#ifndef MDSX_PAIR_ROTATE_ISSUER
#define MDSX_PAIR_ROTATE_ISSUER 1  // single-instance pair kernel: unit m's copies issued by warp m % 8
#endif
#ifndef MDSX_PAIR_EARLY_RELEASE
#define MDSX_PAIR_EARLY_RELEASE 1  // FP32 packs of rows: operands to registers, stage released before the math
#endif

// XB: bytes per location element (4: FP32 math, 8: FP64 math); SB: bytes per
// delta element. FP64 math is bound by the FP64 pipe, so two stages hide the
// copies; FP32 math gets three. B rows are 32 elements: with 8-byte delta they
// come as two 128-byte-swizzled boxes of 16 columns (kBBoxes), one after the other.
template <int P, int XB, int SB = 4>
struct PairShape {
    static constexpr int kStages = XB == 4 ? MDSX_PAIR_F32_STAGES : 2;
    static constexpr int kBBoxCols = 128 / SB;
    static constexpr int kBBoxes = kPairRows / kBBoxCols;
    static constexpr int kBBytes = kPairCols * kPairRows * SB;
    static constexpr int kABytes = kPairRows * kPairCols * SB;
    static constexpr int kXIBytes = (P + 1) * kPairRows * XB;
    static constexpr int kXJBytes = (P + 1) * kPairCols * XB;
    static constexpr int kXIOffset = kBBytes + kABytes;
    static constexpr int kXJOffset = kXIOffset + kXIBytes;
    // stage bases stay 1024-byte aligned, as the 128-byte swizzle of B requires
    static constexpr int kStageBytes = (kXJOffset + kXJBytes + 1023) / 1024 * 1024;
    static constexpr int kSmemBytes = kStages * kStageBytes + 2 * kStages * 8 + 1024;
};

// Optional leapfrog step fused into the finish kernel (the HMC driver): with
// the gradient g of the sweep, p += a (g - x Lambda) and x += b p per location
// (a = coef[0], b = coef[1]), x also written into the sweep's SoA location buffer.
struct PairLeapfrog {
    double* x;            // [N][P] positions
    double* mom;          // [N][P] momenta
    const double* coef;   // [2]: a, b (device memory: a captured graph follows step-size changes)
    void* soa;            // SoA location buffer [P][x_ld] of the sweep (float or double)
    int x_ld;
    int soa_f32;
    double lam[kPairMaxP * kPairMaxP];  // prior precision, row-major P x P
};

struct PairArgs {
    int n;               // locations N
    int nb;              // column blocks ceil(N / 128)
    int nc;              // row chunks ceil(N / 32)
    int grid;            // CTAs launched (<= n_units)
    int max_slots;       // most CTAs meeting one column block
    int truncation;
    long long n_units;   // sum over J of (nc - 4J)
    // FP32 pair constants (d-space), as in SweepArgs
    float k_e, log2_k2;
    float tp0, tp1, tp2, ts0, ts1, ts2;
    double tau, sqrt_tau;
    void* rowpart;     // [n_units][32][P]: per unit, the row sums of the (i, j) terms (partial type)
    void* colpart;     // [nb][max_slots][8][P][128]: per J, CTA slot and warp, column sums of the (j, i) terms
    double* lpart;     // [grid][8][2]: r^2 and logPhi sums per warp
    const long long* cta_begin;  // [grid + 1]: CTA c takes units [cta_begin[c], cta_begin[c+1])
    const int* j_first_cta;      // [nb]: first CTA whose range meets column block J
    const int* j_slots;          // [nb]: CTAs whose ranges meet column block J
    double* grad_out;  // [N][P]
    double* sums_out;  // [0] r^2, [1] logPhi over ordered non-missing pairs, [2] getSumOfIncrements()
    int* err;
    int leapfrog;       // nonzero: the finish applies `leap` to its rows
    PairLeapfrog leap;
    const float* normal_table;       // double-float pair math with truncation: normal_dd_table (kNormalDDFloats)
    const double* normal_table_f64;  // FP64 pair math with truncation: normal_f64_table (kNormalF64Doubles)
};

// Units of the column blocks before J: sum over J' < J of (nc - 4 J').
__host__ __device__ inline long long pair_units_before(int J, int nc) {
    return (long long)J * nc - 2LL * J * (J - 1);
}

// Modelled cost of the units of one column block, used by the host to split
// the units over CTAs: a unit costs 1, a diagonal unit (I < 4J + 4, masked
// path) kPairDiagExtra more, and the first unit of a block kPairBlockExtra
// more (column flush, x_J reload).
#ifndef MDSX_PAIR_DIAG_EXTRA
#define MDSX_PAIR_DIAG_EXTRA 0.6
#endif
#ifndef MDSX_PAIR_BLOCK_EXTRA
#define MDSX_PAIR_BLOCK_EXTRA 0.2
#endif
constexpr double kPairDiagExtra = MDSX_PAIR_DIAG_EXTRA;
constexpr double kPairBlockExtra = MDSX_PAIR_BLOCK_EXTRA;
__host__ __device__ inline double pair_unit_cost(int I, int J) {
    return 1.0 + (I < 4 * J + 4 ? kPairDiagExtra : 0.0) + (I == 4 * J ? kPairBlockExtra : 0.0);
}

// Column block of unit u: the largest J < nb with pair_units_before(J) <= u.
__host__ __device__ inline int pair_block_of_unit(long long u, int nb, int nc) {
    int lo = 0, hi = nb - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (pair_units_before(mid, nc) <= u)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// ------------------------------------------------------------ FP32 pair math

// Two unordered pairs {i, j}, {i+1, j} (one pack) in both directions. A
// direction's residual is d - delta (negated, as in pair2_f32), its
// coefficient c = (d - delta + E'/Phi) / d; the (i, j) term c_A (x_i - x_j)
// accumulates into the row pack racc, the (j, i) term c_B (x_i - x_j) into the
// column pack cacc (the sign and tau are applied by the finish kernel).
// Fast path: 1/Phi multiplies into prod once and is counted for both
// directions; masked path: each valid direction multiplies into prodm.
template <int P, bool TRUNC, bool MASKED>
__device__ __forceinline__ void pair_pack(const f2 (&xi)[P], const f2 (&nxj)[P], f2 dA, f2 dB, bool vA0, bool vA1,
                                          bool vB0, bool vB1, const PairConstsF32& k, f2 (&racc)[P],
                                          f2 (&cacc)[P], f2& r2, f2& prod, f2& prodm) {
    f2 dx[P];
#pragma unroll
    for (int q = 0; q < P; ++q) dx[q] = fadd2(xi[q], nxj[q]);  // x_i - x_j
    f2 d2 = ffma2(dx[0], dx[0], k.tiny);  // coincident points: d ~ 1e-15, not NaN (PairConstsF32)
#pragma unroll
    for (int q = 1; q < P; ++q) d2 = ffma2(dx[q], dx[q], d2);
    const f2 rs = rsqrt2(d2);
    const f2 d = fmul2(d2, rs);
    f2 nA = ffma2(dA, k.m1, d);
    f2 nB = ffma2(dB, k.m1, d);
    if (MASKED) {
        nA = sel2(vA0, vA1, nA, 0.0f);
        nB = sel2(vB0, vB1, nB, 0.0f);
    }
    r2 = ffma2(nA, nA, r2);
    r2 = ffma2(nB, nB, r2);
    f2 cA, cB;
    if (TRUNC) {
        const f2 e = ex2_2(ffma2(d2, k.k_e, k.log2_k2));
        const f2 npp = ffma2(ffma2(k.ntp2, d, k.ntp1), d, k.ntp0);        // -P(d)
        const f2 ss = ffma2(ffma2(fadd2(d, k.ts2), d, k.ts1), d, k.ts0);  // S(d)
        const f2 aa = ffma2(e, npp, ss);                                  // S - E' P
        const f2 iphi = fmul2(ss, rcp2(aa));                              // 1 / Phi
        const f2 trs = fmul2(fmul2(e, iphi), rs);                         // E' / (Phi d)
        if (MASKED) {
            prodm = fmul2(prodm, sel2(vA0, vA1, iphi, 1.0f));
            prodm = fmul2(prodm, sel2(vB0, vB1, iphi, 1.0f));
        } else {
            prod = fmul2(prod, iphi);
        }
        cA = ffma2(nA, rs, trs);
        cB = ffma2(nB, rs, trs);
    } else {
        cA = fmul2(nA, rs);
        cB = fmul2(nB, rs);
    }
    if (MASKED) {
        cA = sel2(vA0, vA1, cA, 0.0f);
        cB = sel2(vB0, vB1, cB, 0.0f);
    }
#pragma unroll
    for (int q = 0; q < P; ++q) {
        racc[q] = ffma2(cA, dx[q], racc[q]);
        cacc[q] = ffma2(cB, dx[q], cacc[q]);
    }
}

// One consumer warp's operands of one unit, held in registers so the warp can
// release the unit's stage before the pair math: the A packs (rows 4w + 2rp,
// 4w + 2rp + 1 of column lane + 32c), this lane's 16-byte chunks of B rows
// lane + 32c (rows 4w .. 4w+3 of the chunk) and the (x_i, x_i+1) packs.
template <int P>
struct PairOperandsF32 {
    f2 a[4][2];
    float4 b[4];
    f2 xi[2][P];
};

template <int P>
__device__ __forceinline__ void pair_load_f32(PairOperandsF32<P>& o, const float* __restrict__ sA,
                                              const float* __restrict__ sB, const float* __restrict__ sXI, int lane,
                                              int warp) {
    // this lane's 16-byte chunk (rows 4w .. 4w+3) of B row `lane`, 128-byte swizzle:
    // chunk c of a 128-byte row r sits at chunk c ^ (r & 7)
    const float* sBl = sB + lane * kPairRows + ((warp ^ (lane & 7)) << 2);
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        o.b[c] = *reinterpret_cast<const float4*>(sBl + c * (32 * kPairRows));
#pragma unroll
        for (int rp = 0; rp < 2; ++rp)
            o.a[c][rp] = pk(sA[(4 * warp + 2 * rp) * kPairCols + lane + 32 * c],
                            sA[(4 * warp + 2 * rp + 1) * kPairCols + lane + 32 * c]);
    }
#pragma unroll
    for (int q = 0; q < P; ++q) {
        const float4 x4 = *reinterpret_cast<const float4*>(sXI + q * kPairRows + 4 * warp);
        o.xi[0][q] = pk(x4.x, x4.y);
        o.xi[1][q] = pk(x4.z, x4.w);
    }
}

// One unit for one consumer warp: 4 rows x 4 columns per lane, both directions,
// from the operands in registers; i0 = first row of the warp, j0 = first column
// of the block.
template <int P, bool TRUNC, bool MASKED>
__device__ __forceinline__ void pair_unit(const PairOperandsF32<P>& o, const f2 (&nxj)[4][P], int i0, int j0, int n,
                                          int lane, const PairConstsF32& k, f2 (&racc)[2][P], f2 (&cacc)[4][P],
                                          f2& r2, f2& prod, float& l1) {
    f2 prodm = pk(1.f, 1.f);
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const float4 b = o.b[c];
        const int j = j0 + lane + 32 * c;
#pragma unroll
        for (int rp = 0; rp < 2; ++rp) {
            float a0, a1;
            upk(o.a[c][rp], a0, a1);
            const float b0 = rp == 0 ? b.x : b.z;
            const float b1 = rp == 0 ? b.y : b.w;
            bool vA0 = true, vA1 = true, vB0 = true, vB1 = true;
            if (MASKED) {
                const int i = i0 + 2 * rp;
                const bool ok0 = (i < n) && (j < n) && (i > j);
                const bool ok1 = (i + 1 < n) && (j < n) && (i + 1 > j);
                vA0 = ok0 && (a0 == a0);
                vA1 = ok1 && (a1 == a1);
                vB0 = ok0 && (b0 == b0);
                vB1 = ok1 && (b1 == b1);
            }
            pair_pack<P, TRUNC, MASKED>(o.xi[rp], nxj[c], o.a[c][rp], pk(b0, b1), vA0, vA1, vB0, vB1, k, racc[rp],
                                        cacc[c], r2, prod, prodm);
        }
    }
    if (MASKED && TRUNC) {
        float m0, m1;
        upk(prodm, m0, m1);
        l1 += lg2_approx(m0) + lg2_approx(m1);  // <= 16 factors in [1, 2] per half
    }
}

// Folds the r^2 pack and the 1/Phi product pack into compensated FP32 sums
// (TwoSum) and resets them.
template <bool TRUNC>
__device__ __forceinline__ void fold_sums(f2& r2, f2& prod, float& r2_hi, float& r2_lo, float& l2_hi, float& l2_lo) {
    float s0, s1, hi, e;
    upk(r2, s0, s1);
    two_sum(r2_hi, s0 + s1, hi, e);
    r2_hi = hi;
    r2_lo += e;
    r2 = pk(0.f, 0.f);
    if (TRUNC) {
        upk(prod, s0, s1);
        two_sum(l2_hi, lg2_approx(s0) + lg2_approx(s1), hi, e);
        l2_hi = hi;
        l2_lo += e;
        prod = pk(1.f, 1.f);
    }
}

// FP32 policy: f32x2 packs of two rows (pair_unit); FP32 partials; r^2 and
// log2 of the 1/Phi products folded every kFoldUnits units into compensated
// FP32 sums (TwoSum).
template <int P, bool TRUNC>
struct PairMathF32 {
    using X = float;     // location element in shared memory
    using S = float;     // delta element
    using Part = float;  // row and column partials
    static constexpr bool kXJEveryUnit = false;  // x_J is copied with the first unit of each block only
    __device__ static void prologue(const PairArgs&) {}  // no shared tables
    static constexpr int kMinCtas = 0;  // pair_min_ctas_of decides
    // The warp copies its operands of a unit into registers and releases the
    // stage before the pair math, so the next copy into it can start a unit
    // earlier (the ring runs one more unit ahead of the consumers).
    static constexpr bool kEarlyRelease = MDSX_PAIR_EARLY_RELEASE != 0;
    using Operands = PairOperandsF32<P>;
    static constexpr int kFoldUnits = 4;  // r^2 pack: 16 terms per half per unit; 1/Phi product: 8 factors
    struct Cols {        // one column block: negated (x_j, x_j) packs and the column sums
        f2 nxj[4][P];
        f2 acc[4][P];
    };
    struct Sums {
        f2 r2, prod;
        float r2_hi, r2_lo, l2_hi, l2_lo;  // l2: log2 of 1/Phi products counted for both directions
        float l1;                          // log2 of masked-path products, counted once
        int since_fold;
    };
    PairConstsF32 k;

    __device__ explicit PairMathF32(const PairArgs& a)
        : k{pk(-1.f, -1.f),     pk(a.k_e, a.k_e),   pk(a.log2_k2, a.log2_k2), pk(-a.tp0, -a.tp0), pk(-a.tp1, -a.tp1),
            pk(-a.tp2, -a.tp2), pk(a.ts0, a.ts0), pk(a.ts1, a.ts1),         pk(a.ts2, a.ts2)} {}

    __device__ static void init(Sums& s) {
        s.r2 = pk(0.f, 0.f);
        s.prod = pk(1.f, 1.f);
        s.r2_hi = s.r2_lo = s.l2_hi = s.l2_lo = s.l1 = 0.f;
        s.since_fold = 0;
    }
    __device__ static void begin_block(Cols& cols, const X* sXJ, int lane) {
#pragma unroll
        for (int c = 0; c < 4; ++c)
#pragma unroll
            for (int q = 0; q < P; ++q) {
                const float v = -sXJ[q * kPairCols + lane + 32 * c];
                cols.nxj[c][q] = pk(v, v);
                cols.acc[c][q] = pk(0.f, 0.f);
            }
    }
    __device__ static void load(Operands& o, const S* sA, const S* sB, const X* sXI, int lane, int warp) {
        pair_load_f32<P>(o, sA, sB, sXI, lane, warp);
    }
    // One unit from its operands: v[r * P + q] = this lane's sum of the (i, j) terms of row 4w + r.
    template <bool MASKED>
    __device__ void compute(const Operands& o, Cols& cols, Sums& s, int i0, int j0, int n, int lane,
                            Part (&v)[4 * P]) const {
        f2 racc[2][P];
#pragma unroll
        for (int q = 0; q < P; ++q) racc[0][q] = racc[1][q] = pk(0.f, 0.f);
        pair_unit<P, TRUNC, MASKED>(o, cols.nxj, i0, j0, n, lane, k, racc, cols.acc, s.r2, s.prod, s.l1);
#pragma unroll
        for (int rp = 0; rp < 2; ++rp)
#pragma unroll
            for (int q = 0; q < P; ++q) upk(racc[rp][q], v[(2 * rp) * P + q], v[(2 * rp + 1) * P + q]);
    }
    template <bool MASKED>
    __device__ void unit(const S* sA, const S* sB, const X* sXI, Cols& cols, Sums& s, int i0, int j0, int n,
                         int lane, int warp, Part (&v)[4 * P]) const {
        Operands o;
        load(o, sA, sB, sXI, lane, warp);
        compute<MASKED>(o, cols, s, i0, j0, n, lane, v);
    }
    __device__ static void after_unit(Sums& s) {
        if (++s.since_fold == kFoldUnits) {
            s.since_fold = 0;
            fold_sums<TRUNC>(s.r2, s.prod, s.r2_hi, s.r2_lo, s.l2_hi, s.l2_lo);
        }
    }
    __device__ static Part col_value(const Cols& cols, int c, int q) { return sum2(cols.acc[c][q]); }
    // Sum of r^2 and of log Phi (natural) over this lane's ordered pairs.
    __device__ static void result(Sums& s, double& r2, double& lsum) {
        fold_sums<TRUNC>(s.r2, s.prod, s.r2_hi, s.r2_lo, s.l2_hi, s.l2_lo);
        r2 = (double)s.r2_hi + (double)s.r2_lo;
        lsum = TRUNC ? -0.69314718055994530942 * (2.0 * ((double)s.l2_hi + (double)s.l2_lo) + (double)s.l1) : 0.0;
    }
};

// FP32 policy for larger P (5, 6): a pack is two columns of one row, so a lane
// keeps only its column sums (two column-pair packs x P) for the block and one
// row's x_i and row sums at a time; x_J comes with every unit and the lane reads
// its x_j pairs from shared memory. Columns (l, l+32) and (l+64, l+96) form the
// two column pairs; B rows come as 128-bit loads of four rows each, and a pack
// takes the same row from two of them.
template <int P, bool TRUNC>
struct PairMathF32Cols {
    using X = float;
    using S = float;
    using Part = float;
    static constexpr int kFoldUnits = 4;  // per half: 16 r^2 terms and 8 factors of 1/Phi per unit
    static constexpr bool kXJEveryUnit = true;
    __device__ static void prologue(const PairArgs&) {}  // no shared tables
    static constexpr int kMinCtas = 0;  // pair_min_ctas_of decides
    static constexpr bool kEarlyRelease = false;  // reads its operands from the stage during the math
    struct Cols {
        f2 acc[2][P];  // column sums of columns (l + 64 cp, l + 64 cp + 32)
    };
    using Sums = typename PairMathF32<P, TRUNC>::Sums;
    PairConstsF32 k;

    __device__ explicit PairMathF32Cols(const PairArgs& a)
        : k{pk(-1.f, -1.f),     pk(a.k_e, a.k_e),   pk(a.log2_k2, a.log2_k2), pk(-a.tp0, -a.tp0), pk(-a.tp1, -a.tp1),
            pk(-a.tp2, -a.tp2), pk(a.ts0, a.ts0), pk(a.ts1, a.ts1),         pk(a.ts2, a.ts2)} {}

    __device__ static void init(Sums& s) { PairMathF32<P, TRUNC>::init(s); }
    __device__ static void begin_block(Cols& cols, const X*, int) {
#pragma unroll
        for (int cp = 0; cp < 2; ++cp)
#pragma unroll
            for (int q = 0; q < P; ++q) cols.acc[cp][q] = pk(0.f, 0.f);
    }
    template <bool MASKED>
    __device__ void unit(const S* sA, const S* sB, const X* sXI, Cols& cols, Sums& s, int i0, int j0, int n,
                         int lane, int warp, Part (&v)[4 * P]) const {
        // B rows l + 32 c, chunk w (rows 4w .. 4w+3 of the chunk), 128-byte swizzle
        const float* sBl = sB + lane * kPairRows + ((warp ^ (lane & 7)) << 2);
        float4 b[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) b[c] = *reinterpret_cast<const float4*>(sBl + c * (32 * kPairRows));
        f2 prodm = pk(1.f, 1.f);
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            f2 xi[P], racc[P];
#pragma unroll
            for (int q = 0; q < P; ++q) {
                const float x = sXI[q * kPairRows + 4 * warp + r];
                xi[q] = pk(x, x);
                racc[q] = pk(0.f, 0.f);
            }
            const int i = i0 + r;
#pragma unroll
            for (int cp = 0; cp < 2; ++cp) {
                // this unit's x_J follows x_I in the stage
                const float* sXJ = sXI + (P + 1) * kPairRows;
                f2 nxj[P];
#pragma unroll
                for (int q = 0; q < P; ++q)
                    nxj[q] = pk(-sXJ[q * kPairCols + lane + 64 * cp], -sXJ[q * kPairCols + lane + 64 * cp + 32]);
                const float a0 = sA[(4 * warp + r) * kPairCols + lane + 64 * cp];
                const float a1 = sA[(4 * warp + r) * kPairCols + lane + 64 * cp + 32];
                const float4& b0 = b[2 * cp];
                const float4& b1 = b[2 * cp + 1];
                const float d0 = r == 0 ? b0.x : r == 1 ? b0.y : r == 2 ? b0.z : b0.w;
                const float d1 = r == 0 ? b1.x : r == 1 ? b1.y : r == 2 ? b1.z : b1.w;
                bool vA0 = true, vA1 = true, vB0 = true, vB1 = true;
                if (MASKED) {
                    const int j = j0 + lane + 64 * cp;
                    const bool ok0 = (i < n) && (j < n) && (i > j);
                    const bool ok1 = (i < n) && (j + 32 < n) && (i > j + 32);
                    vA0 = ok0 && (a0 == a0);
                    vA1 = ok1 && (a1 == a1);
                    vB0 = ok0 && (d0 == d0);
                    vB1 = ok1 && (d1 == d1);
                }
                pair_pack<P, TRUNC, MASKED>(xi, nxj, pk(a0, a1), pk(d0, d1), vA0, vA1, vB0, vB1, k, racc,
                                            cols.acc[cp], s.r2, s.prod, prodm);
            }
#pragma unroll
            for (int q = 0; q < P; ++q) v[r * P + q] = sum2(racc[q]);
        }
        if (MASKED && TRUNC) {
            float m0, m1;
            upk(prodm, m0, m1);
            s.l1 += lg2_approx(m0) + lg2_approx(m1);  // <= 16 factors in [1, 2] per half
        }
    }
    __device__ static void after_unit(Sums& s) { PairMathF32<P, TRUNC>::after_unit(s); }
    __device__ static Part col_value(const Cols& cols, int c, int q) {
        float lo, hi;
        upk(cols.acc[c >> 1][q], lo, hi);
        return (c & 1) ? hi : lo;
    }
    __device__ static void result(Sums& s, double& r2, double& lsum) { PairMathF32<P, TRUNC>::result(s, r2, lsum); }
};

// The FP32 policy for P.
#ifndef MDSX_PAIR_ROWPACK_MAX_P
#define MDSX_PAIR_ROWPACK_MAX_P 6  // FP32: packs of two rows up to this P, packs of two columns above
#endif
template <int P, bool TRUNC>
using PairMathF32For =
    typename std::conditional<(P <= MDSX_PAIR_ROWPACK_MAX_P), PairMathF32<P, TRUNC>, PairMathF32Cols<P, TRUNC>>::type;

// ------------------------------------------------------------ FP64 pair math

// One unordered pair {i, j} in FP64 (rsqrt_f64; log Phi and phi / Phi from
// the Taylor table of normal_f64), both directions: dA = delta_ij, dB = delta_ji.
// With c = [(delta - d) - phi(z) / (Phi(z) sqrt(tau))] / d the (i, j) term
// -c_A (x_i - x_j) accumulates into racc and the (j, i) term -c_B (x_i - x_j)
// into cacc (signs as in the FP32 policy). Fast path: log Phi adds into lf once
// and counts for both directions; masked path: each valid direction into lm.
template <int P, bool TRUNC, bool MASKED>
__device__ __forceinline__ void pair_f64_sym(const double (&xi)[P], const double (&xj)[P], double dA, double dB,
                                             bool vA, bool vB, double sqrt_tau, double inv_sqrt_tau,
                                             const double* tab, double (&racc)[P], double (&cacc)[P], double& r2,
                                             double& lf, double& lm) {
    double dx[P];
#pragma unroll
    for (int q = 0; q < P; ++q) dx[q] = xi[q] - xj[q];
    double d2 = dx[0] * dx[0];
#pragma unroll
    for (int q = 1; q < P; ++q) d2 = fma(dx[q], dx[q], d2);
    if (MASKED && !(vA || vB)) return;
    const double rs = rsqrt_f64(d2);
    // coincident points (d2 = 0, i != j): d = 0 as the reference's sqrt gives, so the
    // likelihood term is finite; rs = NaN makes their gradient terms NaN, as the reference's
    const double d = d2 >= kMinNormalF64 ? d2 * rs : 0.0;
    const double resA = dA - d, resB = dB - d;
    if (!MASKED || vA) r2 = fma(resA, resA, r2);
    if (!MASKED || vB) r2 = fma(resB, resB, r2);
    double t = 0.0;
    if (TRUNC) {
        double lc, ratio;
        normal_f64(d * sqrt_tau, tab, lc, ratio);
        if (MASKED) {
            if (vA) lm += lc;
            if (vB) lm += lc;
        } else {
            lf += lc;
        }
        t = ratio * rs * inv_sqrt_tau;
    }
    if (!MASKED || vA) {
        const double nc = fma(-resA, rs, t);
#pragma unroll
        for (int q = 0; q < P; ++q) racc[q] = fma(nc, dx[q], racc[q]);
    }
    if (!MASKED || vB) {
        const double nc = fma(-resB, rs, t);
#pragma unroll
        for (int q = 0; q < P; ++q) cacc[q] = fma(nc, dx[q], cacc[q]);
    }
}

// delta_ji for row 4w + r of the chunk and column j = lane + 32c of the block,
// from B's 128-byte-swizzled boxes of 128 / sizeof(S) columns (4- or 8-byte
// elements).
template <typename S>
__device__ __forceinline__ S pair_b_value(const S* sB, int lane, int warp, int c, int r) {
    constexpr int kBoxCols = 128 / (int)sizeof(S);     // 32 (4-byte) or 16 (8-byte)
    constexpr int kChunkElems = 16 / (int)sizeof(S);   // 4 or 2
    const int col = 4 * warp + r;                      // column of B = row of the chunk
    const int box = col / kBoxCols, within = col - box * kBoxCols;
    const int jj = lane + 32 * c;                      // row of B
    const int chunk = (within / kChunkElems) ^ (jj & 7);
    return sB[(box * kPairCols + jj) * kBoxCols + chunk * kChunkElems + within % kChunkElems];
}

// FP64 policy: scalar FP64 pairs over FP32- or FP64-stored delta and FP64 locations;
// FP64 partials; log Phi summed per lane. With truncation each CTA copies the
// FP64 normal-tail table (normal_f64_table) into shared memory first.
template <int P, bool TRUNC, typename DeltaT>
struct PairMathF64 {
    using X = double;
    using S = DeltaT;  // float (DELTA_F32 mode) or double (FP64 mode)
    using Part = double;
    static constexpr bool kXJEveryUnit = false;
    static constexpr int kMinCtas = 0;  // pair_min_ctas_of decides
    static constexpr bool kEarlyRelease = false;  // bound by the FP64 pipe: reads its operands from the stage
    struct Cols {
        double xj[4][P];
        double acc[4][P];
    };
    struct Sums {
        double r2;
        double lf;  // log Phi over the fast path's unordered pairs (counted for both directions)
        double lm;  // log Phi over the masked path's valid ordered pairs
    };
    double sqrt_tau, inv_sqrt_tau;

    __device__ explicit PairMathF64(const PairArgs& a) : sqrt_tau(a.sqrt_tau), inv_sqrt_tau(1.0 / a.sqrt_tau) {}

    __device__ static double* table() {
        __shared__ __align__(16) double tab[TRUNC ? kNormalF64Doubles : 2];
        return tab;
    }
    // Every thread of the CTA takes part; the kernel synchronises after it.
    __device__ static void prologue(const PairArgs& a) {
        if (!TRUNC) return;
        const double2* src = reinterpret_cast<const double2*>(a.normal_table_f64);
        double2* dst = reinterpret_cast<double2*>(table());
        for (int k = threadIdx.x; k < kNormalF64Doubles / 2; k += blockDim.x) dst[k] = __ldg(&src[k]);
    }

    __device__ static void init(Sums& s) { s.r2 = s.lf = s.lm = 0.0; }
    __device__ static void begin_block(Cols& cols, const X* sXJ, int lane) {
#pragma unroll
        for (int c = 0; c < 4; ++c)
#pragma unroll
            for (int q = 0; q < P; ++q) {
                cols.xj[c][q] = sXJ[q * kPairCols + lane + 32 * c];
                cols.acc[c][q] = 0.0;
            }
    }
    // One unit, row by row (one row's x_i and sums live at a time).
    template <bool MASKED>
    __device__ void unit(const S* sA, const S* sB, const X* sXI, Cols& cols, Sums& s, int i0, int j0, int n,
                         int lane, int warp, Part (&v)[4 * P]) const {
        const double* tab = table();
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            double xi[P], racc[P];
#pragma unroll
            for (int q = 0; q < P; ++q) {
                xi[q] = sXI[q * kPairRows + 4 * warp + r];
                racc[q] = 0.0;
            }
            const int i = i0 + r;
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const int j = j0 + lane + 32 * c;
                const S a = sA[(4 * warp + r) * kPairCols + lane + 32 * c];
                const S bb = pair_b_value(sB, lane, warp, c, r);
                bool vA = true, vB = true;
                if (MASKED) {
                    const bool ok = (i < n) && (j < n) && (i > j);
                    vA = ok && (a == a);
                    vB = ok && (bb == bb);
                }
                pair_f64_sym<P, TRUNC, MASKED>(xi, cols.xj[c], (double)a, (double)bb, vA, vB, sqrt_tau,
                                               inv_sqrt_tau, tab, racc, cols.acc[c], s.r2, s.lf, s.lm);
            }
#pragma unroll
            for (int q = 0; q < P; ++q) v[r * P + q] = racc[q];
        }
    }
    __device__ static void after_unit(Sums&) {}
    __device__ static Part col_value(const Cols& cols, int c, int q) { return cols.acc[c][q]; }
    __device__ static void result(Sums& s, double& r2, double& lsum) {
        r2 = s.r2;
        lsum = TRUNC ? 2.0 * s.lf + s.lm : 0.0;
    }
};

// One unordered pair {i, j} in double-float arithmetic (pair_f64_sym's steps):
// likelihood terms of (i, j) (delta_ij = dA) and (j, i) (delta_ji = dB), the
// row sums of row i and the column sums of column j.
template <int P, bool TRUNC, bool MASKED>
__device__ __forceinline__ void pair_dd_sym(const dd (&xi)[P], const dd (&xj)[P], dd dA, dd dB, bool vA, bool vB,
                                            dd sqrt_tau, dd inv_sqrt_tau, const float* tab, dd (&racc)[P],
                                            dd (&cacc)[P], dd& r2, dd& lf, dd& lm) {
    dd dx[P];
#pragma unroll
    for (int q = 0; q < P; ++q) dx[q] = dd_sub(xi[q], xj[q]);  // normalised: products drop lo * lo
    dd d2 = dd_of(0.0f);
#pragma unroll
    for (int q = 0; q < P; ++q) dd_acc_sqr(d2, dx[q]);
    d2 = fast_two_sum(d2.hi, d2.lo);
    if (MASKED && !(vA || vB)) return;
    const dd rs = dd_rsqrt(d2);
    // coincident points: d = 0 and a NaN gradient term, as in pair_f64_sym
    const dd d = d2.hi >= 1.17549435e-38f ? dd_mul(d2, rs) : dd_of(0.0f);
    const dd resA = dd_sub(dA, d), resB = dd_sub(dB, d);
    if (!MASKED || vA) dd_acc_sqr(r2, resA);
    if (!MASKED || vB) dd_acc_sqr(r2, resB);
    dd t = dd_of(0.0f);
    if (TRUNC) {
        // log Phi(z) straight into the likelihood sums (the fast path counts it
        // once for both directions) and phi / Phi for the gradient term
        dd lc, ratio;
        normal_dd(dd_mul(d, sqrt_tau), tab, lc, ratio);
        if (MASKED) {
            if (vA) dd_acc_add(lm, lc);
            if (vB) dd_acc_add(lm, lc);
        } else {
            dd_acc_add(lf, lc);
        }
        t = dd_mul(dd_mul(ratio, rs), inv_sqrt_tau);
    }
    if (!MASKED || vA) {
        const dd nc = dd_sub(t, dd_mul(resA, rs));
#pragma unroll
        for (int q = 0; q < P; ++q) dd_acc_fma(racc[q], nc, dx[q]);
    }
    if (!MASKED || vB) {
        const dd nc = dd_sub(t, dd_mul(resB, rs));
#pragma unroll
        for (int q = 0; q < P; ++q) dd_acc_fma(cacc[q], nc, dx[q]);
    }
}

// Double-float policy: the FP64 modes' accuracy from the FP32 pipes. Locations
// arrive as (hi, lo) float pairs in 8-byte slots; delta as FP32 (DeltaT =
// float) or as (hi, lo) pairs in 8-byte slots (DeltaT = double). FP64 partials,
// as the FP64 policy. With truncation each CTA copies the normal tail table
// into shared memory first.
template <int P, bool TRUNC, typename DeltaT>
struct PairMathDD {
    using X = double;
    using S = DeltaT;
    using Part = double;
    static constexpr bool kXJEveryUnit = false;
    static constexpr bool kEarlyRelease = false;
#ifndef MDSX_DD_TWO_CTAS_MAX_P
#define MDSX_DD_TWO_CTAS_MAX_P 3  // FP32-stored delta: compiled for two CTAs per SM up to this P
#endif
    // Two CTAs per SM (128 registers) over FP32-stored delta, where two fit in
    // shared memory; measured on GB300: P = 2 3.72 -> 3.04 ms (no spills), P = 3
    // 4.28 -> 3.95 ms (200 bytes spilled) at N = 20 000. FP64-stored delta fits
    // one CTA per SM, which keeps up to 255 registers (P = 3 at 128: +21 %).
    static constexpr int kMinCtas = sizeof(DeltaT) == 4 && P <= MDSX_DD_TWO_CTAS_MAX_P ? 2 : 1;
    struct Cols {
        dd xj[4][P];
        dd acc[4][P];
    };
    struct Sums {
        dd r2;
        dd lf;  // log Phi over the fast path's unordered pairs (counted for both directions)
        dd lm;  // log Phi over the masked path's valid ordered pairs
    };
    dd sqrt_tau, inv_sqrt_tau;

    __device__ explicit PairMathDD(const PairArgs& a)
        : sqrt_tau(dd_from_double(a.sqrt_tau)), inv_sqrt_tau(dd_from_double(1.0 / a.sqrt_tau)) {}

    __device__ static float* table() {
        __shared__ __align__(16) float tab[TRUNC ? kNormalDDFloats : 4];
        return tab;
    }
    // Every thread of the CTA takes part; the kernel synchronises after it.
    __device__ static void prologue(const PairArgs& a) {
        if (!TRUNC) return;
        const float4* src = reinterpret_cast<const float4*>(a.normal_table);
        float4* dst = reinterpret_cast<float4*>(table());
        for (int k = threadIdx.x; k < kNormalDDFloats / 4; k += blockDim.x) dst[k] = __ldg(&src[k]);
    }
    // an 8-byte slot holding (hi, lo) as two floats, low word first
    __device__ static dd slot(double v) {
        const unsigned long long b = (unsigned long long)__double_as_longlong(v);
        return dd_of(__int_as_float((int)(unsigned)(b & 0xffffffffull)), __int_as_float((int)(unsigned)(b >> 32)));
    }
    __device__ static dd delta(float v) { return dd_of(v); }
    __device__ static dd delta(double v) { return slot(v); }

    __device__ static void init(Sums& s) { s.r2 = s.lf = s.lm = dd_of(0.0f); }
    __device__ static void begin_block(Cols& cols, const X* sXJ, int lane) {
#pragma unroll
        for (int c = 0; c < 4; ++c)
#pragma unroll
            for (int q = 0; q < P; ++q) {
                cols.xj[c][q] = slot(sXJ[q * kPairCols + lane + 32 * c]);
                cols.acc[c][q] = dd_of(0.0f);
            }
    }
    template <bool MASKED>
    __device__ void unit(const S* sA, const S* sB, const X* sXI, Cols& cols, Sums& s, int i0, int j0, int n,
                         int lane, int warp, Part (&v)[4 * P]) const {
        const float* tab = table();
#pragma unroll
        for (int k = 0; k < 4 * P; ++k) v[k] = 0.0;
        // Rows one at a time in a loop that is not unrolled (the four column
        // slots are): an unrolled unit is ~16 x 450 instructions and misses in
        // the instruction cache. The row sums rotate through v, so that every
        // register index stays a constant.
#pragma unroll 1
        for (int r = 0; r < 4; ++r) {
            dd xi[P], racc[P];
#pragma unroll
            for (int q = 0; q < P; ++q) {
                xi[q] = slot(sXI[q * kPairRows + 4 * warp + r]);
                racc[q] = dd_of(0.0f);
            }
            const int i = i0 + r;
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const int j = j0 + lane + 32 * c;
                const dd a = delta(sA[(4 * warp + r) * kPairCols + lane + 32 * c]);
                const dd bb = delta(pair_b_value(sB, lane, warp, c, r));
                bool vA = true, vB = true;
                if (MASKED) {
                    const bool ok = (i < n) && (j < n) && (i > j);
                    vA = ok && (a.hi == a.hi);
                    vB = ok && (bb.hi == bb.hi);
                }
                pair_dd_sym<P, TRUNC, MASKED>(xi, cols.xj[c], a, bb, vA, vB, sqrt_tau, inv_sqrt_tau, tab, racc,
                                              cols.acc[c], s.r2, s.lf, s.lm);
            }
#pragma unroll
            for (int k = 0; k < 3 * P; ++k) v[k] = v[k + P];
#pragma unroll
            for (int q = 0; q < P; ++q) v[3 * P + q] = dd_to_double(racc[q]);
        }
        // the long-lived accumulators: renormalised once per unit (dd_acc_fma)
        s.r2 = dd_renorm(s.r2);
        if (TRUNC) {
            s.lf = dd_renorm(s.lf);
            s.lm = dd_renorm(s.lm);
        }
#pragma unroll
        for (int c = 0; c < 4; ++c)
#pragma unroll
            for (int q = 0; q < P; ++q) cols.acc[c][q] = dd_renorm(cols.acc[c][q]);
    }
    __device__ static void after_unit(Sums&) {}
    __device__ static Part col_value(const Cols& cols, int c, int q) { return dd_to_double(cols.acc[c][q]); }
    __device__ static void result(Sums& s, double& r2, double& lsum) {
        r2 = dd_to_double(s.r2);
        lsum = TRUNC ? 2.0 * dd_to_double(s.lf) + dd_to_double(s.lm) : 0.0;
    }
};

// Sums each of the KV values over the warp's lanes and stores total i at
// out[i]: one transpose-reduce for KV <= 16, else chunks of 8 (fewer live
// registers than one reduce padded to 32 values).
template <int KV, typename T>
__device__ __forceinline__ void flush_row_sums(T (&v)[KV], T* out, int lane) {
    constexpr int CH = KV <= 16 ? KV : 8;
#pragma unroll
    for (int c0 = 0; c0 < KV; c0 += CH) {
        T w[CH];
#pragma unroll
        for (int i = 0; i < CH; ++i) w[i] = c0 + i < KV ? v[c0 + i] : T(0);
        using TS = TransposeShape<CH>;
        warp_transpose_reduce<CH>(w, lane);
        const int idx = lane >> TS::kLaneShift;
        if ((lane & ((1 << TS::kLaneShift) - 1)) == 0 && idx < CH && c0 + idx < KV) out[c0 + idx] = w[0];
    }
}

// One unit of the consumer loop (shared by pair_kernel and batch_pair_kernel):
// waits (bounded) for the unit's stage, takes x_J and the column flags when the
// unit starts a column block, runs the math policy on the masked or fast path,
// releases the stage and writes the unit's row sums to `rowpart_unit` (the
// unit's [32][P] rows). Returns false if the wait gave up.
template <int P, class M, class Shape>
__device__ __forceinline__ bool pair_consume_unit(const M& math, typename M::Sums& sums, typename M::Cols& cols,
                                                  bool& j_masked, bool block_start, const unsigned char* smem,
                                                  uint64_t* full, uint64_t* empty, int k, int I, int J, int n,
                                                  int lane, int warp, int* err, typename M::Part* rowpart_unit) {
    using X = typename M::X;
    using DS = typename M::S;
    constexpr int S = Shape::kStages;
    const int stage = k % S;
    if (!mbar_wait_bounded(&full[stage], (uint32_t)(k / S) & 1u, err, kDevTimeoutFull)) return false;
    const unsigned char* st = smem + stage * Shape::kStageBytes;
    const DS* sB = reinterpret_cast<const DS*>(st);
    const DS* sA = reinterpret_cast<const DS*>(st + Shape::kBBytes);
    const X* sXI = reinterpret_cast<const X*>(st + Shape::kXIOffset);
    if (block_start) {
        // x_J arrived with this unit: the block's x_j and its column flags
        const X* sXJ = reinterpret_cast<const X*>(st + Shape::kXJOffset);
        M::begin_block(cols, sXJ, lane);
        bool bad = false;
#pragma unroll
        for (int c = 0; c < 4; ++c) bad |= sXJ[P * kPairCols + lane + 32 * c] != X(0);
        j_masked = __any_sync(0xffffffffu, bad);
    }
    const X* fl = sXI + P * kPairRows + 4 * warp;
    const bool masked = j_masked || (I < 4 * J + 4) || fl[0] != X(0) || fl[1] != X(0) || fl[2] != X(0) || fl[3] != X(0);
    const int i0 = I * kPairRows + 4 * warp;
    const int j0 = J * kPairCols;
    typename M::Part v[4 * P];
    if constexpr (M::kEarlyRelease) {
        typename M::Operands o;
        M::load(o, sA, sB, sXI, lane, warp);
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[stage]);
        if (masked)
            math.template compute<true>(o, cols, sums, i0, j0, n, lane, v);
        else
            math.template compute<false>(o, cols, sums, i0, j0, n, lane, v);
    } else {
        if (masked)
            math.template unit<true>(sA, sB, sXI, cols, sums, i0, j0, n, lane, warp, v);
        else
            math.template unit<false>(sA, sB, sXI, cols, sums, i0, j0, n, lane, warp, v);
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[stage]);
    }
    // row sums of this unit: rows 4w .. 4w+3, value index r * P + q
    flush_row_sums<4 * P>(v, rowpart_unit + (size_t)(4 * warp) * P, lane);
    M::after_unit(sums);
    return true;
}

// Column sums of one column block from this warp: colpart_block = the block's
// [slots][8 warps][P][128] partials, slot = this CTA's slot of the block.
template <int P, class M>
__device__ __forceinline__ void pair_flush_cols(const typename M::Cols& cols, typename M::Part* colpart_block,
                                                int slot, int warp, int lane) {
#pragma unroll
    for (int q = 0; q < P; ++q)
#pragma unroll
        for (int c = 0; c < 4; ++c)
            colpart_block[((size_t)slot * kPairWarps + warp) * (P * kPairCols) + q * kPairCols + lane + 32 * c] =
                M::col_value(cols, c, q);
}

// This warp's likelihood sums (r^2, log Phi) reduced over its lanes, written by lane 0 at lpart_entry[0..1].
template <class M>
__device__ __forceinline__ void pair_flush_likelihood(typename M::Sums& sums, double* lpart_entry, int lane) {
    double r2_sum, lsum;
    M::result(sums, r2_sum, lsum);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        r2_sum += __shfl_xor_sync(0xffffffffu, r2_sum, off);
        lsum += __shfl_xor_sync(0xffffffffu, lsum, off);
    }
    if (lane == 0) {
        lpart_entry[0] = r2_sum;
        lpart_entry[1] = lsum;
    }
}

// --------------------------------------------------------------- the kernel

// CTAs per SM the kernel is compiled for: two at 128 registers, or one with up
// to 255 where 128 spills. Measured at N = 20 000 (FP32, truncated; two / one):
// P = 3 0.336 / 0.385 ms, P = 4 0.429 / 0.400, P = 5 0.423 / 0.449, P = 6 0.77 / 0.49.
template <int P>
constexpr int pair_min_ctas() {
    return (P >= 4 && P <= MDSX_PAIR_ROWPACK_MAX_P) || P == 6 ? 1 : MDSX_PAIR_F32_CTAS;
}

// FP64 pair math runs one CTA per SM at up to 255 registers: the FP64 pipe bounds
// it, so two warps per scheduler keep the pipe busy, and at 128 registers P <= 3
// spill 400-700 bytes (same time at N = 1000 and 20 000, one CTA slightly ahead).
template <int P, class M>
constexpr int pair_min_ctas_of() {
    return M::kMinCtas > 0 ? M::kMinCtas : std::is_same<typename M::Part, double>::value ? 1 : pair_min_ctas<P>();
}

template <int P, bool TRUNC, class M>
__global__ void __launch_bounds__(kPairThreads, pair_min_ctas_of<P, M>())
    pair_kernel(const __grid_constant__ CUtensorMap tmap_a, const __grid_constant__ CUtensorMap tmap_b,
                const __grid_constant__ CUtensorMap tmap_xi, const __grid_constant__ CUtensorMap tmap_xj,
                const PairArgs a) {
    using X = typename M::X;
    using DS = typename M::S;
    using Part = typename M::Part;
    using Shape = PairShape<P, (int)sizeof(X), (int)sizeof(DS)>;
    constexpr int S = Shape::kStages;
    extern __shared__ unsigned char smem_raw[];
    unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                                           ~uintptr_t(1023));
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + S * Shape::kStageBytes);
    uint64_t* empty = full + S;

    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const long long u_begin = a.cta_begin[blockIdx.x];
    const long long u_end = a.cta_begin[blockIdx.x + 1];
    const int K = (int)(u_end - u_begin);  // >= 1: the host keeps every range non-empty
    const int J_first = pair_block_of_unit(u_begin, a.nb, a.nc);

    if (threadIdx.x == 0) {
        for (int s = 0; s < S; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], kPairWarps);
        }
        fence_mbar_init();
        prefetch_tensormap(&tmap_a);
        prefetch_tensormap(&tmap_b);
        prefetch_tensormap(&tmap_xi);
        prefetch_tensormap(&tmap_xj);
    }
    M::prologue(a);
    __syncthreads();

    // Copy issue state, kept by lane 0 of every warp: next unit and its (J, I).
    // Unit m is issued by warp m % 8 (MDSX_PAIR_ROTATE_ISSUER; else warp 0
    // issues all), so the copy-issue work does not lengthen one warp's path.
    // Deadlock-free: the slowest warp's next unit k was issued by a warp that
    // has passed step k - S + 1, and its stage was released by every warp.
    const bool issuer = MDSX_PAIR_ROTATE_ISSUER ? lane == 0 : threadIdx.x == 0;
    int issued = 0;
    int pJ = J_first;
    int pI = 4 * J_first + (int)(u_begin - pair_units_before(J_first, a.nc));
    int pJ_loaded = -1;
    bool issue_ok = true;
    const uint64_t evict_first = l2_evict_first_policy();
    // Issues units up to k + S - 1: unit m reuses the stage of unit m - S. The
    // stage of m <= k + S - 2 was released before unit k - 1 began (bounded
    // wait); the stage of k + S - 1 is taken only if already free, else it is
    // issued before the next unit.
    auto top_up = [&](int k) {
        while (issue_ok && issued < K && issued <= k + S - 1) {
            const int m = issued;
            const bool mine = !MDSX_PAIR_ROTATE_ISSUER || m % kPairWarps == warp;
            const int stage = m % S;
            if (mine && m >= S) {
                const uint32_t par = ((uint32_t)(m / S) & 1u) ^ 1u;
                if (m <= k + S - 2) {
                    if (!mbar_wait_bounded(&empty[stage], par, a.err, kDevTimeoutEmpty)) {
                        issue_ok = false;
                        break;
                    }
                } else if (!mbar_try_wait(&empty[stage], par)) {
                    break;
                }
            }
            const bool new_j = M::kXJEveryUnit || pJ != pJ_loaded;
            if (mine) {
                unsigned char* st = smem + stage * Shape::kStageBytes;
                const uint32_t bytes =
                    Shape::kBBytes + Shape::kABytes + Shape::kXIBytes + (new_j ? Shape::kXJBytes : 0);
                mbar_arrive_expect_tx(&full[stage], bytes);
                // delta is read once: evict it first, keeping the partials in L2 for the finish kernel
#pragma unroll
                for (int bx = 0; bx < Shape::kBBoxes; ++bx)
                    tma_load_2d_hint(st + bx * (Shape::kBBytes / Shape::kBBoxes), &tmap_b,
                                     pI * kPairRows + bx * Shape::kBBoxCols, pJ * kPairCols, &full[stage],
                                     evict_first);
                tma_load_2d_hint(st + Shape::kBBytes, &tmap_a, pJ * kPairCols, pI * kPairRows, &full[stage],
                                 evict_first);
                tma_load_2d(st + Shape::kXIOffset, &tmap_xi, pI * kPairRows, 0, &full[stage]);
                if (new_j) tma_load_2d(st + Shape::kXJOffset, &tmap_xj, pJ * kPairCols, 0, &full[stage]);
            }
            pJ_loaded = pJ;
            if (++pI == a.nc) {
                ++pJ;
                pI = 4 * pJ;
            }
            ++issued;
        }
    };

    const M math(a);
    Part* rowpart = static_cast<Part*>(a.rowpart);
    Part* colpart = static_cast<Part*>(a.colpart);

    typename M::Sums sums;
    M::init(sums);
    bool alive = true;
    int k = 0;
    for (int J = J_first; k < K && alive; ++J) {
        const long long before = pair_units_before(J, a.nc);
        const long long j_end = before + (a.nc - 4 * J);
        const int k_end = (int)((u_end < j_end ? u_end : j_end) - u_begin);
        const int slot = (int)blockIdx.x - a.j_first_cta[J];
        int I = 4 * J + (int)(u_begin + k - before);
        typename M::Cols cols;
        bool j_masked = false;
        for (const int k_first = k; k < k_end; ++k, ++I) {
            if (issuer) top_up(k);
            if (!pair_consume_unit<P, M, Shape>(math, sums, cols, j_masked, k == k_first, smem, full, empty, k, I, J,
                                                a.n, lane, warp, a.err,
                                                rowpart + (size_t)(u_begin + k) * kPairRows * P)) {
                alive = false;
                break;
            }
        }
        if (!alive) break;
        pair_flush_cols<P, M>(cols, colpart + (size_t)J * a.max_slots * kPairWarps * (P * kPairCols), slot, warp,
                              lane);
    }

    // The finish kernel may be scheduled now; it waits for this grid to complete.
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    if (issuer) {
        // Copies still in flight (only after a failed wait): let this warp's land before the CTA exits.
        for (int m = k; m < issued; ++m)
            if (!MDSX_PAIR_ROTATE_ISSUER || m % kPairWarps == warp)
                mbar_wait_time_only(&full[m % S], (uint32_t)(m / S) & 1u);
    }
    if (!alive) return;

    pair_flush_likelihood<M>(sums, a.lpart + ((size_t)blockIdx.x * kPairWarps + warp) * 2, lane);
}

// Sum of K values (K a power of two) as a fixed pairwise tree in their own
// type: FP32 partials are added in FP32, as GB300 issues few FP64 operations
// per clock. Compile-time levels keep the array in registers.
template <int W>
struct TreeLevel {
    template <typename T, int K>
    __device__ __forceinline__ static void fold(T (&v)[K]) {
#pragma unroll
        for (int k = 0; k < W; ++k) v[k] += v[k + W];
        TreeLevel<W / 2>::fold(v);
    }
};
template <>
struct TreeLevel<0> {
    template <typename T, int K>
    __device__ __forceinline__ static void fold(T (&)[K]) {}
};
template <int K, typename T>
__device__ __forceinline__ T tree_sum(T (&v)[K]) {
    static_assert((K & (K - 1)) == 0, "K must be a power of two");
    TreeLevel<K / 2>::fold(v);
    return v[0];
}

template <int P, typename Part>
struct FinishShape {
    // FP32 partials: small blocks. That finish is latency-bound (a few dependent
    // rounds of partial loads per block), so more resident blocks beat more
    // threads per block. Measured on GB300 (FP32, truncated) against 512 threads
    // for every P: the 64-instance batch 1.428 -> 1.339 ms, N = 20 000 evaluation
    // -0.5 % (P = 2) and -0.8 % (P = 6). FP64 partials: 512 threads, as the
    // blocks of the first column blocks are bound by FP64 adds (N = 1000, P = 2:
    // 9.2 us against 12.3 us with 128 threads).
    static constexpr int kThreads = sizeof(Part) == 8             ? MDSX_FINISH_THREADS_F64
                                    : P <= MDSX_FINISH_SMALL_P ? MDSX_FINISH_THREADS_SMALL_P
                                                               : MDSX_FINISH_THREADS;
    // FP64 partials: each row chunk is split over kSplit blocks of kRows rows, so
    // that the FP64 adds of a chunk's column partials spread over kSplit SMs.
    static constexpr int kSplit = sizeof(Part) == 8 ? MDSX_FINISH_SPLIT_F64 : 1;
    static constexpr int kRows = kPairRows / kSplit;  // rows per block
    static constexpr int kOut = kRows * P;            // outputs per block
    static constexpr int kGroups = kThreads / kOut;   // FP32: P = 1: 4, 2: 2, 3: 2, 4: 2, 5: 1, 6: 1
    static_assert(kGroups >= 1, "a finish block must hold one row chunk's outputs");
    static constexpr int kChunk = MDSX_FINISH_CHUNK;         // row-partial loads in flight per thread
    static constexpr int kColChunk = MDSX_FINISH_COL_CHUNK;  // column-partial loads in flight per thread
};

// Finish blocks of one sweep: the likelihood block and kSplit per row chunk.
template <int P, typename Part>
__host__ __device__ constexpr int pair_finish_blocks(int nc) {
    return 1 + nc * FinishShape<P, Part>::kSplit;
}

// Block `blk` of the finish of one sweep (block 0: likelihood; blocks
// 1 + (nc - 1 - I) * kSplit + h: rows h * kRows .. of row chunk I).
template <int P, typename Part>
__device__ __forceinline__ void pair_finish_block(const PairArgs& a, int blk) {
    using FS = FinishShape<P, Part>;
    const Part* rowpart = static_cast<const Part*>(a.rowpart);
    const Part* colpart = static_cast<const Part*>(a.colpart);
    __shared__ double part[2][FS::kThreads];
    const int t = threadIdx.x;
    if (blk == 0) {
        const int total = a.grid * kPairWarps;
        double s0 = 0.0, s1 = 0.0;
        for (int e0 = t; e0 < total; e0 += FS::kThreads * 8) {
            double v0[8], v1[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const int e = e0 + FS::kThreads * k;
                v0[k] = e < total ? __ldcg(&a.lpart[2 * (size_t)e]) : 0.0;
                v1[k] = e < total ? __ldcg(&a.lpart[2 * (size_t)e + 1]) : 0.0;
            }
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                s0 += v0[k];
                s1 += v1[k];
            }
        }
        part[0][t] = s0;
        part[1][t] = s1;
        __syncthreads();
        for (int o = FS::kThreads / 2; o > 0; o >>= 1) {
            if (t < o) {
                part[0][t] += part[0][t + o];
                part[1][t] += part[1][t + o];
            }
            __syncthreads();
        }
        if (t == 0) {
            const double tr2 = part[0][0], tlog = part[1][0];
            a.sums_out[0] = tr2;
            a.sums_out[1] = tlog;
            // src/NewMultiDimensionalScaling.hpp:198-202 and :554-557: halve the
            // ordered-pair total; without truncation scale by 0.5 * tau.
            a.sums_out[2] = a.truncation ? 0.5 * (0.5 * a.tau * tr2 + tlog) : 0.5 * a.tau * (0.5 * tr2);
        }
        return;
    }
    const int ci = (blk - 1) / FS::kSplit;  // the chunks with the most partials are scheduled first
    const int I = a.nc - 1 - ci;
    const int h0 = (blk - 1 - ci * FS::kSplit) * FS::kRows;  // first row of this block within the chunk
    const int g = t / FS::kOut, o = t - g * FS::kOut;        // o = r * P + q, row h0 + r of the chunk
    double acc = 0.0;
    if (g < FS::kGroups) {
        // row sums: units (J, I), J = 0 .. I/4, each [32 rows][P] contiguous
        const int j_max = I >> 2;
        for (int J0 = g; J0 <= j_max; J0 += FS::kGroups * FS::kChunk) {
            Part v[FS::kChunk];
#pragma unroll
            for (int k = 0; k < FS::kChunk; ++k) {
                const int J = J0 + FS::kGroups * k;
                const long long u = pair_units_before(J, a.nc) + (I - 4 * J);
                v[k] = J <= j_max ? __ldcg(&rowpart[(size_t)u * (kPairRows * P) + h0 * P + o]) : Part(0);
            }
            acc -= (double)tree_sum<FS::kChunk>(v);
        }
        // column sums of block J = I/4 for its rows (I % 4) * 32 + r: entries (slot, warp)
        const int J = I >> 2, r = o / P, q = o - r * P, jj = (I & 3) * kPairRows + h0 + r;
        const long long before = pair_units_before(J, a.nc);
        const int n_e = a.j_slots[J] * kPairWarps;
        for (int e0 = g; e0 < n_e; e0 += FS::kGroups * FS::kColChunk) {
            Part v[FS::kColChunk];
#pragma unroll
            for (int k = 0; k < FS::kColChunk; ++k) {
                const int e = e0 + FS::kGroups * k;  // slot e / 8, warp e % 8
                v[k] = e < n_e ? __ldcg(&colpart[((size_t)J * a.max_slots * kPairWarps + e) * (P * kPairCols) +
                                                 q * kPairCols + jj])
                               : Part(0);
            }
            acc += (double)tree_sum<FS::kColChunk>(v);
        }
    }
    part[0][t] = acc;
    __syncthreads();
    double grad_t = 0.0;
    if (t < FS::kOut) {
        double s = 0.0;
#pragma unroll
        for (int k = 0; k < FS::kGroups; ++k) s += part[0][k * FS::kOut + t];
        grad_t = a.tau * s;
        const int row = I * kPairRows + h0 + t / P;
        if (row < a.n) a.grad_out[(size_t)(I * kPairRows + h0) * P + t] = grad_t;
    }
    if (!a.leapfrog) return;
    // leapfrog for the block's rows: thread r < kRows takes row I * 32 + h0 + r
    __syncthreads();  // every thread has read part[0]
    if (t < FS::kOut) part[1][t] = grad_t;
    __syncthreads();
    const int row = I * kPairRows + h0 + t;
    if (t < FS::kRows && row < a.n) {
        const PairLeapfrog& L = a.leap;
        const double ca = L.coef[0], cb = L.coef[1];
        double xi[P], pi[P];
#pragma unroll
        for (int q = 0; q < P; ++q) {
            xi[q] = L.x[(size_t)row * P + q];
            pi[q] = L.mom[(size_t)row * P + q];
        }
#pragma unroll
        for (int q = 0; q < P; ++q) {
            double prior = 0.0;
#pragma unroll
            for (int r = 0; r < P; ++r) prior += xi[r] * L.lam[r * P + q];
            pi[q] += ca * (part[1][t * P + q] - prior);
        }
#pragma unroll
        for (int q = 0; q < P; ++q) {
            xi[q] += cb * pi[q];
            L.mom[(size_t)row * P + q] = pi[q];
            L.x[(size_t)row * P + q] = xi[q];
            if (L.soa_f32)
                static_cast<float*>(L.soa)[(size_t)q * L.x_ld + row] = (float)xi[q];
            else
                static_cast<double*>(L.soa)[(size_t)q * L.x_ld + row] = xi[q];
        }
    }
}

template <int P, typename Part>
__global__ void __launch_bounds__(FinishShape<P, Part>::kThreads) pair_finish_kernel(const PairArgs a) {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    pair_finish_block<P, Part>(a, (int)blockIdx.x);
}

}  // namespace mdsx
