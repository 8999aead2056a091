// Batched unordered-pair sweep: the pair schedule of pair_kernel.cuh over many
// independent instances of one embedding dimension P in one persistent launch
// (FP32 pair math; no counterpart in the reference, which keeps one engine per
// instance, src/jni/dr_inference_multidimensionalscaling_NativeMDSSingleton.cpp:10-20).
//
// The work list is the concatenation of every instance's units (J, I), I >= 4J
// (pair_kernel.cuh), instance k owning the global units [unit_begin_k,
// unit_begin_k + U_k). CTAs take contiguous, cost-balanced ranges of the list
// and walk them with an instance cursor; per-instance state (four tensor maps,
// the PairArgs of the instance: constants, partial buffers, column-block slot
// tables, outputs) lives in a device array of PairInstance descriptors. At an
// instance boundary the copy issuer switches tensor maps and the consumers
// flush their column and likelihood sums of the finished instance. The finish
// kernel runs pair_finish_block for every (instance, block).
#pragma once

#include <cuda.h>

#include "pair_kernel.cuh"

namespace mdsx {
namespace batch {

struct PairInstance {       // CUtensorMap members keep it 64-byte aligned (TMA requirement)
    CUtensorMap tmap_a;     // delta [N][ld] FP32, box 128 x 32
    CUtensorMap tmap_b;     // delta, box 32 x 128, 128-byte swizzle
    CUtensorMap tmap_xi;    // SoA locations + flag row [P + 1][x_ld], box 32 x (P + 1)
    CUtensorMap tmap_xj;    // the same, box 128 x (P + 1)
    PairArgs args;          // the instance: grid = CTAs meeting it, j_first_cta absolute CTA indices
    long long unit_begin;   // first global unit
    int first_cta;          // first CTA meeting the instance (likelihood slot base)
    int finish_begin;       // first block of the instance in the finish grid
};

struct BatchPairArgs {
    const PairInstance* inst;
    int count;
    const long long* cta_begin;  // [grid + 1]: global units of each CTA
    int* err;
};

// Instance holding global unit u (binary search on unit_begin).
__device__ __forceinline__ int pair_find_instance(const PairInstance* inst, int count, long long u) {
    int lo = 0, hi = count - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (inst[mid].unit_begin <= u)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

template <int P, bool TRUNC>
__global__ void __launch_bounds__(kPairThreads, pair_min_ctas<P>()) batch_pair_kernel(const BatchPairArgs ba) {
    using M = PairMathF32For<P, TRUNC>;
    using Shape = PairShape<P, 4, 4>;
    constexpr int S = Shape::kStages;
    extern __shared__ unsigned char smem_raw[];
    unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                                           ~uintptr_t(1023));
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + S * Shape::kStageBytes);
    uint64_t* empty = full + S;

    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const long long u_begin = ba.cta_begin[blockIdx.x];
    const long long u_end = ba.cta_begin[blockIdx.x + 1];
    const int K = (int)(u_end - u_begin);  // >= 1: the host keeps every range non-empty
    const int k_first_inst = pair_find_instance(ba.inst, ba.count, u_begin);

    if (threadIdx.x == 0) {
        for (int s = 0; s < S; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], kPairWarps);
        }
        fence_mbar_init();
    }
    __syncthreads();

    // Copy issue state (thread 0 only): instance, (J, I) of the next unit.
    const bool issuer = threadIdx.x == 0;
    int issued = 0;
    int pk = k_first_inst;
    int pnc = ba.inst[pk].args.nc, pnb = ba.inst[pk].args.nb;
    int pJ, pI;
    {
        const long long lu = u_begin - ba.inst[pk].unit_begin;
        pJ = pair_block_of_unit(lu, pnb, pnc);
        pI = 4 * pJ + (int)(lu - pair_units_before(pJ, pnc));
    }
    int pJ_loaded = -1;
    bool issue_ok = true;
    const uint64_t evict_first = l2_evict_first_policy();
    if (issuer) {
        prefetch_tensormap(&ba.inst[pk].tmap_a);
        prefetch_tensormap(&ba.inst[pk].tmap_b);
        prefetch_tensormap(&ba.inst[pk].tmap_xi);
        prefetch_tensormap(&ba.inst[pk].tmap_xj);
    }
    // As in pair_kernel: issue units up to k + S - 1; blocking wait for a stage
    // released before unit k - 1 began, try-only for the newest.
    auto top_up = [&](int k) {
        while (issue_ok && issued < K && issued <= k + S - 1) {
            const int m = issued;
            const int stage = m % S;
            if (m >= S) {
                const uint32_t par = ((uint32_t)(m / S) & 1u) ^ 1u;
                if (m <= k + S - 2) {
                    if (!mbar_wait_bounded(&empty[stage], par, ba.err, kDevTimeoutEmpty)) {
                        issue_ok = false;
                        break;
                    }
                } else if (!mbar_try_wait(&empty[stage], par)) {
                    break;
                }
            }
            const PairInstance& in = ba.inst[pk];
            unsigned char* st = smem + stage * Shape::kStageBytes;
            const bool new_j = M::kXJEveryUnit || pJ != pJ_loaded;
            const uint32_t bytes =
                Shape::kBBytes + Shape::kABytes + Shape::kXIBytes + (new_j ? Shape::kXJBytes : 0);
            mbar_arrive_expect_tx(&full[stage], bytes);
            tma_load_2d_hint(st, &in.tmap_b, pI * kPairRows, pJ * kPairCols, &full[stage], evict_first);
            tma_load_2d_hint(st + Shape::kBBytes, &in.tmap_a, pJ * kPairCols, pI * kPairRows, &full[stage],
                             evict_first);
            tma_load_2d(st + Shape::kXIOffset, &in.tmap_xi, pI * kPairRows, 0, &full[stage]);
            if (new_j) tma_load_2d(st + Shape::kXJOffset, &in.tmap_xj, pJ * kPairCols, 0, &full[stage]);
            pJ_loaded = pJ;
            if (++pI == pnc) {
                ++pJ;
                pI = 4 * pJ;
                if (pJ == pnb && pk + 1 < ba.count) {  // next instance
                    ++pk;
                    pnc = ba.inst[pk].args.nc;
                    pnb = ba.inst[pk].args.nb;
                    pJ = pI = 0;
                    pJ_loaded = -1;
                    prefetch_tensormap(&ba.inst[pk].tmap_a);
                    prefetch_tensormap(&ba.inst[pk].tmap_b);
                    prefetch_tensormap(&ba.inst[pk].tmap_xi);
                    prefetch_tensormap(&ba.inst[pk].tmap_xj);
                }
            }
            ++issued;
        }
    };

    bool alive = true;
    int k = 0;  // CTA-local unit index, continuous over instances (the ring's sequence)
    for (int ik = k_first_inst; k < K && alive; ++ik) {
        const PairInstance& in = ba.inst[ik];
        const PairArgs& a = in.args;
        const long long in_end = in.unit_begin + a.n_units;
        const int k_inst_end = (int)((u_end < in_end ? u_end : in_end) - u_begin);
        const M math(a);
        typename M::Sums sums;
        M::init(sums);
        float* rowpart = static_cast<float*>(a.rowpart);
        float* colpart = static_cast<float*>(a.colpart);
        const long long lu0 = u_begin + k - in.unit_begin;  // first local unit of this CTA in the instance
        for (int J = pair_block_of_unit(lu0, a.nb, a.nc); k < k_inst_end && alive; ++J) {
            const long long before = pair_units_before(J, a.nc);
            const long long j_end = in.unit_begin + before + (a.nc - 4 * J);  // global
            const int k_end = (int)((u_end < j_end ? u_end : j_end) - u_begin);
            const int slot = (int)blockIdx.x - a.j_first_cta[J];
            int I = 4 * J + (int)(u_begin + k - in.unit_begin - before);
            typename M::Cols cols;
            bool j_masked = false;
            for (const int k_first = k; k < k_end; ++k, ++I) {
                if (issuer) top_up(k);
                if (!pair_consume_unit<P, M, Shape>(math, sums, cols, j_masked, k == k_first, smem, full, empty, k, I,
                                                    J, a.n, lane, warp, ba.err,
                                                    rowpart + (size_t)(u_begin + k - in.unit_begin) * kPairRows * P)) {
                    alive = false;
                    break;
                }
            }
            if (!alive) break;
            pair_flush_cols<P, M>(cols, colpart + (size_t)J * a.max_slots * kPairWarps * (P * kPairCols), slot, warp,
                                  lane);
        }
        if (!alive) break;
        // this CTA's likelihood sums of the instance, per warp
        pair_flush_likelihood<M>(sums, a.lpart + ((size_t)(blockIdx.x - in.first_cta) * kPairWarps + warp) * 2, lane);
    }

    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    if (issuer) {
        // Copies still in flight (only after a failed wait): let them land before the CTA exits.
        for (int m = k; m < issued; ++m) mbar_wait_time_only(&full[m % S], (uint32_t)(m / S) & 1u);
    }
}

// The finish of every instance: block b belongs to the instance whose
// finish_begin is the largest <= b.
template <int P>
__global__ void __launch_bounds__(FinishShape<P, float>::kThreads) batch_pair_finish_kernel(const BatchPairArgs ba) {
    static_assert(pair_finish_blocks<P, float>(1) == 2, "the batch plans nc + 1 finish blocks per instance");
    asm volatile("griddepcontrol.wait;" ::: "memory");
    int lo = 0, hi = ba.count - 1;
    const int b = (int)blockIdx.x;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (ba.inst[mid].finish_begin <= b)
            lo = mid;
        else
            hi = mid - 1;
    }
    pair_finish_block<P, float>(ba.inst[lo].args, b - ba.inst[lo].finish_begin);
}

}  // namespace batch
}  // namespace mdsx
