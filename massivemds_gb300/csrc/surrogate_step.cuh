// Fused surrogate leapfrog step (no counterpart in the reference).
//
// One CTA owns a tile of kRows = 32 locations and, in one launch:
//   1. builds their features in shared memory: the scaled residuals
//      d(x_i, x_{l_k}) - delta_{i, l_k} to the K landmarks (computed in FP32
//      from the current positions, then rounded to BF16, so the rounding is
//      relative to the residual and not to the distance) and the standardised
//      dissimilarities delta_{i, l_k};
//   2. runs the MLP on the tensor cores (mma.sync m16n8k16 BF16 -> FP32):
//      activations stay in shared memory (two ping-pong buffers); weights are
//      streamed from L2 as pre-packed BF16 chunks of 32 input columns through
//      a kStages-deep cp.async ring shared by the whole network;
//   3. contracts the K outputs alpha_ik with the landmark directions
//      x_i - x_{l_k} into the surrogate gradient g_i (fixed-order reductions);
//   4. optionally writes g_i and/or applies the leapfrog kick and drift
//      p_i += a (g_i - x_i Lambda), x_i' = x_i + b p_i, writing x' to a second
//      location buffer (other CTAs still read the landmarks' old positions)
//      and to the sweep's SoA location buffer.
// The forward arithmetic (features, k-order of the MMAs, bias, SiLU, BF16
// rounding points) is the same as the training path in surrogate.cu, so the
// network evaluated here is the network that was trained.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "mlp_gemm.cuh"

namespace mdsx {
namespace surr {

constexpr int kRows = 32;          // locations per CTA (two m16 tiles)
constexpr int kStepWarps = 8;
constexpr int kStepThreads = kStepWarps * 32;
constexpr int kChunkK = 32;        // input columns per weight chunk
constexpr int kStages = 3;         // cp.async ring depth
constexpr int kMaxLayers = 9;      // hidden layers + output
constexpr int kMaxP = 10;

enum StepMode : int { kWriteGradient = 1, kKickDrift = 2 };

struct StepLambda {
    double m[kMaxP * kMaxP];
};

struct StepArgs {
    const double* x_in;      // N x P positions read (landmarks and own rows)
    double* x_out;           // N x P positions written (kKickDrift)
    double* mom;             // N x P momenta, updated in place (kKickDrift)
    double* g_out;           // N x P surrogate gradient (kWriteGradient)
    const double* coef;      // device {a, b} of the kick and drift
    void* soa;               // sweep location buffer [P][x_ld] (kKickDrift)
    int soa_f32, x_ld;
    int n, p, k, layers;     // layers = hidden layers; layer `layers` is the output
    int fo[kMaxLayers], fi[kMaxLayers];
    const float* bias[kMaxLayers];
    long long wofs[kMaxLayers];  // element offset of each layer's first chunk in wpack
    const __nv_bfloat16* wpack;  // chunks [fi/32][fo][32], 16-byte segments swizzled by (row >> 1) & 3
    const int* lm;               // landmark indices [K]
    const float* dland;          // delta_{i, l_k} [N][K]
    float mu, inv_sigma;         // delta-feature standardisation
    float inv_sigma_r;           // residual-feature scale
    float gscale;                // contraction scale x target scale
    int mode;
    int stage_bytes, act_ld0, act_ld1;  // ring stage size; activation row pitches (elements)
    StepLambda lam;
};

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(mlp::smem_u32(smem)), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Packed offset of weight element (row n, input column k) within its layer.
__host__ __device__ __forceinline__ long long packed_index(int n, int k, int fo) {
    const int c = k / kChunkK, kk = k % kChunkK, seg = kk >> 3;
    return (long long)c * fo * kChunkK + (long long)n * kChunkK + (((seg ^ ((n >> 1) & 3)) << 3) | (kk & 7));
}

// Features shared with the training path: the residual from the squared
// distance (float coordinates, square root rounded to nearest), and delta.
__device__ __forceinline__ __nv_bfloat16 residual_feature(float d2, float delta, float inv_sigma_r) {
    return __float2bfloat16_rn((__fsqrt_rn(d2) - delta) * inv_sigma_r);
}
__device__ __forceinline__ __nv_bfloat16 delta_feature(float delta, float mu, float inv_sigma) {
    return __float2bfloat16_rn((delta - mu) * inv_sigma);
}

// Host side (surrogate_step.cu).
size_t step_smem_bytes(const StepArgs& a);
cudaError_t launch_step(const StepArgs& a, cudaStream_t st);
cudaError_t pack_weight(const float* w, int fo, int fi, __nv_bfloat16* dst, cudaStream_t st);

}  // namespace surr
}  // namespace mdsx
