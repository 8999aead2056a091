// Fused surrogate leapfrog step kernel; see surrogate_step.cuh for the design.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "surrogate_step.cuh"

namespace mdsx {
namespace surr {

using bf16 = __nv_bfloat16;

// Two CTAs per SM while the widest layer has at most 256 outputs.
template <int TPW>  // n8 tiles per warp of the widest layer (widest layer = 64 * TPW outputs)
__global__ void __launch_bounds__(kStepThreads, TPW <= 4 ? 2 : 1) step_kernel(const StepArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, gid = lane >> 2, tig = lane & 3;
    const int row0 = blockIdx.x * kRows;
    const int p = a.p, k = a.k, n = a.n;

    unsigned char* ring = smem;
    bf16* act0 = reinterpret_cast<bf16*>(smem + kStages * a.stage_bytes);  // [kRows][act_ld0]
    bf16* act1 = act0 + kRows * a.act_ld0;                                // [kRows][act_ld1]
    float* lmx = reinterpret_cast<float*>(act1 + kRows * a.act_ld1);     // [K][P] landmark positions
    float* xr = lmx + k * p;                                              // [kRows][P] own positions
    float* red = xr + kRows * p;                                          // [warps][kRows][P]

    int total_chunks = 0;
    for (int l = 0; l <= a.layers; ++l) total_chunks += a.fi[l] / kChunkK;

    // Weight chunk `ch` (in network order) -> ring stage ch % kStages; always commits a group.
    auto issue = [&](int ch) {
        if (ch < total_chunks) {
            int l = 0, c = ch;
            while (c >= a.fi[l] / kChunkK) {
                c -= a.fi[l] / kChunkK;
                ++l;
            }
            const char* src = reinterpret_cast<const char*>(a.wpack + a.wofs[l] + (long long)c * a.fo[l] * kChunkK);
            unsigned char* dst = ring + (ch % kStages) * a.stage_bytes;
            const int pieces = a.fo[l] * (kChunkK * 2 / 16);
            for (int q = tid; q < pieces; q += kStepThreads) cp_async16(dst + q * 16, src + q * 16);
        }
        cp_async_commit();
    };
#pragma unroll
    for (int s = 0; s < kStages - 1; ++s) issue(s);

    // 1. positions (float) of the landmarks and of this tile's rows
    for (int e = tid; e < k * p; e += kStepThreads) {
        const int c = e / p, q = e - c * p;
        lmx[e] = (float)a.x_in[(size_t)a.lm[c] * p + q];
    }
    for (int e = tid; e < kRows * p; e += kStepThreads) {
        const int r = e / p, q = e - r * p, i = row0 + r;
        xr[e] = i < n ? (float)a.x_in[(size_t)i * p + q] : 0.0f;
    }
    __syncthreads();

    // 2. features: [r][c] residual to landmark c, [r][K + c] delta to landmark c
    for (int e = tid; e < kRows * k; e += kStepThreads) {
        const int r = e / k, c = e - r * k, i = row0 + r;
        bf16 fd = __float2bfloat16_rn(0.0f), fdel = fd;
        if (i < n) {
            float d2 = 0.0f;
            for (int q = 0; q < p; ++q) {
                const float d = xr[r * p + q] - lmx[c * p + q];
                d2 = fmaf(d, d, d2);
            }
            const float dl = a.dland[(size_t)i * k + c];
            fd = residual_feature(d2, dl, a.inv_sigma_r);
            fdel = delta_feature(dl, a.mu, a.inv_sigma);
        }
        act0[r * a.act_ld0 + c] = fd;
        act0[r * a.act_ld0 + k + c] = fdel;
    }

    // 3. the network
    float acc[TPW][2][4];
#pragma unroll
    for (int t = 0; t < TPW; ++t)
#pragma unroll
        for (int m = 0; m < 2; ++m)
#pragma unroll
            for (int r = 0; r < 4; ++r) acc[t][m][r] = 0.0f;

    const bf16* in = act0;
    int in_ld = a.act_ld0;
    bf16* out = act1;
    int out_ld = a.act_ld1;
    int ch = 0;
    for (int l = 0; l <= a.layers; ++l) {
        const int tpw = a.fo[l] / 64, nchunks = a.fi[l] / kChunkK;
        for (int c = 0; c < nchunks; ++c, ++ch) {
            cp_async_wait<kStages - 2>();
            __syncthreads();  // chunk ch has landed for every thread; stage of ch - 1 is free
            issue(ch + kStages - 1);
            const unsigned char* stage = ring + (ch % kStages) * a.stage_bytes;
#pragma unroll
            for (int kk = 0; kk < kChunkK; kk += 16) {
                uint32_t af[2][4];
#pragma unroll
                for (int m = 0; m < 2; ++m)
                    mlp::ldsm_x4(af[m], in + (16 * m + (lane & 15)) * in_ld + c * kChunkK + kk + ((lane >> 4) << 3));
#pragma unroll
                for (int t = 0; t < TPW; ++t) {
                    if (t < tpw) {
                        const int nr = (warp * tpw + t) * 8 + (lane & 7);
                        const int seg = (kk >> 3) + ((lane >> 3) & 1);
                        uint32_t bfr[2];
                        mlp::ldsm_x2(bfr, stage + nr * (kChunkK * 2) + ((seg ^ ((nr >> 1) & 3)) << 4));
                        mlp::mma_bf16(acc[t][0], af[0], bfr);
                        mlp::mma_bf16(acc[t][1], af[1], bfr);
                    }
                }
            }
        }
        if (l == a.layers) break;
        // hidden epilogue: bias + SiLU, BF16 into the other activation buffer
        const float* bias = a.bias[l];
#pragma unroll
        for (int t = 0; t < TPW; ++t) {
            if (t < tpw) {
                const int col = (warp * tpw + t) * 8 + 2 * tig;
                const float b0 = bias[col], b1 = bias[col + 1];
#pragma unroll
                for (int m = 0; m < 2; ++m)
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const int row = 16 * m + gid + 8 * h;
                        const float v0 = acc[t][m][2 * h] + b0, v1 = acc[t][m][2 * h + 1] + b1;
                        *reinterpret_cast<__nv_bfloat162*>(out + row * out_ld + col) =
                            __floats2bfloat162_rn(mlp::silu(v0), mlp::silu(v1));
                    }
            }
#pragma unroll
            for (int m = 0; m < 2; ++m)
#pragma unroll
                for (int r = 0; r < 4; ++r) acc[t][m][r] = 0.0f;
        }
        const bf16* next_in = out;
        const int next_ld = out_ld;
        out = const_cast<bf16*>(in);
        out_ld = in_ld;
        in = next_in;
        in_ld = next_ld;
    }

    // 4. contraction g_i = gscale * sum_k alpha_ik (x_i - x_{l_k}), per thread then tig lanes, then warps
    {
        const int tpw = a.fo[a.layers] / 64;
        const float* bias = a.bias[a.layers];
#pragma unroll
        for (int m = 0; m < 2; ++m) {
            float part[2][kMaxP];
#pragma unroll
            for (int h = 0; h < 2; ++h)
#pragma unroll
                for (int q = 0; q < kMaxP; ++q) part[h][q] = 0.0f;
#pragma unroll
            for (int t = 0; t < TPW; ++t) {
                if (t >= tpw) continue;
#pragma unroll
                for (int e = 0; e < 2; ++e) {
                    const int col = (warp * tpw + t) * 8 + 2 * tig + e;
                    const float b = bias[col];
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const int row = 16 * m + gid + 8 * h;
                        const float alpha = acc[t][m][2 * h + e] + b;
#pragma unroll
                        for (int q = 0; q < kMaxP; ++q)
                            if (q < p) part[h][q] = fmaf(alpha, xr[row * p + q] - lmx[col * p + q], part[h][q]);
                    }
                }
            }
#pragma unroll
            for (int h = 0; h < 2; ++h)
#pragma unroll
                for (int q = 0; q < kMaxP; ++q) {
                    if (q >= p) continue;
                    float v = part[h][q];
                    v += __shfl_xor_sync(0xffffffffu, v, 1);
                    v += __shfl_xor_sync(0xffffffffu, v, 2);
                    if (tig == 0) red[(warp * kRows + 16 * m + gid + 8 * h) * p + q] = v;
                }
        }
    }
    __syncthreads();

    // 5. per (row, dimension): gradient, kick and drift
    for (int e = tid; e < kRows * p; e += kStepThreads) {
        const int r = e / p, q = e - r * p, i = row0 + r;
        if (i >= n) continue;
        float s = 0.0f;
        for (int w = 0; w < kStepWarps; ++w) s += red[(w * kRows + r) * p + q];
        const double g = (double)s * (double)a.gscale;
        const size_t at = (size_t)i * p + q;
        if (a.mode & kWriteGradient) a.g_out[at] = g;
        if (a.mode & kKickDrift) {
            double prior = 0.0;
            for (int rr = 0; rr < p; ++rr) prior += a.x_in[(size_t)i * p + rr] * a.lam.m[rr * p + q];
            const double pm = a.mom[at] + a.coef[0] * (g - prior);
            const double xn = a.x_in[at] + a.coef[1] * pm;
            a.mom[at] = pm;
            a.x_out[at] = xn;
            if (a.soa_f32)
                static_cast<float*>(a.soa)[(size_t)q * a.x_ld + i] = (float)xn;
            else
                static_cast<double*>(a.soa)[(size_t)q * a.x_ld + i] = xn;
        }
    }
}

// Shared memory of one CTA for these arguments.
size_t step_smem_bytes(const StepArgs& a) {
    return (size_t)kStages * a.stage_bytes + (size_t)kRows * (a.act_ld0 + a.act_ld1) * 2 +
           (size_t)(a.k * a.p + kRows * a.p + kStepWarps * kRows * a.p) * 4;
}

template <int TPW>
static cudaError_t launch_tpw(const StepArgs& a, cudaStream_t st) {
    const size_t smem = step_smem_bytes(a);
    cudaError_t e = cudaFuncSetAttribute(step_kernel<TPW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int grid = (a.n + kRows - 1) / kRows;
    step_kernel<TPW><<<grid, kStepThreads, smem, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_step(const StepArgs& a, cudaStream_t st) {
    int widest = 0;
    for (int l = 0; l <= a.layers; ++l) widest = widest > a.fo[l] ? widest : a.fo[l];
    switch (widest / 64) {
        case 1: return launch_tpw<1>(a, st);
        case 2: return launch_tpw<2>(a, st);
        case 3:
        case 4: return launch_tpw<4>(a, st);
        case 5: case 6: case 7:
        case 8: return launch_tpw<8>(a, st);
        default: return cudaErrorInvalidValue;
    }
}

// Packs an FP32 weight [fo][fi] into the BF16 chunk layout the step kernel streams.
__global__ void pack_weight_kernel(const float* __restrict__ w, int fo, int fi, bf16* __restrict__ dst) {
    const long long total = (long long)fo * fi;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int nrow = (int)(e / fi), kcol = (int)(e - (long long)nrow * fi);
        dst[packed_index(nrow, kcol, fo)] = __float2bfloat16_rn(w[e]);
    }
}

cudaError_t pack_weight(const float* w, int fo, int fi, bf16* dst, cudaStream_t st) {
    const long long total = (long long)fo * fi;
    const int grid = (int)((total + 255) / 256 < 4096 ? (total + 255) / 256 : 4096);
    pack_weight_kernel<<<grid, 256, 0, st>>>(w, fo, fi, dst);
    return cudaGetLastError();
}

}  // namespace surr
}  // namespace mdsx
