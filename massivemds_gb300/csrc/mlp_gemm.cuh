// BF16 tensor-core GEMM for the gradient-surrogate MLP (not the hot path).
//
// C[M x N] = op(A)[M x K] * op(B)[K x N] with FP32 accumulation on the tensor
// cores (mma.sync.m16n8k16 bf16 -> f32), operands staged in shared memory and
// fed with ldmatrix (".trans" where a tile is stored the other way round).
// Layouts, all row-major in memory with leading dimensions:
//   A_T = false: A stored [M][K];  A_T = true: A stored [K][M] (A = stored^T)
//   B_T = false: B stored [N][K] (the nn.Linear weight layout [out][in]);
//   B_T = true:  B stored [K][N].
// The three products of an MLP layer are then
//   forward   Z = X W^T      : A = X [M][in],    B = W [out][in]    (A_T=0, B_T=0)
//   backward  dX = dZ W      : A = dZ [M][out],  B = W [out][in]    (A_T=0, B_T=1)
//   weights   dW = dZ^T X    : A = dZ [M][out]^T, B = X [M][in]     (A_T=1, B_T=1)
// Shapes must be padded by the caller to multiples of the tile (M, N: 64;
// K: 32), so the kernel has no bounds checks. Epilogues fuse bias, SiLU and
// its derivative.
#pragma once

#include <cuda_bf16.h>
#include <cstdint>

namespace mdsx {
namespace mlp {

constexpr int kBM = 64, kBN = 64, kBK = 32;
constexpr int kGemmThreads = 128;  // 4 warps, 2 x 2, each 32 x 32
constexpr int kPad = 8;            // bf16 elements of row padding in shared memory

enum Epilogue : int {
    kStoreF32 = 0,        // C (fp32)
    kBiasSiluF32Bf16 = 1, // Z = acc + bias -> Zout (fp32), H = silu(Z) -> Hout (bf16)
    kBiasF32 = 2,         // acc + bias -> C (fp32)
    kSiluGradBf16 = 3,    // dZ = acc * silu'(Zsaved) -> C (fp32) and Hout (bf16)
};

struct GemmArgs {
    const __nv_bfloat16* a;
    const __nv_bfloat16* b;
    int lda, ldb;      // leading dimensions of the stored arrays (elements)
    int m, n, k;       // padded sizes
    float* c;          // fp32 output [M][N], ldc
    int ldc;
    const float* bias; // [N] (epilogues 1, 2)
    const float* zsaved;  // [M][N] fp32 pre-activations (epilogue 3), ldc
    __nv_bfloat16* hout;  // bf16 output [M][N], ldh (epilogues 1, 3)
    int ldh;
    int epilogue;
};

__device__ __forceinline__ float silu(float z) { return z / (1.0f + __expf(-z)); }
__device__ __forceinline__ float silu_grad(float z) {
    const float s = 1.0f / (1.0f + __expf(-z));
    return s * (1.0f + z * (1.0f - s));
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], const void* p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(smem_u32(p)));
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t (&r)[4], const void* p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(smem_u32(p)));
}
__device__ __forceinline__ void ldsm_x2(uint32_t (&r)[2], const void* p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];" : "=r"(r[0]), "=r"(r[1]) : "r"(smem_u32(p)));
}
__device__ __forceinline__ void ldsm_x2_t(uint32_t (&r)[2], const void* p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x2.trans.shared.b16 {%0,%1}, [%2];"
                 : "=r"(r[0]), "=r"(r[1])
                 : "r"(smem_u32(p)));
}
__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// Shared tiles. Non-transposed A: [kBM][kBK]; transposed A: [kBK][kBM].
// B stored [N][K]: [kBN][kBK]; B stored [K][N]: [kBK][kBN]. Rows padded by kPad.
template <bool A_T, bool B_T>
__global__ void __launch_bounds__(kGemmThreads) gemm_kernel(const GemmArgs g) {
    constexpr int A_ROWS = A_T ? kBK : kBM, A_COLS = (A_T ? kBM : kBK) + kPad;
    constexpr int B_ROWS = B_T ? kBK : kBN, B_COLS = (B_T ? kBN : kBK) + kPad;
    __shared__ __align__(16) __nv_bfloat16 sa[A_ROWS][A_COLS];
    __shared__ __align__(16) __nv_bfloat16 sb[B_ROWS][B_COLS];

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.y * kBM, n0 = blockIdx.x * kBN;
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;

    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int r = 0; r < 4; ++r) acc[i][j][r] = 0.f;

    for (int k0 = 0; k0 < g.k; k0 += kBK) {
        // global -> shared, 16-byte chunks (8 bf16); each tile is 256 chunks
#pragma unroll
        for (int it = 0; it < 2; ++it) {
            const int chunk = tid + it * kGemmThreads;
            {
                const int cols = (A_T ? kBM : kBK) / 8;
                const int r = chunk / cols, c = (chunk % cols) * 8;
                const __nv_bfloat16* src = A_T ? g.a + (size_t)(k0 + r) * g.lda + m0 + c
                                               : g.a + (size_t)(m0 + r) * g.lda + k0 + c;
                *reinterpret_cast<uint4*>(&sa[r][c]) = *reinterpret_cast<const uint4*>(src);
            }
            {
                const int cols = (B_T ? kBN : kBK) / 8;
                const int r = chunk / cols, c = (chunk % cols) * 8;
                const __nv_bfloat16* src = B_T ? g.b + (size_t)(k0 + r) * g.ldb + n0 + c
                                               : g.b + (size_t)(n0 + r) * g.ldb + k0 + c;
                *reinterpret_cast<uint4*>(&sb[r][c]) = *reinterpret_cast<const uint4*>(src);
            }
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < kBK; kk += 16) {
            uint32_t af[2][4], bfr[4][2];
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const int mb = wm + 16 * i;
                if (A_T) {
                    // lanes 0-7: k rows 0-7 at m; 8-15: k 0-7 at m+8; 16-23: k 8-15 at m; 24-31: k 8-15 at m+8
                    const int kr = kk + (lane & 7) + ((lane >> 4) << 3);
                    const int mc = mb + (((lane >> 3) & 1) << 3);
                    ldsm_x4_t(af[i], &sa[kr][mc]);
                } else {
                    // lanes 0-15: rows 0-15 at k; 16-31: rows 0-15 at k+8
                    const int mr = mb + (lane & 15);
                    const int kc = kk + ((lane >> 4) << 3);
                    ldsm_x4(af[i], &sa[mr][kc]);
                }
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int nb = wn + 8 * j;
                if (B_T) {
                    // stored [K][N]: lanes 0-7 rows k 0-7, lanes 8-15 rows k 8-15, at column nb
                    const int kr = kk + (lane & 15);
                    ldsm_x2_t(bfr[j], &sb[kr][nb]);
                } else {
                    // stored [N][K]: lanes 0-7 rows n 0-7 at k, lanes 8-15 at k+8
                    const int nr = nb + (lane & 7);
                    const int kc = kk + (((lane >> 3) & 1) << 3);
                    ldsm_x2(bfr[j], &sb[nr][kc]);
                }
            }
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) mma_bf16(acc[i][j], af[i], bfr[j]);
        }
        __syncthreads();
    }

    // epilogue: accumulator (row groupID (+8), cols 2*(lane%4) (+1))
    const int gid = lane >> 2, tig = lane & 3;
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int row = m0 + wm + 16 * i + gid + 8 * h;
                const int col = n0 + wn + 8 * j + 2 * tig;
                float v0 = acc[i][j][2 * h], v1 = acc[i][j][2 * h + 1];
                float* cp = g.c + (size_t)row * g.ldc + col;
                if (g.epilogue == kBiasSiluF32Bf16 || g.epilogue == kBiasF32) {
                    v0 += g.bias[col];
                    v1 += g.bias[col + 1];
                }
                if (g.epilogue == kSiluGradBf16) {
                    const float* zp = g.zsaved + (size_t)row * g.ldc + col;
                    v0 *= silu_grad(zp[0]);
                    v1 *= silu_grad(zp[1]);
                }
                *reinterpret_cast<float2*>(cp) = make_float2(v0, v1);
                if (g.epilogue == kBiasSiluF32Bf16) {
                    *reinterpret_cast<__nv_bfloat162*>(g.hout + (size_t)row * g.ldh + col) =
                        __floats2bfloat162_rn(silu(v0), silu(v1));
                } else if (g.epilogue == kSiluGradBf16) {
                    *reinterpret_cast<__nv_bfloat162*>(g.hout + (size_t)row * g.ldh + col) =
                        __floats2bfloat162_rn(v0, v1);
                }
            }
}

}  // namespace mlp
}  // namespace mdsx
