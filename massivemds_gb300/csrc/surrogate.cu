// Learned gradient surrogate for HMC on the MDS posterior (no counterpart in
// the reference).
//
// The exact likelihood gradient is g_i = sum_j c_ij (x_i - x_j), an O(N) sum
// per location. The surrogate keeps that form over K landmark locations
// l_1..l_K (a seeded random subset of the N locations):
//     g_i ~= s * sum_k alpha_ik(f_i) (x_i - x_{l_k}),
// where f_i = [(d(x_i, x_{l_k}) - mu)/sigma, (delta_{i,l_k} - mu)/sigma]_k are
// rotation-invariant features and alpha_i = MLP(f_i) has K outputs, so the
// prediction rotates with the configuration. Cost O(N K) per gradient plus
// the MLP. The MLP (2K -> H -> ... -> H -> K, SiLU) runs on the tensor cores
// through mlp_gemm.cuh (BF16 operands, FP32 accumulation) forward and
// backward, and is trained with Adam (FP32 master weights) on rows
// (features, landmark directions, exact gradient) harvested from exact-gradient
// HMC trajectories. HMC uses it only inside trajectories; every accept is
// decided with the exact potential (hmc.cu).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "../../include/mdsx.h"
#include "engine_internal.h"
#include "mlp_gemm.cuh"
#include "surrogate.h"
#include "surrogate_step.cuh"

namespace mdsx {
namespace surr {

using bf16 = __nv_bfloat16;

// ---------------------------------------------------------------- kernels

template <typename S>
__global__ void gather_landmark_delta_kernel(const S* __restrict__ delta, long long ld, int n, const int* __restrict__ lm,
                                             int k, float* __restrict__ out) {
    const long long total = (long long)n * k;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const long long i = idx / k;
        const int c = (int)(idx - i * k);
        const float v = (float)delta[i * ld + lm[c]];
        out[idx] = (v == v) ? v : 0.0f;  // a missing landmark pair contributes a neutral feature
    }
}

// Training features of rows r < rows, location loc[r], at positions x (N x
// P), with the arithmetic of the step kernel (surrogate_step.cuh): BF16
// features [rows][ldf] (2K used), directions x_i - x_{l_k} (fp32
// [rows][K][P]) and the target gradient rows (fp32 [rows][P]) from g.
__global__ void features_kernel(const double* __restrict__ x, int p, const int* __restrict__ loc, int rows,
                                const int* __restrict__ lm, int k, const float* __restrict__ dland, float mu,
                                float inv_sigma, float inv_sigma_r, bf16* __restrict__ feat, int ldf,
                                float* __restrict__ dirs,
                                const double* __restrict__ g, float* __restrict__ target) {
    const long long total = (long long)rows * k;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(idx / k), c = (int)(idx - (long long)(idx / k) * k);
        const int i = loc[r];
        const int l = lm[c];
        float d2 = 0.0f;
        for (int q = 0; q < p; ++q) {
            const float d = (float)x[(size_t)i * p + q] - (float)x[(size_t)l * p + q];
            d2 = fmaf(d, d, d2);
            dirs[((size_t)r * k + c) * p + q] = d;
        }
        const float dl = dland[(size_t)i * k + c];
        feat[(size_t)r * ldf + c] = residual_feature(d2, dl, inv_sigma_r);
        feat[(size_t)r * ldf + k + c] = delta_feature(dl, mu, inv_sigma);
        if (c == 0)
            for (int q = 0; q < p; ++q) target[(size_t)r * p + q] = (float)g[(size_t)i * p + q];
    }
}

// Sum of squared residuals d(x_i, x_{l_k}) - delta_{i, l_k} over rows loc[r] (into *out).
__global__ void residual_sq_kernel(const double* __restrict__ x, int p, const int* __restrict__ loc, int rows,
                                   const int* __restrict__ lm, int k, const float* __restrict__ dland,
                                   double* __restrict__ out) {
    double acc = 0.0;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < (long long)rows * k;
         idx += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(idx / k), c = (int)(idx - (long long)r * k);
        const int i = loc[r], l = lm[c];
        float d2 = 0.0f;
        for (int q = 0; q < p; ++q) {
            const float d = (float)x[(size_t)i * p + q] - (float)x[(size_t)l * p + q];
            d2 = fmaf(d, d, d2);
        }
        const double res = (double)__fsqrt_rn(d2) - (double)dland[(size_t)i * k + c];
        acc += res * res;
    }
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(out, acc);
}

// Training contraction and loss: per row r, pred = scale * sum_k alpha[r][k] dir[r][k],
// res = pred - target / tscale; loss += |res|^2 / rows; dalpha = 2 scale/rows * res . dir.
// One warp per row; writes dalpha fp32 and bf16.
__global__ void loss_kernel(const float* __restrict__ alpha, int lda, const float* __restrict__ dirs,
                            const float* __restrict__ target, int rows, int k, int p, float scale, float inv_tscale,
                            float* __restrict__ dalpha, bf16* __restrict__ dalpha_h, float* __restrict__ loss) {
    const int warps = (gridDim.x * blockDim.x) >> 5, lane = threadIdx.x & 31;
    for (int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < rows; r += warps) {
        float pred[MDSX_MAX_DIMENSION];
        for (int q = 0; q < p; ++q) pred[q] = 0.f;
        for (int c = lane; c < k; c += 32) {
            const float a = alpha[(size_t)r * lda + c];
            for (int q = 0; q < p; ++q) pred[q] += a * dirs[((size_t)r * k + c) * p + q];
        }
        float res[MDSX_MAX_DIMENSION], l2 = 0.f;
        for (int q = 0; q < p; ++q) {
            float v = pred[q];
            for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
            res[q] = scale * v - target[(size_t)r * p + q] * inv_tscale;
            l2 += res[q] * res[q];
        }
        const float coef = 2.f * scale / rows;
        for (int c = lane; c < k; c += 32) {
            float d = 0.f;
            for (int q = 0; q < p; ++q) d += res[q] * dirs[((size_t)r * k + c) * p + q];
            dalpha[(size_t)r * lda + c] = coef * d;
            dalpha_h[(size_t)r * lda + c] = __float2bfloat16_rn(coef * d);
        }
        if (lane == 0) atomicAdd(loss, l2 / rows);
    }
}

// db[n] = sum over rows of dz[r][n] (fixed order per column).
__global__ void bias_grad_kernel(const float* __restrict__ dz, int ld, int rows, int cols, float* __restrict__ db) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cols) return;
    float s = 0.f;
    for (int r = 0; r < rows; ++r) s += dz[(size_t)r * ld + c];
    db[c] = s;
}

// Adam on FP32 master parameters; refreshes the bf16 copy when wh != NULL.
__global__ void adam_kernel(float* __restrict__ w, const float* __restrict__ gw, float* __restrict__ m,
                            float* __restrict__ v, long long count, float lr, float b1, float b2, float bc1, float bc2,
                            float eps, bf16* __restrict__ wh) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
         i += (long long)gridDim.x * blockDim.x) {
        const float gi = gw[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float wi = w[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
        w[i] = wi;
        if (wh) wh[i] = __float2bfloat16_rn(wi);
    }
}

__global__ void to_bf16_kernel(const float* __restrict__ a, bf16* __restrict__ b, long long count) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
         i += (long long)gridDim.x * blockDim.x)
        b[i] = __float2bfloat16_rn(a[i]);
}

// rows of a training set gathered into a batch (features, directions, targets)
__global__ void gather_rows_kernel(const int* __restrict__ idx, int rows, const bf16* __restrict__ feat, int ldf,
                                   const float* __restrict__ dirs, const float* __restrict__ target, int k, int p,
                                   bf16* __restrict__ bfeat, float* __restrict__ bdirs, float* __restrict__ btarget) {
    const int r = blockIdx.x;
    if (r >= rows) return;
    const int s = idx[r];
    for (int c = threadIdx.x; c < ldf; c += blockDim.x) bfeat[(size_t)r * ldf + c] = feat[(size_t)s * ldf + c];
    for (int c = threadIdx.x; c < k * p; c += blockDim.x) bdirs[(size_t)r * k * p + c] = dirs[(size_t)s * k * p + c];
    if (threadIdx.x < p) btarget[(size_t)r * p + threadIdx.x] = target[(size_t)s * p + threadIdx.x];
}

int grid_for(long long work) { return (int)std::max(1LL, std::min(4096LL, (work + 255) / 256)); }

}  // namespace surr
}  // namespace mdsx

namespace mdsx {
namespace surr {
namespace {

using mlp::GemmArgs;

int fail(mdsx_surrogate* s, int code, const std::string& msg) {
    s->last_error = msg;
    return code;
}
int cfail(mdsx_surrogate* s, cudaError_t e, const char* what) {
    return fail(s, e == cudaErrorMemoryAllocation ? MDSX_ENOMEM : MDSX_ECUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}
#define SURR_CUDA(s, call)                                         \
    do {                                                           \
        cudaError_t _e = (call);                                   \
        if (_e != cudaSuccess) return cfail(s, _e, #call);         \
    } while (0)

template <bool AT, bool BT>
cudaError_t gemm(const GemmArgs& g, cudaStream_t st) {
    const dim3 grid(g.n / mlp::kBN, g.m / mlp::kBM);
    mlp::gemm_kernel<AT, BT><<<grid, mlp::kGemmThreads, 0, st>>>(g);
    return cudaGetLastError();
}

GemmArgs args(const bf16* a, int lda, const bf16* b, int ldb, int m, int n, int k, float* c, int ldc, int epi) {
    GemmArgs g{};
    g.a = a;
    g.lda = lda;
    g.b = b;
    g.ldb = ldb;
    g.m = m;
    g.n = n;
    g.k = k;
    g.c = c;
    g.ldc = ldc;
    g.epilogue = epi;
    return g;
}

// Forward over `rows` rows of a_feat: hidden z/h, output z[layers] (alpha).
int forward(mdsx_surrogate* s, int rows, cudaStream_t st) {
    const bf16* x = s->a_feat;
    int ldx = s->in;
    for (int l = 0; l <= s->layers; ++l) {
        const bool out = l == s->layers;
        GemmArgs g = args(x, ldx, s->wh[l], s->fan_in[l], rows, s->fan_out[l], s->fan_in[l], s->z[l], s->fan_out[l],
                          out ? mlp::kBiasF32 : mlp::kBiasSiluF32Bf16);
        g.bias = s->b[l];
        if (!out) {
            g.hout = s->h[l];
            g.ldh = s->fan_out[l];
        }
        SURR_CUDA(s, (gemm<false, false>(g, st)));
        if (!out) {
            x = s->h[l];
            ldx = s->fan_out[l];
        }
    }
    return MDSX_OK;
}

// Backward from d alpha (s->dz / s->dzh, [rows][K]) into gw, gb of every layer.
int backward(mdsx_surrogate* s, int rows, cudaStream_t st) {
    float* dz = s->dz;
    bf16* dzh = s->dzh;
    float* dzn = s->dz2;
    bf16* dzhn = s->dzh2;
    for (int l = s->layers; l >= 0; --l) {
        const int fo = s->fan_out[l], fi = s->fan_in[l];
        const bf16* in = l == 0 ? s->a_feat : s->h[l - 1];
        // dW = dZ^T X
        SURR_CUDA(s, (gemm<true, true>(args(dzh, fo, in, fi, fo, fi, rows, s->gw[l], fi, mlp::kStoreF32), st)));
        bias_grad_kernel<<<(fo + 127) / 128, 128, 0, st>>>(dz, fo, rows, fo, s->gb[l]);
        SURR_CUDA(s, cudaGetLastError());
        if (l > 0) {
            // dX = dZ W, times silu'(z of the layer below)
            GemmArgs g = args(dzh, fo, s->wh[l], fi, rows, fi, fo, dzn, fi, mlp::kSiluGradBf16);
            g.zsaved = s->z[l - 1];
            g.hout = dzhn;
            g.ldh = fi;
            SURR_CUDA(s, (gemm<false, true>(g, st)));
            std::swap(dz, dzn);
            std::swap(dzh, dzhn);
        }
    }
    return MDSX_OK;
}

int adam_step(mdsx_surrogate* s, float lr, cudaStream_t st) {
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    ++s->adam_t;
    const float bc1 = 1.f - std::pow(b1, (float)s->adam_t), bc2 = 1.f - std::pow(b2, (float)s->adam_t);
    for (int l = 0; l <= s->layers; ++l) {
        const long long nw = (long long)s->fan_out[l] * s->fan_in[l];
        adam_kernel<<<grid_for(nw), 256, 0, st>>>(s->w[l], s->gw[l], s->mw[l], s->vw[l], nw, lr, b1, b2, bc1, bc2,
                                                   eps, s->wh[l]);
        adam_kernel<<<grid_for(s->fan_out[l]), 256, 0, st>>>(s->b[l], s->gb[l], s->mb[l], s->vb[l], s->fan_out[l], lr,
                                                              b1, b2, bc1, bc2, eps, nullptr);
    }
    SURR_CUDA(s, cudaGetLastError());
    return MDSX_OK;
}

void free_all(mdsx_surrogate* s) {
    for (auto* v : {&s->w, &s->b, &s->gw, &s->gb, &s->mw, &s->vw, &s->mb, &s->vb, &s->z})
        for (float* q : *v) cudaFree(q);
    for (bf16* q : s->wh) cudaFree(q);
    for (bf16* q : s->h) cudaFree(q);
    cudaFree(s->landmarks);
    cudaFree(s->dland);
    cudaFree(s->wpack);
    cudaFree(s->t_feat);
    cudaFree(s->t_dirs);
    cudaFree(s->t_target);
    cudaFree(s->a_feat);
    cudaFree(s->a_dirs);
    cudaFree(s->a_target);
    cudaFree(s->dz);
    cudaFree(s->dzh);
    cudaFree(s->dz2);
    cudaFree(s->dzh2);
    cudaFree(s->idx);
    cudaFree(s->loss);
}

StepArgs step_args(const mdsx_surrogate* s) {
    StepArgs a{};
    a.n = s->n;
    a.p = s->p;
    a.k = s->k;
    a.layers = s->layers;
    int widest = 0;
    for (int l = 0; l <= s->layers; ++l) {
        a.fo[l] = s->fan_out[l];
        a.fi[l] = s->fan_in[l];
        a.bias[l] = s->b[l];
        a.wofs[l] = s->wofs[l];
        widest = std::max(widest, s->fan_out[l]);
    }
    a.wpack = s->wpack;
    a.lm = s->landmarks;
    a.dland = s->dland;
    a.mu = s->mu;
    a.inv_sigma = s->inv_sigma;
    a.inv_sigma_r = s->inv_sigma_r;
    a.gscale = s->scale * s->tscale;
    a.stage_bytes = widest * kChunkK * 2;
    a.act_ld0 = std::max(s->in, s->width) + 8;
    a.act_ld1 = s->width + 8;
    return a;
}

}  // namespace

// Refreshes the step kernel's packed BF16 weights from the FP32 masters.
int pack_all(mdsx_surrogate* s, cudaStream_t st) {
    for (int l = 0; l <= s->layers; ++l)
        SURR_CUDA(s, pack_weight(s->w[l], s->fan_out[l], s->fan_in[l], s->wpack + s->wofs[l], st));
    return MDSX_OK;
}

int gradient(mdsx_surrogate* s, const double* d_x, double* d_out, cudaStream_t st) {
    StepArgs a = step_args(s);
    a.x_in = d_x;
    a.g_out = d_out;
    a.mode = kWriteGradient;
    SURR_CUDA(s, launch_step(a, st));
    return MDSX_OK;
}

int kick_drift(mdsx_surrogate* s, const double* x_in, double* x_out, double* mom, double* g_out, const double* coef,
               const double* lam, cudaStream_t st) {
    StepArgs a = step_args(s);
    a.x_in = x_in;
    a.x_out = x_out;
    a.mom = mom;
    a.g_out = g_out;
    a.coef = coef;
    mdsx_engine* e = s->engine;
    a.soa = e->d_x[e->xcur];
    a.soa_f32 = e->x_f32 ? 1 : 0;
    a.x_ld = e->x_ld;
    for (int i = 0; i < s->p * s->p; ++i) a.lam.m[i] = lam[i];
    a.mode = kKickDrift | (g_out ? kWriteGradient : 0);
    SURR_CUDA(s, launch_step(a, st));
    return MDSX_OK;
}

int add_state(mdsx_surrogate* s, const double* d_x, const double* d_grad, int rows, unsigned long long seed,
              cudaStream_t st) {
    rows = std::min(rows, s->max_rows - s->rows);
    if (rows <= 0) return MDSX_OK;
    std::mt19937_64 rng(seed);
    std::uniform_int_distribution<int> pick(0, s->n - 1);
    std::vector<int> loc(rows);
    for (int& v : loc) v = pick(rng);
    int* d_loc = s->idx;  // reuse the batch index buffer (work_rows >= rows checked at create)
    if (rows > s->work_rows) return fail(s, MDSX_EINVAL, "surrogate: too many rows in one state");
    SURR_CUDA(s, cudaMemcpyAsync(d_loc, loc.data(), rows * sizeof(int), cudaMemcpyHostToDevice, st));
    if (!s->resid_fixed) {  // the residual scale: RMS residual of the first harvested state
        SURR_CUDA(s, cudaMemsetAsync(s->loss, 0, sizeof(double), st));
        residual_sq_kernel<<<grid_for((long long)rows * s->k), 256, 0, st>>>(d_x, s->p, d_loc, rows, s->landmarks,
                                                                              s->k, s->dland,
                                                                              reinterpret_cast<double*>(s->loss));
        SURR_CUDA(s, cudaGetLastError());
        double sq = 0.0;
        SURR_CUDA(s, cudaMemcpyAsync(&sq, s->loss, sizeof(double), cudaMemcpyDeviceToHost, st));
        SURR_CUDA(s, cudaStreamSynchronize(st));
        const double rms = std::sqrt(sq / ((double)rows * s->k));
        s->inv_sigma_r = rms > 0.0 && std::isfinite(rms) ? (float)(1.0 / rms) : 1.0f;
        s->resid_fixed = true;
    }
    features_kernel<<<grid_for((long long)rows * s->k), 256, 0, st>>>(
        d_x, s->p, d_loc, rows, s->landmarks, s->k, s->dland, s->mu, s->inv_sigma, s->inv_sigma_r,
        s->t_feat + (size_t)s->rows * s->in,
        s->in, s->t_dirs + (size_t)s->rows * s->k * s->p, d_grad, s->t_target + (size_t)s->rows * s->p);
    SURR_CUDA(s, cudaGetLastError());
    SURR_CUDA(s, cudaStreamSynchronize(st));  // loc lives on the host stack
    s->rows += rows;
    return MDSX_OK;
}

}  // namespace surr
}  // namespace mdsx

using namespace mdsx::surr;

extern "C" {

int mdsx_surrogate_create(mdsx_engine* e, int landmarks, int hidden_width, int hidden_layers, int max_rows,
                          unsigned long long seed, mdsx_surrogate** out) {
    using mdsx::internal::fail;
    if (!e) return MDSX_EINVAL;
    if (!out) return fail(e, MDSX_EINVAL, "surrogate: out is NULL");
    *out = nullptr;
    if (landmarks < 64 || landmarks % 64 || landmarks > e->n)
        return fail(e, MDSX_EINVAL, "surrogate: landmarks must be a multiple of 64 and at most N");
    if (hidden_width < 64 || hidden_width % 64) return fail(e, MDSX_EINVAL, "surrogate: hidden width must be a multiple of 64");
    if (hidden_layers < 1 || hidden_layers > 8) return fail(e, MDSX_EINVAL, "surrogate: 1..8 hidden layers");
    if (max_rows < 64) return fail(e, MDSX_EINVAL, "surrogate: max_rows must be >= 64");
    if (!e->data_set) return fail(e, MDSX_ESTATE, "surrogate: setPairwiseData has not been called");
    if (e->rows != e->n) return fail(e, MDSX_EUNSUPPORTED, "surrogate: needs an engine over the whole matrix");
    if (e->dd) return fail(e, MDSX_EUNSUPPORTED, "surrogate: not built for double-float pair math");
    mdsx::internal::DeviceGuard guard(e->device);
    auto* s = new mdsx_surrogate;
    s->engine = e;
    s->device = e->device;
    s->n = e->n;
    s->p = e->p;
    s->k = landmarks;
    s->width = hidden_width;
    s->layers = hidden_layers;
    s->n_pad = (e->n + 63) / 64 * 64;
    s->in = 2 * landmarks;
    s->max_rows = max_rows;
    s->work_rows = 8192;  // largest training batch
    s->scale = 1.0f / std::sqrt((float)landmarks);
    cudaStream_t st = e->stream;
    auto bail = [&](int rc) {
        e->last_error = s->last_error;
        free_all(s);
        delete s;
        return rc;
    };
#define SC(call)                                                                     \
    do {                                                                             \
        cudaError_t _e = (call);                                                     \
        if (_e != cudaSuccess) {                                                     \
            s->last_error = std::string(#call) + ": " + cudaGetErrorString(_e);      \
            return bail(_e == cudaErrorMemoryAllocation ? MDSX_ENOMEM : MDSX_ECUDA);  \
        }                                                                            \
    } while (0)
    // landmarks: a seeded random subset of the locations
    std::mt19937_64 rng(seed);
    std::vector<int> all(e->n);
    for (int i = 0; i < e->n; ++i) all[i] = i;
    std::shuffle(all.begin(), all.end(), rng);
    std::vector<int> lm(all.begin(), all.begin() + landmarks);
    std::sort(lm.begin(), lm.end());
    SC(cudaMalloc(&s->landmarks, landmarks * sizeof(int)));
    SC(cudaMemcpy(s->landmarks, lm.data(), landmarks * sizeof(int), cudaMemcpyHostToDevice));
    SC(cudaMalloc(&s->dland, (size_t)e->n * landmarks * sizeof(float)));
    if (e->delta_f32)
        gather_landmark_delta_kernel<float><<<grid_for((long long)e->n * landmarks), 256, 0, st>>>(
            static_cast<const float*>(e->d_delta), e->ld, e->n, s->landmarks, landmarks, s->dland);
    else
        gather_landmark_delta_kernel<double><<<grid_for((long long)e->n * landmarks), 256, 0, st>>>(
            static_cast<const double*>(e->d_delta), e->ld, e->n, s->landmarks, landmarks, s->dland);
    SC(cudaGetLastError());
    {  // delta-feature standardisation
        std::vector<float> host((size_t)e->n * landmarks);
        SC(cudaMemcpyAsync(host.data(), s->dland, host.size() * sizeof(float), cudaMemcpyDeviceToHost, st));
        SC(cudaStreamSynchronize(st));
        double m = 0.0, m2 = 0.0;
        for (float v : host) {
            m += v;
            m2 += (double)v * v;
        }
        m /= host.size();
        const double var = std::max(1e-12, m2 / host.size() - m * m);
        s->mu = (float)m;
        s->inv_sigma = (float)(1.0 / std::sqrt(var));
    }
    // layers
    for (int l = 0; l <= hidden_layers; ++l) {
        s->fan_in.push_back(l == 0 ? s->in : hidden_width);
        s->fan_out.push_back(l == hidden_layers ? landmarks : hidden_width);
    }
    for (int l = 0; l <= hidden_layers; ++l) {
        const size_t nw = (size_t)s->fan_out[l] * s->fan_in[l], nb = s->fan_out[l];
        float *w, *b, *gw, *gb, *mw, *vw, *mb, *vb;
        bf16* wh;
        SC(cudaMalloc(&w, nw * 4)); s->w.push_back(w);
        SC(cudaMalloc(&gw, nw * 4)); s->gw.push_back(gw);
        SC(cudaMalloc(&mw, nw * 4)); s->mw.push_back(mw);
        SC(cudaMalloc(&vw, nw * 4)); s->vw.push_back(vw);
        SC(cudaMalloc(&b, nb * 4)); s->b.push_back(b);
        SC(cudaMalloc(&gb, nb * 4)); s->gb.push_back(gb);
        SC(cudaMalloc(&mb, nb * 4)); s->mb.push_back(mb);
        SC(cudaMalloc(&vb, nb * 4)); s->vb.push_back(vb);
        SC(cudaMalloc(&wh, nw * 2)); s->wh.push_back(wh);
        SC(cudaMemsetAsync(mw, 0, nw * 4, st));
        SC(cudaMemsetAsync(vw, 0, nw * 4, st));
        SC(cudaMemsetAsync(b, 0, nb * 4, st));
        SC(cudaMemsetAsync(mb, 0, nb * 4, st));
        SC(cudaMemsetAsync(vb, 0, nb * 4, st));
        // Glorot-uniform initial weights (smaller for the output layer)
        const double lim = std::sqrt(6.0 / (s->fan_in[l] + s->fan_out[l])) * (l == hidden_layers ? 0.1 : 1.0);
        std::uniform_real_distribution<double> u(-lim, lim);
        std::vector<float> hw(nw);
        for (float& v : hw) v = (float)u(rng);
        SC(cudaMemcpy(w, hw.data(), nw * 4, cudaMemcpyHostToDevice));
        to_bf16_kernel<<<grid_for((long long)nw), 256, 0, st>>>(w, wh, (long long)nw);
        SC(cudaGetLastError());
    }
    // the step kernel's packed weights
    {
        long long total = 0;
        for (int l = 0; l <= hidden_layers; ++l) {
            s->wofs.push_back(total);
            total += (long long)s->fan_out[l] * s->fan_in[l];
        }
        SC(cudaMalloc(&s->wpack, (size_t)total * sizeof(bf16)));
        if (pack_all(s, st)) return bail(MDSX_ECUDA);
        int max_smem = 0;
        SC(cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, e->device));
        if (step_smem_bytes(step_args(s)) > (size_t)max_smem) {
            s->last_error = "surrogate: landmarks and width too large for one CTA's shared memory";
            return bail(MDSX_EINVAL);
        }
    }
    // training set and work buffers
    SC(cudaMalloc(&s->t_feat, (size_t)max_rows * s->in * 2));
    SC(cudaMalloc(&s->t_dirs, (size_t)max_rows * landmarks * s->p * 4));
    SC(cudaMalloc(&s->t_target, (size_t)max_rows * s->p * 4));
    const size_t wr = s->work_rows, wide = std::max(hidden_width, landmarks);
    SC(cudaMalloc(&s->a_feat, wr * s->in * 2));
    SC(cudaMemsetAsync(s->a_feat, 0, wr * s->in * 2, st));
    SC(cudaMalloc(&s->a_dirs, wr * landmarks * s->p * 4));
    SC(cudaMalloc(&s->a_target, wr * s->p * 4));
    for (int l = 0; l <= hidden_layers; ++l) {
        float* z;
        SC(cudaMalloc(&z, wr * s->fan_out[l] * 4));
        s->z.push_back(z);
        if (l < hidden_layers) {
            bf16* h;
            SC(cudaMalloc(&h, wr * hidden_width * 2));
            s->h.push_back(h);
        }
    }
    SC(cudaMalloc(&s->dz, wr * wide * 4));
    SC(cudaMalloc(&s->dzh, wr * wide * 2));
    SC(cudaMalloc(&s->dz2, wr * wide * 4));
    SC(cudaMalloc(&s->dzh2, wr * wide * 2));
    SC(cudaMalloc(&s->idx, wr * sizeof(int)));
    SC(cudaMalloc(&s->loss, (size_t)1 << 20));
    SC(cudaStreamSynchronize(st));
#undef SC
    *out = s;
    return MDSX_OK;
}

void mdsx_surrogate_destroy(mdsx_surrogate* s) {
    if (!s) return;
    mdsx::internal::DeviceGuard guard(s->device);
    free_all(s);  // cudaFree waits for the device
    delete s;
}

const char* mdsx_surrogate_last_error(const mdsx_surrogate* s) { return s ? s->last_error.c_str() : "NULL surrogate"; }

int mdsx_surrogate_info(const mdsx_surrogate* s, int* ints, double* reals) {
    if (!s) return MDSX_EINVAL;
    if (ints) {
        ints[0] = s->n;
        ints[1] = s->p;
        ints[2] = s->k;
        ints[3] = s->width;
        ints[4] = s->layers;
        ints[5] = s->rows;
        ints[6] = s->max_rows;
        ints[7] = (int)std::min<long long>(s->adam_t, 0x7fffffff);
    }
    if (reals) {
        reals[0] = s->mu;
        reals[1] = s->inv_sigma;
        reals[2] = s->scale;
        reals[3] = s->tscale;
        reals[4] = s->inv_sigma_r;
    }
    return MDSX_OK;
}

int mdsx_surrogate_landmarks(const mdsx_surrogate* s, int* out) {
    if (!s || !out) return MDSX_EINVAL;
    mdsx::internal::DeviceGuard guard(s->engine->device);
    return cudaMemcpy(out, s->landmarks, s->k * sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess ? MDSX_OK
                                                                                                     : MDSX_ECUDA;
}

// which: 0 read the FP32 master weight and bias of `layer`, 1 write them (the
// BF16 copy is refreshed), 2 read the gradients of the last training step or
// of mdsx_surrogate_batch_gradient.
int mdsx_surrogate_parameters(mdsx_surrogate* s, int layer, int which, float* w, float* b) {
    if (!s) return MDSX_EINVAL;
    if (layer < 0 || layer > s->layers || which < 0 || which > 2 || !w || !b)
        return fail(s, MDSX_EINVAL, "surrogate_parameters: bad layer, mode or NULL buffer");
    mdsx::internal::DeviceGuard guard(s->engine->device);
    cudaStream_t st = s->engine->stream;
    const size_t nw = (size_t)s->fan_out[layer] * s->fan_in[layer], nb = s->fan_out[layer];
    float* dw = which == 2 ? s->gw[layer] : s->w[layer];
    float* db = which == 2 ? s->gb[layer] : s->b[layer];
    if (which == 1) {
        SURR_CUDA(s, cudaMemcpyAsync(dw, w, nw * 4, cudaMemcpyHostToDevice, st));
        SURR_CUDA(s, cudaMemcpyAsync(db, b, nb * 4, cudaMemcpyHostToDevice, st));
        to_bf16_kernel<<<grid_for((long long)nw), 256, 0, st>>>(dw, s->wh[layer], (long long)nw);
        SURR_CUDA(s, cudaGetLastError());
        int rc = pack_all(s, st);
        if (rc) return rc;
    } else {
        SURR_CUDA(s, cudaMemcpyAsync(w, dw, nw * 4, cudaMemcpyDeviceToHost, st));
        SURR_CUDA(s, cudaMemcpyAsync(b, db, nb * 4, cudaMemcpyDeviceToHost, st));
    }
    SURR_CUDA(s, cudaStreamSynchronize(st));
    return MDSX_OK;
}

// Harvest: `rows` training rows at randomly chosen locations of the state
// (locations, gradient), both host N x P row-major doubles. The gradient is
// the exact log-likelihood gradient at those locations.
int mdsx_surrogate_add_state(mdsx_surrogate* s, const double* locations, const double* gradient, int rows,
                             unsigned long long seed) {
    if (!s) return MDSX_EINVAL;
    if (!locations || !gradient || rows < 0) return fail(s, MDSX_EINVAL, "surrogate_add_state: bad argument");
    mdsx::internal::DeviceGuard guard(s->engine->device);
    cudaStream_t st = s->engine->stream;
    const size_t xb = (size_t)s->n * s->p * sizeof(double);
    double* d = nullptr;
    SURR_CUDA(s, cudaMalloc(&d, 2 * xb));
    int rc = MDSX_OK;
    if (cudaMemcpyAsync(d, locations, xb, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(d + (size_t)s->n * s->p, gradient, xb, cudaMemcpyHostToDevice, st) != cudaSuccess)
        rc = fail(s, MDSX_ECUDA, "surrogate_add_state: copy failed");
    if (!rc) rc = add_state(s, d, d + (size_t)s->n * s->p, rows, seed, st);
    cudaStreamSynchronize(st);
    cudaFree(d);
    return rc;
}

// Training rows [first, first + count) as FP32: features [count][2K] (the
// BF16 values), directions [count][K][P], targets [count][P]. NULL skips.
int mdsx_surrogate_training_rows(mdsx_surrogate* s, int first, int count, float* features, float* directions,
                                 float* targets) {
    if (!s) return MDSX_EINVAL;
    if (first < 0 || count < 0 || first + count > s->rows) return fail(s, MDSX_EINVAL, "surrogate_training_rows: range");
    mdsx::internal::DeviceGuard guard(s->engine->device);
    cudaStream_t st = s->engine->stream;
    if (features) {
        std::vector<bf16> tmp((size_t)count * s->in);
        SURR_CUDA(s, cudaMemcpyAsync(tmp.data(), s->t_feat + (size_t)first * s->in, tmp.size() * 2,
                                     cudaMemcpyDeviceToHost, st));
        SURR_CUDA(s, cudaStreamSynchronize(st));
        for (size_t i = 0; i < tmp.size(); ++i) features[i] = __bfloat162float(tmp[i]);
    }
    if (directions)
        SURR_CUDA(s, cudaMemcpyAsync(directions, s->t_dirs + (size_t)first * s->k * s->p,
                                     (size_t)count * s->k * s->p * 4, cudaMemcpyDeviceToHost, st));
    if (targets)
        SURR_CUDA(s, cudaMemcpyAsync(targets, s->t_target + (size_t)first * s->p, (size_t)count * s->p * 4,
                                     cudaMemcpyDeviceToHost, st));
    SURR_CUDA(s, cudaStreamSynchronize(st));
    return MDSX_OK;
}

}  // extern "C"

namespace mdsx {
namespace surr {
namespace {

// Target scale: RMS of the harvested gradient entries, fixed at the first training call.
int fix_target_scale(mdsx_surrogate* s, cudaStream_t st) {
    if (s->adam_t > 0) return MDSX_OK;
    std::vector<float> t((size_t)s->rows * s->p);
    SURR_CUDA(s, cudaMemcpyAsync(t.data(), s->t_target, t.size() * 4, cudaMemcpyDeviceToHost, st));
    SURR_CUDA(s, cudaStreamSynchronize(st));
    double sq = 0.0;
    for (float v : t) sq += (double)v * v;
    const double rms = std::sqrt(sq / std::max<size_t>(1, t.size()));
    s->tscale = rms > 0.0 && std::isfinite(rms) ? (float)rms : 1.0f;
    return MDSX_OK;
}

// Loss and parameter gradients of the batch whose row indices are at d_idx.
int batch_loss_and_gradients(mdsx_surrogate* s, const int* d_idx, int batch, float* d_loss, cudaStream_t st) {
    gather_rows_kernel<<<batch, 256, 0, st>>>(d_idx, batch, s->t_feat, s->in, s->t_dirs, s->t_target, s->k, s->p,
                                              s->a_feat, s->a_dirs, s->a_target);
    SURR_CUDA(s, cudaGetLastError());
    int rc = forward(s, batch, st);
    if (rc) return rc;
    SURR_CUDA(s, cudaMemsetAsync(d_loss, 0, sizeof(float), st));
    loss_kernel<<<grid_for((long long)batch * 32), 256, 0, st>>>(s->z[s->layers], s->k, s->a_dirs, s->a_target, batch,
                                                                   s->k, s->p, s->scale, 1.0f / s->tscale, s->dz,
                                                                   s->dzh, d_loss);
    SURR_CUDA(s, cudaGetLastError());
    return backward(s, batch, st);
}

int check_batch(mdsx_surrogate* s, int batch) {
    if (batch < 64 || batch % 64 || batch > s->work_rows)
        return fail(s, MDSX_EINVAL, "surrogate: batch must be a positive multiple of 64 and at most the work rows");
    if (s->rows < 1) return fail(s, MDSX_ESTATE, "surrogate: no training rows harvested");
    return MDSX_OK;
}

}  // namespace
}  // namespace surr
}  // namespace mdsx

extern "C" {

// `steps` Adam steps on batches of `batch` rows drawn uniformly (with
// replacement, seeded) from the harvested rows. loss_trace (optional, host)
// receives each step's mean squared error in target-scale units.
int mdsx_surrogate_train(mdsx_surrogate* s, int steps, int batch, double learning_rate, unsigned long long seed,
                         double* loss_trace) {
    if (!s) return MDSX_EINVAL;
    if (steps < 0 || !(learning_rate > 0.0)) return fail(s, MDSX_EINVAL, "surrogate_train: bad steps or learning rate");
    int rc = check_batch(s, batch);
    if (rc) return rc;
    mdsx::internal::DeviceGuard guard(s->engine->device);
    cudaStream_t st = s->engine->stream;
    if ((rc = fix_target_scale(s, st))) return rc;
    if (steps == 0) return MDSX_OK;
    std::mt19937_64 rng(seed);
    std::uniform_int_distribution<int> pick(0, s->rows - 1);
    std::vector<int> idx((size_t)steps * batch);
    for (int& v : idx) v = pick(rng);
    int* d_idx = nullptr;
    float* d_loss = nullptr;
    SURR_CUDA(s, cudaMalloc(&d_idx, idx.size() * sizeof(int)));
    if (cudaMalloc(&d_loss, (size_t)steps * sizeof(float)) != cudaSuccess) {
        cudaFree(d_idx);
        return fail(s, MDSX_ENOMEM, "surrogate_train: loss buffer");
    }
    if (cudaMemcpyAsync(d_idx, idx.data(), idx.size() * sizeof(int), cudaMemcpyHostToDevice, st) != cudaSuccess)
        rc = fail(s, MDSX_ECUDA, "surrogate_train: index copy");
    for (int t = 0; !rc && t < steps; ++t) {
        rc = batch_loss_and_gradients(s, d_idx + (size_t)t * batch, batch, d_loss + t, st);
        if (!rc) rc = adam_step(s, (float)learning_rate, st);
    }
    if (!rc) rc = pack_all(s, st);
    std::vector<float> losses(steps);
    if (!rc && cudaMemcpyAsync(losses.data(), d_loss, steps * sizeof(float), cudaMemcpyDeviceToHost, st) != cudaSuccess)
        rc = fail(s, MDSX_ECUDA, "surrogate_train: loss copy");
    if (cudaStreamSynchronize(st) != cudaSuccess && !rc) rc = fail(s, MDSX_ECUDA, "surrogate_train: synchronize");
    cudaFree(d_idx);
    cudaFree(d_loss);
    if (!rc && loss_trace)
        for (int t = 0; t < steps; ++t) loss_trace[t] = losses[t];
    return rc;
}

// Loss and parameter gradients (read back with mdsx_surrogate_parameters,
// which = 2) of the given training rows, without an update.
int mdsx_surrogate_batch_gradient(mdsx_surrogate* s, const int* rows, int count, double* loss) {
    if (!s) return MDSX_EINVAL;
    if (!rows || !loss) return fail(s, MDSX_EINVAL, "surrogate_batch_gradient: NULL argument");
    int rc = check_batch(s, count);
    if (rc) return rc;
    for (int r = 0; r < count; ++r)
        if (rows[r] < 0 || rows[r] >= s->rows) return fail(s, MDSX_EINVAL, "surrogate_batch_gradient: row out of range");
    mdsx::internal::DeviceGuard guard(s->engine->device);
    cudaStream_t st = s->engine->stream;
    if ((rc = fix_target_scale(s, st))) return rc;
    float h_loss = 0.f;
    SURR_CUDA(s, cudaMemcpyAsync(s->idx, rows, count * sizeof(int), cudaMemcpyHostToDevice, st));
    if ((rc = batch_loss_and_gradients(s, s->idx, count, s->loss, st))) return rc;
    SURR_CUDA(s, cudaMemcpyAsync(&h_loss, s->loss, sizeof(float), cudaMemcpyDeviceToHost, st));
    SURR_CUDA(s, cudaStreamSynchronize(st));
    *loss = h_loss;
    return MDSX_OK;
}

// Surrogate log-likelihood gradient at host locations (N x P) into host gradient (N x P).
int mdsx_surrogate_gradient(mdsx_surrogate* s, const double* locations, double* out) {
    if (!s) return MDSX_EINVAL;
    if (!locations || !out) return fail(s, MDSX_EINVAL, "surrogate_gradient: NULL argument");
    mdsx::internal::DeviceGuard guard(s->engine->device);
    cudaStream_t st = s->engine->stream;
    const size_t xb = (size_t)s->n * s->p * sizeof(double);
    double* d = nullptr;
    SURR_CUDA(s, cudaMalloc(&d, 2 * xb));
    int rc = MDSX_OK;
    if (cudaMemcpyAsync(d, locations, xb, cudaMemcpyHostToDevice, st) != cudaSuccess)
        rc = fail(s, MDSX_ECUDA, "surrogate_gradient: copy in");
    if (!rc) rc = gradient(s, d, d + (size_t)s->n * s->p, st);
    if (!rc && cudaMemcpyAsync(out, d + (size_t)s->n * s->p, xb, cudaMemcpyDeviceToHost, st) != cudaSuccess)
        rc = fail(s, MDSX_ECUDA, "surrogate_gradient: copy out");
    if (cudaStreamSynchronize(st) != cudaSuccess && !rc) rc = fail(s, MDSX_ECUDA, "surrogate_gradient: synchronize");
    cudaFree(d);
    return rc;
}

// Test hook for the tensor-core GEMM of the MLP: C = op(A) op(B) on host
// buffers, BF16 bit patterns in, FP32 out, on the current device. a_t / b_t
// select the stored layouts of mlp_gemm.cuh; m, n multiples of 64, k of 32.
int mdsx_test_gemm_bf16(int a_t, int b_t, int m, int n, int k, const unsigned short* a, const unsigned short* b,
                        float* c) {
    if (!a || !b || !c || m <= 0 || n <= 0 || k <= 0 || m % 64 || n % 64 || k % 32 || (a_t && !b_t))
        return MDSX_EINVAL;
    const size_t na = (size_t)m * k, nb = (size_t)k * n, nc = (size_t)m * n;
    void *da = nullptr, *db = nullptr, *dc = nullptr;
    int rc = MDSX_OK;
    if (cudaMalloc(&da, na * 2) != cudaSuccess || cudaMalloc(&db, nb * 2) != cudaSuccess ||
        cudaMalloc(&dc, nc * 4) != cudaSuccess)
        rc = MDSX_ENOMEM;
    if (!rc && (cudaMemcpy(da, a, na * 2, cudaMemcpyHostToDevice) != cudaSuccess ||
                cudaMemcpy(db, b, nb * 2, cudaMemcpyHostToDevice) != cudaSuccess))
        rc = MDSX_ECUDA;
    if (!rc) {
        mdsx::mlp::GemmArgs g{};
        g.a = static_cast<const bf16*>(da);
        g.b = static_cast<const bf16*>(db);
        g.lda = a_t ? m : k;
        g.ldb = b_t ? n : k;
        g.m = m;
        g.n = n;
        g.k = k;
        g.c = static_cast<float*>(dc);
        g.ldc = n;
        g.epilogue = mdsx::mlp::kStoreF32;
        const dim3 grid(n / mdsx::mlp::kBN, m / mdsx::mlp::kBM);
        if (!a_t && !b_t) mdsx::mlp::gemm_kernel<false, false><<<grid, mdsx::mlp::kGemmThreads>>>(g);
        else if (!a_t) mdsx::mlp::gemm_kernel<false, true><<<grid, mdsx::mlp::kGemmThreads>>>(g);
        else mdsx::mlp::gemm_kernel<true, true><<<grid, mdsx::mlp::kGemmThreads>>>(g);
        if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess ||
            cudaMemcpy(c, dc, nc * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = MDSX_ECUDA;
    }
    cudaFree(da);
    cudaFree(db);
    cudaFree(dc);
    return rc;
}

}  // extern "C"
