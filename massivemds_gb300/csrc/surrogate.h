// Gradient surrogate object shared by surrogate.cu and hmc.cu (not public ABI).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/mdsx.h"

struct mdsx_surrogate {
    mdsx_engine* engine = nullptr;
    int device = 0;                                   // the engine's GPU (destroy does not touch the engine)
    int n = 0, p = 0, k = 0, width = 0, layers = 0;  // locations, dimension, landmarks, hidden width, hidden layers
    int n_pad = 0;                                    // N rounded up to 64 (inference rows)
    int in = 0;                                       // 2K (input features)
    float mu = 0.f, inv_sigma = 1.f;                  // standardisation of the delta features
    float inv_sigma_r = 1.f;                          // scale of the residual features d - delta
    bool resid_fixed = false;                         // inv_sigma_r fixed (first harvested state)
    float scale = 1.f;                                // contraction scale
    float tscale = 1.f;                               // target scale (RMS of harvested gradients)
    int* landmarks = nullptr;                         // [K]
    float* dland = nullptr;                           // delta[i][l_k], [N][K] (missing pairs: 0)
    // layers: 0..layers-1 hidden (SiLU), layers = output (K, linear)
    std::vector<int> fan_in, fan_out;
    std::vector<float*> w, b, gw, gb, mw, vw, mb, vb;  // fp32 [out][in], [out]
    std::vector<__nv_bfloat16*> wh;                     // bf16 [out][in] (training GEMMs)
    __nv_bfloat16* wpack = nullptr;                     // all layers in the step kernel's chunk layout
    std::vector<long long> wofs;                        // element offset of each layer in wpack
    long long adam_t = 0;
    // training set
    int rows = 0, max_rows = 0;
    __nv_bfloat16* t_feat = nullptr;  // [max_rows][in]
    float* t_dirs = nullptr;          // [max_rows][K][P]
    float* t_target = nullptr;        // [max_rows][P]
    double target_sq = 0.0;           // running sum of squared target entries
    // work buffers sized for max(batch, n_pad) rows
    int work_rows = 0;
    __nv_bfloat16* a_feat = nullptr;  // [work_rows][in]
    float* a_dirs = nullptr;          // [work_rows][K][P]
    float* a_target = nullptr;        // [work_rows][P]
    std::vector<float*> z;            // per layer fp32 [work_rows][fan_out]
    std::vector<__nv_bfloat16*> h;    // per hidden layer bf16 [work_rows][width]
    float* dz = nullptr;              // fp32 [work_rows][max(width, K)]
    __nv_bfloat16* dzh = nullptr;     // bf16 copy
    float* dz2 = nullptr;
    __nv_bfloat16* dzh2 = nullptr;
    int* idx = nullptr;               // batch row indices
    float* loss = nullptr;
    std::string last_error;
};

namespace mdsx {
namespace surr {
// Leapfrog kick and drift with the surrogate gradient at x_in (one fused
// launch): mom += coef[0] (g - x Lambda), x_out = x_in + coef[1] mom, also into
// the engine's SoA location buffer; g_out (may be NULL) receives g. x_out must
// not alias x_in. lam: P x P row-major column precision.
int kick_drift(mdsx_surrogate* s, const double* x_in, double* x_out, double* mom, double* g_out, const double* coef,
               const double* lam, cudaStream_t stream);
// Surrogate likelihood gradient at locations d_x (N x P doubles, device) into
// d_out (N x P doubles, device), enqueued on `stream`.
int gradient(mdsx_surrogate* s, const double* d_x, double* d_out, cudaStream_t stream);
// Appends `rows` training rows sampled from state (d_x, d_grad) (device pointers).
int add_state(mdsx_surrogate* s, const double* d_x, const double* d_grad, int rows, unsigned long long seed,
              cudaStream_t stream);
}  // namespace surr
}  // namespace mdsx
