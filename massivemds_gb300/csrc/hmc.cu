// On-device Hamiltonian Monte Carlo for the MDS posterior.
//
// A C++/CUDA restatement of the reference's R sampler hmcsampler
// (R/Untitled.R:477-729 of MassiveMDS) over this engine's fused sweep:
//   potential U(x) = -(log-likelihood(x) + log matrix-normal prior(x))
//     log-likelihood as R/mds.R:24-28 assembles it; prior with row covariance
//     I_N and column precision Lambda (R/Untitled.R:68-95 with treeCov = I,
//     the case without a phylogeny, :531-540);
//   momentum ~ N(0, I); leapfrog with step eps and L steps (:509-510, :605-621);
//   Metropolis accept on the FP64 Hamiltonian difference (:626-640);
//   optional Metropolis step on the precision tau with the reflected uniform
//   proposal |U(tau - h, tau + h)| (:668-691);
//   optional Gibbs draw Lambda ~ Wishart(d0 + N, (T0 + X'X)^-1) with d0 = P,
//   T0 = I_P (:538-540, :694-700).
//
// Differences from the reference, all leaving the target distribution as the
// reference intends it:
//   - one likelihood gradient per leapfrog step: the reference's second
//     half-kick and the next step's first half-kick evaluate the gradient at
//     the same point (:612, :618); the value is reused here;
//   - after an accepted tau move or a Lambda draw the current potential is
//     recomputed; the reference keeps the stale value (:676-686, :694-700);
//   - the step size may be tuned during burn-in by dual averaging (Hoffman and
//     Gelman 2014, Algorithm 5) toward a target acceptance rate;
//   - optionally (no reference counterpart) a learned gradient surrogate
//     (surrogate.cu) drives the leapfrog steps after a harvest phase. Any
//     deterministic vector field in the kicks keeps leapfrog volume-preserving
//     and reversible, and the accept uses the exact potential at the proposal,
//     so the chain still targets the exact posterior. The first half-kick
//     uses the surrogate at the start point too, for reversibility.
//
// Everything per location stays on the GPU. Each leapfrog step is one fused
// sweep (likelihood + gradient) and one kick/drift kernel that also writes the
// sweep's location buffer; the L steps of a trajectory are captured once as a
// CUDA graph and relaunched. Momenta come from a counter-based Philox4x32-10
// generator (Salmon et al., SC'11) with the Box-Muller transform; all
// reductions are FP64 in a fixed order, so a chain is reproducible.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <random>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/mdsx.h"
#include "engine_internal.h"
#include "surrogate.h"

namespace mdsx {
namespace hmc {

constexpr int kMaxP = MDSX_MAX_DIMENSION;
constexpr int kReduceBlocks = 128;
constexpr int kReduceThreads = 256;
constexpr int kMaxReduce = kMaxP * kMaxP + 2;  // X'X entries + two scalars

struct Lambda {
    double m[kMaxP * kMaxP];  // column precision, row-major P x P
};

// ------------------------------------------------------------------ Philox

struct Philox {
    // Philox4x32 with 10 rounds: multipliers and Weyl key increments of the
    // published generator.
    __device__ static uint4 round(uint4 c, uint2 k) {
        const uint32_t m0 = 0xD2511F53u, m1 = 0xCD9E8D57u;
        const uint32_t hi0 = __umulhi(m0, c.x), lo0 = m0 * c.x;
        const uint32_t hi1 = __umulhi(m1, c.z), lo1 = m1 * c.z;
        return make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    }
    __device__ static uint4 generate(uint4 ctr, uint2 key) {
#pragma unroll
        for (int r = 0; r < 10; ++r) {
            ctr = round(ctr, key);
            key.x += 0x9E3779B9u;
            key.y += 0xBB67AE85u;
        }
        return ctr;
    }
};

__device__ inline double u01(uint32_t a, uint32_t b) {
    // 53-bit uniform in (0, 1]
    const unsigned long long v = ((unsigned long long)(a >> 5) << 26) | (b >> 6);
    return ((double)v + 1.0) * (1.0 / 9007199254740992.0);
}

// p[k] ~ N(0, 1) for k < count, from counter (stream, k/2) and the seed.
__global__ void normal_kernel(double* __restrict__ p, long long count, unsigned long long seed,
                              unsigned long long stream) {
    for (long long k = 2LL * (blockIdx.x * (long long)blockDim.x + threadIdx.x); k < count;
         k += 2LL * gridDim.x * blockDim.x) {
        const uint4 ctr = make_uint4((uint32_t)(k >> 1), (uint32_t)((k >> 1) >> 32), (uint32_t)stream,
                                     (uint32_t)(stream >> 32));
        const uint4 r = Philox::generate(ctr, make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)));
        const double rad = sqrt(-2.0 * log(u01(r.x, r.y)));
        const double ang = 6.283185307179586476925 * u01(r.z, r.w);
        p[k] = rad * cos(ang);
        if (k + 1 < count) p[k + 1] = rad * sin(ang);
    }
}

// ----------------------------------------------------- leapfrog kernels

// p += a * (g_lik - x Lambda); x += b * p; writes x into the sweep's SoA
// location buffer (float or double). a and b are read from device memory so
// a captured graph follows step-size changes.
template <typename C, int P>
__global__ void kick_drift_kernel(double* __restrict__ x, double* __restrict__ p, const double* __restrict__ g_lik,
                                  const Lambda lam, const double* __restrict__ coef, int n, C* __restrict__ soa,
                                  int x_ld) {
    const double a = coef[0], b = coef[1];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double xi[P], pi[P];
#pragma unroll
        for (int q = 0; q < P; ++q) {
            xi[q] = x[(size_t)i * P + q];
            pi[q] = p[(size_t)i * P + q];
        }
#pragma unroll
        for (int q = 0; q < P; ++q) {
            double prior = 0.0;
#pragma unroll
            for (int r = 0; r < P; ++r) prior += xi[r] * lam.m[r * P + q];
            pi[q] += a * (g_lik[(size_t)i * P + q] - prior);
        }
#pragma unroll
        for (int q = 0; q < P; ++q) {
            xi[q] += b * pi[q];
            p[(size_t)i * P + q] = pi[q];
            x[(size_t)i * P + q] = xi[q];
            soa[(size_t)q * x_ld + i] = (C)xi[q];
        }
    }
}

// Fixed-order FP64 partial sums per block. mode 0: 0.5*|p|^2 into out[0].
// mode 1: X'X (P*P entries) and sum_i x_i' Lambda x_i into out[P*P].
template <int P>
__global__ void __launch_bounds__(kReduceThreads) reduce_kernel(int mode, const double* __restrict__ v, int n,
                                                                const Lambda lam, double* __restrict__ partial) {
    constexpr int K = P * P + 1;
    double acc[K];
#pragma unroll
    for (int k = 0; k < K; ++k) acc[k] = 0.0;
    for (int i = blockIdx.x * kReduceThreads + threadIdx.x; i < n; i += kReduceBlocks * kReduceThreads) {
        double xi[P];
#pragma unroll
        for (int q = 0; q < P; ++q) xi[q] = v[(size_t)i * P + q];
        if (mode == 0) {
#pragma unroll
            for (int q = 0; q < P; ++q) acc[0] += 0.5 * xi[q] * xi[q];
        } else {
#pragma unroll
            for (int r = 0; r < P; ++r)
#pragma unroll
                for (int q = 0; q < P; ++q) {
                    acc[r * P + q] += xi[r] * xi[q];
                    acc[P * P] += xi[r] * lam.m[r * P + q] * xi[q];
                }
        }
    }
    __shared__ double sh[kReduceThreads];
    for (int k = 0; k < K; ++k) {
        sh[threadIdx.x] = acc[k];
        __syncthreads();
        for (int s = kReduceThreads / 2; s > 0; s >>= 1) {
            if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
            __syncthreads();
        }
        if (threadIdx.x == 0) partial[(size_t)blockIdx.x * kMaxReduce + k] = sh[0];
        __syncthreads();
    }
}

// out[k] = sum over blocks of partial[block][k], blocks in order.
__global__ void reduce_final_kernel(const double* __restrict__ partial, int count, double* __restrict__ out) {
    const int k = threadIdx.x;
    if (k >= count) return;
    double s = 0.0;
    for (int b = 0; b < kReduceBlocks; ++b) s += partial[(size_t)b * kMaxReduce + k];
    out[k] = s;
}

// Traced functionals: distances between fixed pairs and norms of fixed locations.
template <int P>
__global__ void functionals_kernel(const double* __restrict__ x, const int* __restrict__ pairs, int n_pairs,
                                   const int* __restrict__ locs, int n_locs, double* __restrict__ out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n_pairs) {
        const int i = pairs[2 * k], j = pairs[2 * k + 1];
        double s = 0.0;
#pragma unroll
        for (int q = 0; q < P; ++q) {
            const double d = x[(size_t)i * P + q] - x[(size_t)j * P + q];
            s += d * d;
        }
        out[k] = sqrt(s);
    } else if (k < n_pairs + n_locs) {
        const int i = locs[k - n_pairs];
        double s = 0.0;
#pragma unroll
        for (int q = 0; q < P; ++q) s += x[(size_t)i * P + q] * x[(size_t)i * P + q];
        out[k] = sqrt(s);
    }
}

}  // namespace hmc
}  // namespace mdsx

// ------------------------------------------------------------- host side

namespace mdsx {
namespace hmc {
namespace {

using internal::DeviceGuard;
using internal::fail;

// Compile-time dispatch of the per-P kernels.
template <int P>
struct Kernels {
    static cudaError_t kick_drift(double* x, double* p, const double* g, const Lambda& lam, const double* coef, int n,
                                  void* soa, bool f32, int x_ld, cudaStream_t s) {
        const int grid = std::max(1, std::min(1024, (n + 255) / 256));
        if (f32)
            kick_drift_kernel<float, P><<<grid, 256, 0, s>>>(x, p, g, lam, coef, n, static_cast<float*>(soa), x_ld);
        else
            kick_drift_kernel<double, P><<<grid, 256, 0, s>>>(x, p, g, lam, coef, n, static_cast<double*>(soa), x_ld);
        return cudaGetLastError();
    }
    static cudaError_t reduce(int mode, const double* v, int n, const Lambda& lam, double* partial, double* out,
                              cudaStream_t s) {
        reduce_kernel<P><<<kReduceBlocks, kReduceThreads, 0, s>>>(mode, v, n, lam, partial);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        reduce_final_kernel<<<1, 128, 0, s>>>(partial, P * P + 1, out);
        return cudaGetLastError();
    }
    static cudaError_t functionals(const double* x, const int* pairs, int n_pairs, const int* locs, int n_locs,
                                   double* out, cudaStream_t s) {
        const int total = n_pairs + n_locs;
        if (total == 0) return cudaSuccess;
        functionals_kernel<P><<<(total + 127) / 128, 128, 0, s>>>(x, pairs, n_pairs, locs, n_locs, out);
        return cudaGetLastError();
    }
};

template <typename F>
auto with_p(int p, F&& f) -> decltype(f.template run<1>()) {
    switch (p) {
        case 1: return f.template run<1>();
        case 2: return f.template run<2>();
        case 3: return f.template run<3>();
        case 4: return f.template run<4>();
        case 5: return f.template run<5>();
        case 6: return f.template run<6>();
        case 7: return f.template run<7>();
        case 8: return f.template run<8>();
        case 9: return f.template run<9>();
        case 10: return f.template run<10>();
        default: return cudaErrorInvalidValue;
    }
}

struct KickDriftF {
    double *x, *p;
    const double* g;
    const Lambda& lam;
    const double* coef;
    int n;
    void* soa;
    bool f32;
    int x_ld;
    cudaStream_t s;
    template <int P>
    cudaError_t run() const {
        return Kernels<P>::kick_drift(x, p, g, lam, coef, n, soa, f32, x_ld, s);
    }
};
struct ReduceF {
    int mode;
    const double* v;
    int n;
    const Lambda& lam;
    double *partial, *out;
    cudaStream_t s;
    template <int P>
    cudaError_t run() const {
        return Kernels<P>::reduce(mode, v, n, lam, partial, out, s);
    }
};
struct FunctionalsF {
    const double* x;
    const int* pairs;
    int n_pairs;
    const int* locs;
    int n_locs;
    double* out;
    cudaStream_t s;
    template <int P>
    cudaError_t run() const {
        return Kernels<P>::functionals(x, pairs, n_pairs, locs, n_locs, out, s);
    }
};

// Cholesky of a P x P symmetric positive-definite matrix (row-major, lower L).
bool cholesky(const double* a, int p, double* l) {
    std::memset(l, 0, sizeof(double) * p * p);
    for (int i = 0; i < p; ++i)
        for (int j = 0; j <= i; ++j) {
            double s = a[i * p + j];
            for (int k = 0; k < j; ++k) s -= l[i * p + k] * l[j * p + k];
            if (i == j) {
                if (!(s > 0.0)) return false;
                l[i * p + i] = std::sqrt(s);
            } else {
                l[i * p + j] = s / l[j * p + j];
            }
        }
    return true;
}

bool spd_inverse(const double* a, int p, double* inv) {
    double l[kMaxP * kMaxP], li[kMaxP * kMaxP] = {};
    if (!cholesky(a, p, l)) return false;
    for (int c = 0; c < p; ++c)  // solve L y = e_c by forward substitution, column c of L^-1
        for (int i = 0; i < p; ++i) {
            double s = (i == c) ? 1.0 : 0.0;
            for (int k = 0; k < i; ++k) s -= l[i * p + k] * li[k * p + c];
            li[i * p + c] = s / l[i * p + i];
        }
    for (int i = 0; i < p; ++i)  // inv = L^-T L^-1
        for (int j = 0; j < p; ++j) {
            double s = 0.0;
            for (int k = 0; k < p; ++k) s += li[k * p + i] * li[k * p + j];
            inv[i * p + j] = s;
        }
    return true;
}

double log_det_spd(const double* a, int p) {
    double l[kMaxP * kMaxP];
    if (!cholesky(a, p, l)) return NAN;
    double s = 0.0;
    for (int i = 0; i < p; ++i) s += 2.0 * std::log(l[i * p + i]);
    return s;
}

// Wishart(df, scale) by the Bartlett decomposition: W = (L A)(L A)', L L' = scale,
// A lower triangular with A_ii = sqrt(chi2(df - i)), A_ij ~ N(0, 1) below.
bool wishart(std::mt19937_64& rng, double df, const double* scale, int p, double* out) {
    double l[kMaxP * kMaxP], a[kMaxP * kMaxP] = {}, la[kMaxP * kMaxP] = {};
    if (!cholesky(scale, p, l)) return false;
    std::normal_distribution<double> nrm(0.0, 1.0);
    for (int i = 0; i < p; ++i) {
        std::gamma_distribution<double> g(0.5 * (df - i), 2.0);
        a[i * p + i] = std::sqrt(g(rng));
        for (int j = 0; j < i; ++j) a[i * p + j] = nrm(rng);
    }
    for (int i = 0; i < p; ++i)
        for (int j = 0; j < p; ++j) {
            double s = 0.0;
            for (int k = 0; k < p; ++k) s += l[i * p + k] * a[k * p + j];
            la[i * p + j] = s;
        }
    for (int i = 0; i < p; ++i)
        for (int j = 0; j < p; ++j) {
            double s = 0.0;
            for (int k = 0; k < p; ++k) s += la[i * p + k] * la[j * p + k];
            out[i * p + j] = s;
        }
    return true;
}

}  // namespace
}  // namespace hmc
}  // namespace mdsx

namespace mdsx {
namespace hmc {
namespace {

constexpr int kTraceBase = MDSX_HMC_TRACE_BASE;

struct Chain {
    mdsx_engine* e;
    mdsx_hmc_config cfg;
    int n, p, n_func;
    cudaStream_t s;
    double *x0 = nullptr, *xp = nullptr, *mom = nullptr, *gl0 = nullptr, *coef = nullptr;
    double *partial = nullptr, *red_k0 = nullptr, *red_k = nullptr, *red_q = nullptr, *func = nullptr;
    int *pairs = nullptr, *locs = nullptr;
    double* h = nullptr;  // pinned: [0..3] sums, [4] K0, [5] K*, [6..] X'X* and Q*, then functionals
    double *gs0 = nullptr, *gsur = nullptr;  // surrogate gradients at x0 and at the proposal
    double* xq = nullptr;                    // second position buffer of surrogate trajectories
    double* xfinal = nullptr;                // the buffer holding the last trajectory's proposal
    cudaGraph_t graph = nullptr, graph_s = nullptr;
    cudaGraphExec_t exec = nullptr, exec_s = nullptr;
    bool graph_dirty = true, graph_s_dirty = true;
    Lambda lam{};
    double logdet_lam = 0.0;
    double eps = 0.0;
    std::mt19937_64 rng;
    long long sweeps = 0;

    double* h_sums() { return h; }
    double* h_k0() { return h + 4; }
    double* h_k() { return h + 5; }
    double* h_q() { return h + 6; }  // P*P entries of X'X then sum x' Lambda x
    double* h_func() { return h + 6 + kMaxReduce; }

    ~Chain() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (exec_s) cudaGraphExecDestroy(exec_s);
        if (graph_s) cudaGraphDestroy(graph_s);
        cudaFree(gs0);
        cudaFree(gsur);
        cudaFree(xq);
        cudaFree(x0);
        cudaFree(xp);
        cudaFree(mom);
        cudaFree(gl0);
        cudaFree(coef);
        cudaFree(partial);
        cudaFree(red_k0);
        cudaFree(red_k);
        cudaFree(red_q);
        cudaFree(func);
        cudaFree(pairs);
        cudaFree(locs);
        if (h) cudaFreeHost(h);
    }

    int alloc() {
        const size_t xb = (size_t)n * p * sizeof(double);
        MDSX_CUDA(e, cudaMalloc(&x0, xb));
        MDSX_CUDA(e, cudaMalloc(&xp, xb));
        MDSX_CUDA(e, cudaMalloc(&mom, xb));
        MDSX_CUDA(e, cudaMalloc(&gl0, xb));
        MDSX_CUDA(e, cudaMalloc(&coef, 6 * sizeof(double)));
        if (cfg.surrogate) {
            MDSX_CUDA(e, cudaMalloc(&gs0, xb));
            MDSX_CUDA(e, cudaMalloc(&gsur, xb));
            MDSX_CUDA(e, cudaMalloc(&xq, xb));
        }
        MDSX_CUDA(e, cudaMalloc(&partial, (size_t)kReduceBlocks * kMaxReduce * sizeof(double)));
        MDSX_CUDA(e, cudaMalloc(&red_k0, kMaxReduce * sizeof(double)));
        MDSX_CUDA(e, cudaMalloc(&red_k, kMaxReduce * sizeof(double)));
        MDSX_CUDA(e, cudaMalloc(&red_q, kMaxReduce * sizeof(double)));
        MDSX_CUDA(e, cudaMalloc(&func, std::max(1, n_func) * sizeof(double)));
        MDSX_CUDA(e, cudaMalloc(&pairs, std::max(1, 2 * cfg.n_traced_pairs) * sizeof(int)));
        MDSX_CUDA(e, cudaMalloc(&locs, std::max(1, cfg.n_traced_locations) * sizeof(int)));
        MDSX_CUDA(e, cudaMallocHost(&h, (6 + kMaxReduce + std::max(1, n_func)) * sizeof(double)));
        if (cfg.n_traced_pairs)
            MDSX_CUDA(e, cudaMemcpy(pairs, cfg.traced_pairs, 2 * cfg.n_traced_pairs * sizeof(int),
                                    cudaMemcpyHostToDevice));
        if (cfg.n_traced_locations)
            MDSX_CUDA(e, cudaMemcpy(locs, cfg.traced_locations, cfg.n_traced_locations * sizeof(int),
                                    cudaMemcpyHostToDevice));
        return MDSX_OK;
    }

    int set_coef() {
        const double c[6] = {0.5 * eps, eps, eps, eps, 0.5 * eps, 0.0};
        MDSX_CUDA(e, cudaMemcpyAsync(coef, c, sizeof c, cudaMemcpyHostToDevice, s));
        MDSX_CUDA(e, cudaStreamSynchronize(s));  // c lives on the host stack
        return MDSX_OK;
    }

    double log_likelihood(double sum_of_increments) const {
        // R/mds.R:24-28
        const double obs = (double)n * (double)(n - 1) / 2.0;
        return 0.5 * (std::log(e->tau) - std::log(2.0 * M_PI)) * obs - sum_of_increments;
    }
    double log_prior(double q) const {
        // R/Untitled.R:68-95 with U = I_N, V = Lambda^-1
        return -0.5 * q - 0.5 * (double)n * p * std::log(2.0 * M_PI) + 0.5 * (double)n * logdet_lam;
    }

    int kick_drift(double* x, const double* g, const double* c) {
        MDSX_CUDA(e, with_p(p, KickDriftF{x, mom, g, lam, c, n, e->d_x[e->xcur], e->x_f32, e->x_ld, s}));
        return MDSX_OK;
    }
    int reduce(int mode, const double* v, double* out) {
        MDSX_CUDA(e, with_p(p, ReduceF{mode, v, n, lam, partial, out, s}));
        return MDSX_OK;
    }

    // The trajectory from x0 (momentum already drawn): xp, mom end at the
    // proposal; sums, K* and X'X*, Q* land in the pinned host buffer. With
    // `surr` the kicks use the surrogate gradient (gs0 at x0, gsur after each
    // drift) and one exact sweep at the proposal gives its potential.
    int enqueue_trajectory(bool surr) {
        const int L = cfg.leapfrog_steps;
        MDSX_CUDA(e, cudaMemcpyAsync(xp, x0, (size_t)n * p * sizeof(double), cudaMemcpyDeviceToDevice, s));
        int rc = kick_drift(xp, surr ? gs0 : gl0, coef);
        xfinal = xp;
        if (surr) {
            // fused surrogate steps: positions ping-pong between xp and xq
            double* cur = xp;
            double* nxt = xq;
            for (int k = 1; !rc && k <= L; ++k) {
                rc = surr::kick_drift(cfg.surrogate, cur, nxt, mom, k == L ? gsur : nullptr, k < L ? coef + 2 : coef + 4,
                                      lam.m, s);
                if (rc) e->last_error = cfg.surrogate->last_error;
                std::swap(cur, nxt);
            }
            xfinal = cur;
            if (!rc) rc = internal::enqueue_sweep(e);  // exact potential at the proposal
        } else {
            // with the unordered-pair schedule the sweep's finish kernel applies the
            // kick/drift to the rows it completes (one launch less per step)
            const bool fused = e->schedule == MDSX_SWEEP_PAIRS && p <= mdsx::kPairMaxP;
            mdsx::PairLeapfrog lf{};
            if (fused) {
                lf.x = xp;
                lf.mom = mom;
                lf.soa = e->d_x[e->xcur];
                lf.x_ld = e->x_ld;
                lf.soa_f32 = e->x_f32 ? 1 : 0;
                for (int r = 0; r < p; ++r)
                    for (int q = 0; q < p; ++q) lf.lam[r * p + q] = lam.m[r * p + q];
            }
            for (int k = 1; !rc && k <= L; ++k) {
                const double* ck = k < L ? coef + 2 : coef + 4;
                if (fused) {
                    lf.coef = ck;
                    rc = internal::enqueue_sweep_leapfrog(e, lf);
                } else {
                    rc = internal::enqueue_sweep(e);
                    if (!rc) rc = kick_drift(xp, e->d_grad[e->gcur], ck);
                }
            }
        }
        if (!rc) rc = reduce(0, mom, red_k);
        if (!rc) rc = reduce(1, xfinal, red_q);
        if (rc) return rc;
        MDSX_CUDA(e, cudaMemcpyAsync(h_sums(), e->d_out, 4 * sizeof(double), cudaMemcpyDeviceToHost, s));
        MDSX_CUDA(e, cudaMemcpyAsync(h_k(), red_k, sizeof(double), cudaMemcpyDeviceToHost, s));
        MDSX_CUDA(e, cudaMemcpyAsync(h_q(), red_q, (p * p + 1) * sizeof(double), cudaMemcpyDeviceToHost, s));
        return MDSX_OK;
    }

    int run_trajectory(bool surr) {
        if (!cfg.use_graph) return enqueue_trajectory(surr);
        xfinal = (surr && cfg.leapfrog_steps % 2 == 1) ? xq : xp;  // as enqueue_trajectory leaves it
        cudaGraph_t& gr = surr ? graph_s : graph;
        cudaGraphExec_t& ex = surr ? exec_s : exec;
        bool& dirty = surr ? graph_s_dirty : graph_dirty;
        if (dirty) {
            if (ex) cudaGraphExecDestroy(ex);
            if (gr) cudaGraphDestroy(gr);
            ex = nullptr;
            gr = nullptr;
            MDSX_CUDA(e, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
            const int rc = enqueue_trajectory(surr);
            cudaGraph_t g = nullptr;
            const cudaError_t ce = cudaStreamEndCapture(s, &g);
            if (rc) {
                if (g) cudaGraphDestroy(g);
                return rc;
            }
            MDSX_CUDA(e, ce);
            gr = g;
            MDSX_CUDA(e, cudaGraphInstantiate(&ex, gr, 0));
            dirty = false;
        }
        MDSX_CUDA(e, cudaGraphLaunch(ex, s));
        return MDSX_OK;
    }

    int check_device_error() {
        int dev_err = 0;
        std::memcpy(&dev_err, &h_sums()[3], sizeof(int));
        if (dev_err) return fail(e, MDSX_ETIMEOUT, "a bounded device wait in the sweep kernel timed out");
        return MDSX_OK;
    }

    // Sweep at the engine's current locations; returns the log-likelihood.
    int sweep_loglik(double* loglik) {
        int rc = internal::enqueue_sweep(e);
        if (rc) return rc;
        ++sweeps;
        MDSX_CUDA(e, cudaMemcpyAsync(h_sums(), e->d_out, 4 * sizeof(double), cudaMemcpyDeviceToHost, s));
        MDSX_CUDA(e, cudaStreamSynchronize(s));
        rc = check_device_error();
        if (rc) return rc;
        *loglik = log_likelihood(h_sums()[2]);
        return MDSX_OK;
    }

    int set_lambda(const double* m) {
        std::memset(&lam, 0, sizeof lam);
        std::memcpy(lam.m, m, sizeof(double) * p * p);
        logdet_lam = log_det_spd(m, p);
        if (!std::isfinite(logdet_lam)) return fail(e, MDSX_EINVAL, "trait precision is not positive definite");
        graph_dirty = true;
        graph_s_dirty = true;
        return MDSX_OK;
    }
};

}  // namespace
}  // namespace hmc
}  // namespace mdsx

using mdsx::hmc::Chain;

namespace mdsx {
namespace hmc {
namespace {

// Chain checkpoint: a fixed header, then s0 (P*P), Lambda (P*P), x0 (N*P),
// gl0 (N*P) and the host generator's state as text (std::mt19937_64 << ).
constexpr char kCkptMagic[8] = {'M', 'D', 'S', 'X', 'H', 'M', 'C', '2'};
struct CkptHeader {
    char magic[8];
    int32_t n, p;
    uint64_t seed;
    int64_t next_iteration;
    double tau, eps, hbar, log_eps_bar, loglik0, logprior0, u0;
    int32_t rng_len, pad;
    double precision_half_width;  // the precision proposal's (adapted) half-width
    int64_t reserved;
};
static_assert(sizeof(CkptHeader) == 112, "checkpoint header layout");

struct CkptState {
    CkptHeader h{};
    std::vector<double> s0, lambda, x0, gl0;
    std::string rng;
};

size_t ckpt_bytes(const CkptState& c) {
    return sizeof(CkptHeader) + 8 * (c.s0.size() + c.lambda.size() + c.x0.size() + c.gl0.size()) + c.rng.size();
}

bool ckpt_read(const void* src, size_t bytes, int n, int p, CkptState* out) {
    if (!src || bytes < sizeof(CkptHeader)) return false;
    const unsigned char* b = static_cast<const unsigned char*>(src);
    std::memcpy(&out->h, b, sizeof(CkptHeader));
    if (std::memcmp(out->h.magic, kCkptMagic, 8) != 0 || out->h.n != n || out->h.p != p || out->h.rng_len < 0 ||
        out->h.rng_len > 8192)
        return false;
    const size_t pp = (size_t)p * p, np = (size_t)n * p;
    if (bytes != sizeof(CkptHeader) + 8 * (2 * pp + 2 * np) + (size_t)out->h.rng_len) return false;
    size_t off = sizeof(CkptHeader);
    auto take = [&](std::vector<double>& v, size_t count) {
        v.resize(count);
        std::memcpy(v.data(), b + off, 8 * count);
        off += 8 * count;
    };
    take(out->s0, pp);
    take(out->lambda, pp);
    take(out->x0, np);
    take(out->gl0, np);
    out->rng.assign(reinterpret_cast<const char*>(b + off), (size_t)out->h.rng_len);
    return true;
}

void ckpt_write(const CkptState& c, void* dst) {
    unsigned char* b = static_cast<unsigned char*>(dst);
    std::memcpy(b, &c.h, sizeof(CkptHeader));
    size_t off = sizeof(CkptHeader);
    for (const std::vector<double>* v : {&c.s0, &c.lambda, &c.x0, &c.gl0}) {
        std::memcpy(b + off, v->data(), 8 * v->size());
        off += 8 * v->size();
    }
    std::memcpy(b + off, c.rng.data(), c.rng.size());
}

}  // namespace
}  // namespace hmc
}  // namespace mdsx

extern "C" int mdsx_hmc_run(mdsx_engine* e, const mdsx_hmc_config* cfg, const double* initial_locations,
                            double* trace, double* final_locations, mdsx_hmc_stats* stats) {
    using namespace mdsx::hmc;
    using mdsx::internal::fail;
    if (!e) return MDSX_EINVAL;
    if (!cfg || !initial_locations || !trace) return fail(e, MDSX_EINVAL, "hmc: NULL argument");
    if (cfg->iterations < 1 || cfg->burn_in < 0 || (!cfg->resume && !cfg->checkpoint && cfg->burn_in > cfg->iterations) ||
        cfg->leapfrog_steps < 1 ||
        !(cfg->step_size > 0.0) || cfg->n_traced_pairs < 0 || cfg->n_traced_locations < 0)
        return fail(e, MDSX_EINVAL, "hmc: bad configuration");
    if ((cfg->n_traced_pairs && !cfg->traced_pairs) || (cfg->n_traced_locations && !cfg->traced_locations))
        return fail(e, MDSX_EINVAL, "hmc: traced index arrays are NULL");
    for (int k = 0; k < 2 * cfg->n_traced_pairs; ++k)
        if (cfg->traced_pairs[k] < 0 || cfg->traced_pairs[k] >= e->n) return fail(e, MDSX_EINVAL, "hmc: traced pair out of range");
    for (int k = 0; k < cfg->n_traced_locations; ++k)
        if (cfg->traced_locations[k] < 0 || cfg->traced_locations[k] >= e->n)
            return fail(e, MDSX_EINVAL, "hmc: traced location out of range");
    if (!e->data_set) return fail(e, MDSX_ESTATE, "hmc: setPairwiseData has not been called");
    if (e->rows != e->n) return fail(e, MDSX_EUNSUPPORTED, "hmc: needs an engine over the whole matrix");
    if (e->dd) return fail(e, MDSX_EUNSUPPORTED, "hmc: not built for double-float pair math");
    if (!(e->tau > 0.0)) return fail(e, MDSX_ESTATE, "hmc: precision (setParameters) not set");
    if (cfg->learn_precision && !(cfg->precision_half_width > 0.0))
        return fail(e, MDSX_EINVAL, "hmc: precision_half_width must be > 0");
    if (cfg->adapt_step_size && !(cfg->target_accept > 0.0 && cfg->target_accept < 1.0))
        return fail(e, MDSX_EINVAL, "hmc: target_accept must be in (0, 1)");
    if (cfg->surrogate && (cfg->resume || cfg->checkpoint))
        return fail(e, MDSX_EUNSUPPORTED, "hmc: checkpoint and resume are for exact-gradient chains");
    if (cfg->checkpoint && cfg->checkpoint_capacity < MDSX_HMC_CHECKPOINT_BYTES(e->n, e->p))
        return fail(e, MDSX_EINVAL, "hmc: checkpoint capacity below MDSX_HMC_CHECKPOINT_BYTES(N, P)");
    CkptState resume_state;
    if (cfg->resume) {
        if (!ckpt_read(cfg->resume, cfg->resume_bytes, e->n, e->p, &resume_state))
            return fail(e, MDSX_EINVAL, "hmc: resume data is not a checkpoint of a chain with these dimensions");
        if (resume_state.h.seed != cfg->seed) return fail(e, MDSX_EINVAL, "hmc: resume with the chain's own seed");
        if (!(resume_state.h.tau > 0.0) || !(resume_state.h.eps > 0.0))
            return fail(e, MDSX_EINVAL, "hmc: checkpoint holds a bad precision or step size");
    }
    if (cfg->surrogate) {
        if (cfg->surrogate->engine != e) return fail(e, MDSX_EINVAL, "hmc: the surrogate belongs to another engine");
        if (cfg->harvest_iterations < 0 || cfg->harvest_iterations > cfg->iterations || cfg->harvest_rows < 0 ||
            cfg->harvest_start < 0 ||
            cfg->train_steps < 0 || cfg->fallback_window < 1 || !(cfg->fallback_accept >= 0.0 && cfg->fallback_accept <= 1.0))
            return fail(e, MDSX_EINVAL, "hmc: bad surrogate configuration");
        if (cfg->train_steps > 0 && !(cfg->train_learning_rate > 0.0))
            return fail(e, MDSX_EINVAL, "hmc: train_learning_rate must be > 0");
    }

    mdsx::internal::DeviceGuard guard(e->device);
    Chain c;
    c.e = e;
    c.cfg = *cfg;
    c.n = e->n;
    c.p = e->p;
    c.n_func = cfg->n_traced_pairs + cfg->n_traced_locations;
    c.s = e->stream;
    c.rng.seed(cfg->seed ^ 0x5DEECE66DULL);
    c.eps = cfg->step_size;
    const long long it0 = cfg->resume ? resume_state.h.next_iteration : 0;
    double tau_hw = cfg->precision_half_width;  // the precision proposal's half-width (adapted in burn-in)
    if (cfg->resume) {
        std::istringstream in(resume_state.rng);
        in >> c.rng;
        if (in.fail()) return fail(e, MDSX_EINVAL, "hmc: checkpoint holds a bad generator state");
        c.eps = resume_state.h.eps;
        e->tau = resume_state.h.tau;
        if (resume_state.h.precision_half_width > 0.0) tau_hw = resume_state.h.precision_half_width;
        e->sum_known = e->grad_known = false;
    }
    int rc = c.alloc();
    if (rc) return rc;
    const int n = c.n, p = c.p;
    const int cols = kTraceBase + c.n_func;

    // Lambda = I_P (R/Untitled.R:537-540 without a tree: traitVcv = diag(P)), or the checkpoint's.
    if (cfg->resume) {
        if ((rc = c.set_lambda(resume_state.lambda.data()))) return rc;
    } else {
        double eye[kMaxP * kMaxP] = {};
        for (int q = 0; q < p; ++q) eye[q * p + q] = 1.0;
        if ((rc = c.set_lambda(eye))) return rc;
    }
    if ((rc = c.set_coef())) return rc;

    // Initial state: x0, its likelihood gradient, potential and X'X (from the
    // checkpoint when resuming, so the continued chain is the same chain).
    double loglik0 = 0.0, logprior0 = 0.0, u0 = 0.0;
    std::vector<double> s0;
    if (cfg->resume) {
        MDSX_CUDA(e, cudaMemcpyAsync(c.x0, resume_state.x0.data(), (size_t)n * p * sizeof(double),
                                     cudaMemcpyHostToDevice, c.s));
        MDSX_CUDA(e, cudaMemcpyAsync(c.gl0, resume_state.gl0.data(), (size_t)n * p * sizeof(double),
                                     cudaMemcpyHostToDevice, c.s));
        MDSX_CUDA(e, mdsx::convert_locations(c.x0, n, p, e->d_x[e->xcur], e->x_ld, e->x_f32, c.s));
        MDSX_CUDA(e, cudaStreamSynchronize(c.s));
        loglik0 = resume_state.h.loglik0;
        logprior0 = resume_state.h.logprior0;
        u0 = resume_state.h.u0;
        s0 = resume_state.s0;
    } else {
        MDSX_CUDA(e, cudaMemcpyAsync(c.x0, initial_locations, (size_t)n * p * sizeof(double), cudaMemcpyHostToDevice,
                                     c.s));
        MDSX_CUDA(e, mdsx::convert_locations(c.x0, n, p, e->d_x[e->xcur], e->x_ld, e->x_f32, c.s));
        if ((rc = c.sweep_loglik(&loglik0))) return rc;
        MDSX_CUDA(e, cudaMemcpyAsync(c.gl0, e->d_grad[e->gcur], (size_t)n * p * sizeof(double),
                                     cudaMemcpyDeviceToDevice, c.s));
        if ((rc = c.reduce(1, c.x0, c.red_q))) return rc;
        MDSX_CUDA(e, cudaMemcpyAsync(c.h_q(), c.red_q, (p * p + 1) * sizeof(double), cudaMemcpyDeviceToHost, c.s));
        MDSX_CUDA(e, cudaStreamSynchronize(c.s));
        s0.assign(c.h_q(), c.h_q() + p * p);
        logprior0 = c.log_prior(c.h_q()[p * p]);
        u0 = -(loglik0 + logprior0);
    }

    // dual averaging (Hoffman & Gelman 2014, Algorithm 5)
    const double mu = std::log(10.0 * cfg->step_size), gamma = 0.05, t0 = 10.0, kappa = 0.75;
    double hbar = cfg->resume ? resume_state.h.hbar : 0.0, log_eps_bar = cfg->resume ? resume_state.h.log_eps_bar : 0.0;
    std::uniform_real_distribution<double> unif(0.0, 1.0);
    long long accepted_after = 0, kept = 0;
    auto t_start = std::chrono::steady_clock::now();
    bool timing = it0 >= cfg->burn_in;
    // surrogate phase
    mdsx_surrogate* const sg = cfg->surrogate;
    bool surr_ready = false;
    int fallback_it = -1;
    long long surr_evals = 0;
    double train_seconds = 0.0, train_loss = NAN;
    std::vector<char> window;  // accept flags of recent surrogate iterations (ring)
    int window_pos = 0, window_sum = 0;
    auto start_surrogate = [&]() -> int {
        const auto t0 = std::chrono::steady_clock::now();
        std::vector<double> losses(std::max(1, cfg->train_steps));
        int r = MDSX_OK;
        if (cfg->train_steps > 0)
            r = mdsx_surrogate_train(sg, cfg->train_steps, cfg->train_batch, cfg->train_learning_rate, cfg->seed + 17,
                                     losses.data());
        if (!r) r = mdsx::surr::gradient(sg, c.x0, c.gs0, c.s);
        if (r) {
            e->last_error = sg->last_error;
            return r;
        }
        MDSX_CUDA(e, cudaStreamSynchronize(c.s));
        train_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (cfg->train_steps > 0) {
            const int tail = std::max(1, cfg->train_steps / 10);
            double acc = 0.0;
            for (int k = cfg->train_steps - tail; k < cfg->train_steps; ++k) acc += losses[k];
            train_loss = acc / tail;
        }
        surr_ready = true;
        return MDSX_OK;
    };
    if (sg && cfg->harvest_iterations == 0 && (rc = start_surrogate())) return rc;

    for (int k_it = 0; k_it < cfg->iterations; ++k_it) {
        const int it = (int)(it0 + k_it);  // the chain's iteration index (keys the momentum draws)
        if (!timing && it == cfg->burn_in) {
            timing = true;
            t_start = std::chrono::steady_clock::now();
        }
        // momentum ~ N(0, I) and its kinetic energy
        {
            const long long count = (long long)n * p;
            const int grid = (int)std::max(1LL, std::min(1024LL, (count / 2 + 255) / 256));
            mdsx::hmc::normal_kernel<<<grid, 256, 0, c.s>>>(c.mom, count, cfg->seed, (unsigned long long)it);
            MDSX_CUDA(e, cudaGetLastError());
            if ((rc = c.reduce(0, c.mom, c.red_k0))) return rc;
            MDSX_CUDA(e, cudaMemcpyAsync(c.h_k0(), c.red_k0, sizeof(double), cudaMemcpyDeviceToHost, c.s));
        }
        const bool use_surr = surr_ready && fallback_it < 0;
        if ((rc = c.run_trajectory(use_surr))) return rc;
        MDSX_CUDA(e, cudaStreamSynchronize(c.s));
        if ((rc = c.check_device_error())) return rc;
        if (use_surr) {
            c.sweeps += 1;
            surr_evals += cfg->leapfrog_steps;
        } else {
            c.sweeps += cfg->leapfrog_steps;
        }
        const double loglik_p = c.log_likelihood(c.h_sums()[2]);
        const double logprior_p = c.log_prior(c.h_q()[p * p]);
        const double u_p = -(loglik_p + logprior_p);
        const double dh = (u0 + c.h_k0()[0]) - (u_p + c.h_k()[0]);  // FP64 Hamiltonian difference
        const bool accept = std::isfinite(dh) && std::log(unif(c.rng)) < dh;
        const double alpha = std::isfinite(dh) ? std::min(1.0, std::exp(dh)) : 0.0;
        const double eps_used = c.eps;
        if (accept) {
            MDSX_CUDA(e, cudaMemcpyAsync(c.x0, c.xfinal, (size_t)n * p * sizeof(double), cudaMemcpyDeviceToDevice, c.s));
            MDSX_CUDA(e, cudaMemcpyAsync(c.gl0, e->d_grad[e->gcur], (size_t)n * p * sizeof(double),
                                         cudaMemcpyDeviceToDevice, c.s));
            if (use_surr)
                MDSX_CUDA(e, cudaMemcpyAsync(c.gs0, c.gsur, (size_t)n * p * sizeof(double), cudaMemcpyDeviceToDevice,
                                             c.s));
            loglik0 = loglik_p;
            logprior0 = logprior_p;
            u0 = u_p;
            s0.assign(c.h_q(), c.h_q() + p * p);
        }
        if (it >= cfg->burn_in) {
            ++kept;
            if (accept) ++accepted_after;
        }
        // harvest (chain state, its exact gradient)
        if (sg && it >= cfg->harvest_start && it < cfg->harvest_iterations && cfg->harvest_rows > 0) {
            rc = mdsx::surr::add_state(sg, c.x0, c.gl0, cfg->harvest_rows,
                                       cfg->seed * 0x9E3779B97F4A7C15ULL + (unsigned long long)it, c.s);
            if (rc) {
                e->last_error = sg->last_error;
                return rc;
            }
        }
        if (use_surr) {  // rolling acceptance and fallback to exact gradients
            if ((int)window.size() < cfg->fallback_window) {
                window.push_back(accept);
                window_sum += accept;
            } else {
                window_sum += (int)accept - window[window_pos];
                window[window_pos] = accept;
                window_pos = (window_pos + 1) % cfg->fallback_window;
            }
            if ((int)window.size() == cfg->fallback_window &&
                window_sum < cfg->fallback_accept * cfg->fallback_window)
                fallback_it = it;
        }

        if (cfg->adapt_step_size && it < cfg->burn_in) {
            const double m = it + 1;
            hbar = (1.0 - 1.0 / (m + t0)) * hbar + (cfg->target_accept - alpha) / (m + t0);
            const double log_eps = mu - std::sqrt(m) / gamma * hbar;
            const double w = std::pow(m, -kappa);
            log_eps_bar = w * log_eps + (1.0 - w) * log_eps_bar;
            c.eps = (it + 1 == cfg->burn_in) ? std::exp(log_eps_bar) : std::exp(log_eps);
            if ((rc = c.set_coef())) return rc;
        }

        // Metropolis step on the precision (R/Untitled.R:668-691)
        if (cfg->learn_precision) {
            const double tau_old = e->tau;
            const double tau_new = std::fabs(tau_old + tau_hw * (2.0 * unif(c.rng) - 1.0));
            MDSX_CUDA(e, mdsx::convert_locations(c.x0, n, p, e->d_x[e->xcur], e->x_ld, e->x_f32, c.s));
            e->tau = tau_new;
            double loglik_t = 0.0;
            if ((rc = c.sweep_loglik(&loglik_t))) {
                e->tau = tau_old;
                return rc;
            }
            const double u_t = -(loglik_t + logprior0);
            const bool tau_accept = std::isfinite(u_t) && std::log(unif(c.rng)) < u0 - u_t;
            if (cfg->adapt_precision_proposal && it < cfg->burn_in) {
                // Robbins-Monro on the log half-width toward 44 % acceptance (diminishing steps)
                tau_hw *= std::exp(((tau_accept ? 1.0 : 0.0) - 0.44) / std::sqrt((double)it + 1.0));
                tau_hw = std::min(std::max(tau_hw, 1e-12), 1e12);
            }
            if (tau_accept) {
                loglik0 = loglik_t;
                u0 = u_t;
                MDSX_CUDA(e, cudaMemcpyAsync(c.gl0, e->d_grad[e->gcur], (size_t)n * p * sizeof(double),
                                             cudaMemcpyDeviceToDevice, c.s));
                c.graph_dirty = true;  // the captured sweeps hold the old precision
                c.graph_s_dirty = true;
            } else {
                e->tau = tau_old;
            }
        }

        // Gibbs draw of the trait precision (R/Untitled.R:694-700; d0 = P, T0 = I)
        if (cfg->learn_trait_precision) {
            double a[kMaxP * kMaxP], scale[kMaxP * kMaxP], draw[kMaxP * kMaxP];
            for (int i = 0; i < p * p; ++i) a[i] = s0[i] + ((i % (p + 1)) == 0 ? 1.0 : 0.0);
            if (!spd_inverse(a, p, scale) || !wishart(c.rng, (double)(p + n), scale, p, draw))
                return fail(e, MDSX_ECUDA, "hmc: Wishart draw failed");
            if ((rc = c.set_lambda(draw))) return rc;
            double q = 0.0;
            for (int i = 0; i < p; ++i)
                for (int j = 0; j < p; ++j) q += draw[i * p + j] * s0[j * p + i];
            logprior0 = c.log_prior(q);
            u0 = -(loglik0 + logprior0);
        }

        // end of the harvest phase: train, then start from the surrogate gradient at x0
        if (sg && !surr_ready && it + 1 == cfg->harvest_iterations && (rc = start_surrogate())) return rc;

        // trace row
        double* row = trace + (size_t)k_it * cols;
        row[0] = loglik0;
        row[1] = logprior0;
        row[2] = u0;
        row[3] = e->tau;
        row[4] = accept ? 1.0 : 0.0;
        row[5] = eps_used;
        row[6] = dh;
        row[7] = use_surr ? 1.0 : 0.0;
        if (c.n_func) {
            MDSX_CUDA(e, with_p(p, FunctionalsF{c.x0, c.pairs, cfg->n_traced_pairs, c.locs, cfg->n_traced_locations,
                                                 c.func, c.s}));
            MDSX_CUDA(e, cudaMemcpyAsync(c.h_func(), c.func, c.n_func * sizeof(double), cudaMemcpyDeviceToHost, c.s));
            MDSX_CUDA(e, cudaStreamSynchronize(c.s));
            std::memcpy(row + kTraceBase, c.h_func(), c.n_func * sizeof(double));
        }
    }
    MDSX_CUDA(e, cudaStreamSynchronize(c.s));
    const double seconds =
        std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();

    // Leave the engine at the chain's final state.
    MDSX_CUDA(e, mdsx::convert_locations(c.x0, n, p, e->d_x[e->xcur], e->x_ld, e->x_f32, c.s));
    if (final_locations)
        MDSX_CUDA(e, cudaMemcpyAsync(final_locations, c.x0, (size_t)n * p * sizeof(double), cudaMemcpyDeviceToHost, c.s));
    MDSX_CUDA(e, cudaStreamSynchronize(c.s));
    e->sum_known = false;
    e->grad_known = false;
    long long ckpt_size = 0;
    if (cfg->checkpoint) {
        CkptState out;
        std::memcpy(out.h.magic, kCkptMagic, 8);
        out.h.n = n;
        out.h.p = p;
        out.h.seed = cfg->seed;
        out.h.next_iteration = it0 + cfg->iterations;
        out.h.tau = e->tau;
        out.h.eps = c.eps;
        out.h.hbar = hbar;
        out.h.log_eps_bar = log_eps_bar;
        out.h.loglik0 = loglik0;
        out.h.logprior0 = logprior0;
        out.h.u0 = u0;
        out.h.precision_half_width = tau_hw;
        out.s0 = s0;
        out.lambda.assign(c.lam.m, c.lam.m + p * p);
        out.x0.resize((size_t)n * p);
        out.gl0.resize((size_t)n * p);
        MDSX_CUDA(e, cudaMemcpyAsync(out.x0.data(), c.x0, (size_t)n * p * sizeof(double), cudaMemcpyDeviceToHost, c.s));
        MDSX_CUDA(e, cudaMemcpyAsync(out.gl0.data(), c.gl0, (size_t)n * p * sizeof(double), cudaMemcpyDeviceToHost,
                                     c.s));
        MDSX_CUDA(e, cudaStreamSynchronize(c.s));
        std::ostringstream os;
        os << c.rng;
        out.rng = os.str();
        out.h.rng_len = (int32_t)out.rng.size();
        if (out.rng.size() > 8192 || ckpt_bytes(out) > cfg->checkpoint_capacity)
            return fail(e, MDSX_EINVAL, "hmc: checkpoint larger than its buffer");
        ckpt_write(out, cfg->checkpoint);
        ckpt_size = (long long)ckpt_bytes(out);
    }
    if (stats) {
        stats->checkpoint_bytes = ckpt_size;
        stats->accept_rate = kept > 0 ? (double)accepted_after / kept : 0.0;
        stats->step_size = c.eps;
        stats->seconds = seconds;
        stats->gradient_evaluations = c.sweeps;
        stats->precision = e->tau;
        stats->surrogate_evaluations = surr_evals;
        stats->fallback_iteration = fallback_it;
        stats->train_seconds = train_seconds;
        stats->train_loss = train_loss;
    }
    return MDSX_OK;
}
