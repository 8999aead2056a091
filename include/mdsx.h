/*
 * mdsx: GB300-native engine for the MassiveMDS likelihood/gradient sweep.
 *
 * C ABI of libmdsx.so. Plain pointers and sizes only. Every call returns an
 * int status (MDSX_OK == 0); on error, mdsx_last_error() gives a message.
 *
 * Each entry point replaces one method of the reference engine interface
 * mds::AbstractMultiDimensionalScaling (src/AbstractMultiDimensionalScaling.hpp:38-73)
 * or the engine factory mds::factory (src/AbstractMultiDimensionalScaling.hpp:77,
 * src/factory.cpp:32-118). The header-only C++ class in
 * include/mdsx/CudaMultiDimensionalScaling.hpp wraps this ABI behind that
 * interface.
 *
 * Semantics (same as the reference CPU engine, src/NewMultiDimensionalScaling.hpp):
 *   - delta is a full N x N row-major matrix; (i,j) is missing when i == j or
 *     delta_ij is NaN, and missing pairs add nothing.
 *   - getSumOfIncrements sums the increments of all ordered pairs and halves;
 *     with LEFT_TRUNCATION it returns that total, without it 0.5*tau*total.
 *   - the gradient is d loglik / d x_i, row i of delta only.
 * Calls are synchronous: results are on the host when a call returns. One
 * engine is used by one host thread at a time; engines are independent.
 */
#ifndef MDSX_H
#define MDSX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define MDSX_OK 0
#define MDSX_EINVAL 1   /* bad argument: null handle/pointer, wrong length, bad tau */
#define MDSX_ENOMEM 2   /* device or pinned host allocation failed */
#define MDSX_ECUDA 3    /* a CUDA runtime/driver call failed */
#define MDSX_ETIMEOUT 4 /* a device-side bounded wait gave up; engine reset its scratch */
#define MDSX_ESTATE 5   /* call out of order, e.g. a sweep before setPairwiseData */
#define MDSX_EUNSUPPORTED 6 /* configuration this build does not provide (e.g. P > 10) */

/* Flag bits. Bits 2..9 are the reference's (src/flags.h:6-14); 10.. are ours. */
#define MDSX_FLAG_FLOAT (1L << 2)           /* FP32 sweep, FP32-stored delta, FP64 reductions */
#define MDSX_FLAG_TBB (1L << 3)             /* accepted and ignored (CPU threading) */
#define MDSX_FLAG_OPENCL (1L << 4)          /* routed to this CUDA engine */
#define MDSX_FLAG_LEFT_TRUNCATION (1L << 5) /* truncated likelihood, logPhi(d*sqrt(tau)) term */
#define MDSX_FLAG_SSE (1L << 7)             /* accepted and ignored */
#define MDSX_FLAG_AVX (1L << 8)             /* accepted and ignored */
#define MDSX_FLAG_AVX512 (1L << 9)          /* accepted and ignored */
#define MDSX_FLAG_CUDA (1L << 10)           /* select this engine explicitly */
#define MDSX_FLAG_DELTA_F32 (1L << 11)      /* FP64 sweep over FP32-stored delta */

/* Largest embedding dimension the CUDA kernels are built for. */
#define MDSX_MAX_DIMENSION 10

typedef struct mdsx_engine mdsx_engine;

/* Replaces mds::factory(dim, N, flags, device, threads) (src/factory.cpp:32) for
 * the GPU branch and the engine constructor
 * NewMultiDimensionalScaling(embeddingDimension, locationCount, flags, threads)
 * (src/NewMultiDimensionalScaling.hpp:79). device < 0 selects the current device. */
int mdsx_create(int embedding_dimension, int location_count, long flags, int device,
                mdsx_engine** out);

/* Replaces the engine destructor (src/NewMultiDimensionalScaling.hpp:130). */
int mdsx_destroy(mdsx_engine* engine);

/* Replaces updateLocations(int, double*, size_t) (src/AbstractMultiDimensionalScaling.hpp:48,
 * src/NewMultiDimensionalScaling.hpp:134-166). index == -1: all N locations,
 * length == N*P row-major; index >= 0: one location, length == P. */
int mdsx_update_locations(mdsx_engine* engine, int index, const double* locations, size_t length);

/* Replaces getSumOfIncrements() (src/AbstractMultiDimensionalScaling.hpp:51,
 * src/NewMultiDimensionalScaling.hpp:193-203). */
int mdsx_get_sum_of_increments(mdsx_engine* engine, double* out);

/* Replaces getLogLikelihoodGradient(double*, size_t)
 * (src/AbstractMultiDimensionalScaling.hpp:52, src/NewMultiDimensionalScaling.hpp:281-302).
 * length == N*P (== N*getInternalDimension()). */
int mdsx_get_log_likelihood_gradient(mdsx_engine* engine, double* out, size_t length);

/* Replace storeState/restoreState/acceptState (src/AbstractMultiDimensionalScaling.hpp:53-55,
 * src/NewMultiDimensionalScaling.hpp:205-255). */
int mdsx_store_state(mdsx_engine* engine);
int mdsx_restore_state(mdsx_engine* engine);
int mdsx_accept_state(mdsx_engine* engine);

/* Replaces setPairwiseData(double*, size_t) (src/AbstractMultiDimensionalScaling.hpp:56,
 * src/NewMultiDimensionalScaling.hpp:257-260 with the NaN-preserving conversion of
 * src/MemoryManagement.hpp:45-56). length == N*N. */
int mdsx_set_pairwise_data(mdsx_engine* engine, const double* data, size_t length);

/* FP32 ingest of the same matrix (no counterpart in the reference interface; the
 * reference's FLOAT engine rounds its double input to float the same way). */
int mdsx_set_pairwise_data_f32(mdsx_engine* engine, const float* data, size_t length);

/* Replaces setParameters(double*, size_t) (src/AbstractMultiDimensionalScaling.hpp:57,
 * src/NewMultiDimensionalScaling.hpp:262-274): data[0] = precision tau > 0, length == 1. */
int mdsx_set_parameters(mdsx_engine* engine, const double* data, size_t length);

/* Replaces makeDirty() (src/AbstractMultiDimensionalScaling.hpp:58,
 * src/NewMultiDimensionalScaling.hpp:276-279). */
int mdsx_make_dirty(mdsx_engine* engine);

/* Replaces getInternalDimension() (src/AbstractMultiDimensionalScaling.hpp:59,
 * src/NewMultiDimensionalScaling.hpp:132): P (no padding in this engine's layout). */
int mdsx_get_internal_dimension(mdsx_engine* engine, int* out);

/* Log-likelihood as the R layer assembles it (R/mds.R:24-28):
 * 0.5*(log tau - log 2pi)*N(N-1)/2 - sumOfIncrements. */
int mdsx_get_log_likelihood(mdsx_engine* engine, double* out);

/* Message for the last failed call on this engine (or of mdsx_create when
 * engine is NULL). Valid until the next call on the same engine. */
const char* mdsx_last_error(const mdsx_engine* engine);

/* ---- Device-resident variants (no counterpart in the reference interface) ----
 * For callers that keep locations and results in device memory (an on-GPU
 * sampler, or throughput measurement with inputs already in HBM). Pointers are
 * device pointers; work is ordered on the engine's stream and these calls do
 * not synchronise. */

/* Use `stream` (a cudaStream_t) for all work of this engine; NULL = the
 * engine's own stream. The caller keeps ownership. */
int mdsx_set_stream(mdsx_engine* engine, void* stream);

/* Like mdsx_update_locations(engine, -1, ...) from N*P row-major device doubles. */
int mdsx_update_locations_device(mdsx_engine* engine, const double* d_locations, size_t length);

/* One fused sweep at the current state. Writes the sum of increments to
 * *d_sum (device double) and, when d_gradient != NULL, the gradient (N*P
 * row-major device doubles). Marks both results known. */
int mdsx_evaluate_device(mdsx_engine* engine, double* d_sum, double* d_gradient);

/* Number of kernel launches the last sweep issued (for launch accounting). */
int mdsx_last_launch_count(mdsx_engine* engine, int* out);

/* ---- Hamiltonian Monte Carlo (no counterpart in the reference's C++ engine;
 * restates the R sampler hmcsampler, R/Untitled.R:477-729) ----
 * Runs a whole chain on the engine's GPU: momentum N(0, I), leapfrog with one
 * fused sweep per step, Metropolis accept on the FP64 Hamiltonian difference,
 * optional Metropolis step on the precision tau (|U(tau - h, tau + h)|
 * proposal) and Gibbs draw of the P x P trait precision
 * (Wishart(P + N, (I + X'X)^-1)); prior on locations: matrix normal with row
 * covariance I_N and column precision Lambda (initially I_P). The engine must
 * hold delta and tau. Trace: `iterations` rows of MDSX_HMC_TRACE_BASE columns
 * (log-likelihood, log prior, potential, tau, accepted, step size, Hamiltonian
 * difference) followed by the traced pair distances and location norms. */
#define MDSX_HMC_TRACE_BASE 7
typedef struct {
    int iterations;
    int burn_in;              /* step size adapts over these if adapt_step_size */
    int leapfrog_steps;       /* the reference uses 20 */
    double step_size;         /* initial; the reference uses trajectory / 20 = 0.01 */
    int adapt_step_size;      /* dual averaging during burn-in */
    double target_accept;     /* e.g. 0.8 */
    int learn_precision;      /* Metropolis step on tau each iteration */
    double precision_half_width; /* the reference uses 0.01 */
    int learn_trait_precision;   /* Gibbs draw of the trait precision each iteration */
    unsigned long long seed;
    int n_traced_pairs;          /* distances |x_i - x_j| traced per iteration */
    const int* traced_pairs;     /* 2 * n_traced_pairs location indices */
    int n_traced_locations;      /* norms |x_i| traced per iteration */
    const int* traced_locations;
    int use_graph;               /* capture each trajectory as a CUDA graph */
} mdsx_hmc_config;

typedef struct {
    double accept_rate;              /* after burn-in */
    double step_size;                /* final */
    double seconds;                  /* wall time of the iterations after burn-in */
    long long gradient_evaluations;  /* fused sweeps run */
    double precision;                /* final tau */
} mdsx_hmc_stats;

/* initial_locations: N*P host doubles; trace: iterations * (MDSX_HMC_TRACE_BASE +
 * n_traced_pairs + n_traced_locations) host doubles; final_locations (N*P) and
 * stats may be NULL. The engine is left at the final locations and precision. */
int mdsx_hmc_run(mdsx_engine* engine, const mdsx_hmc_config* config, const double* initial_locations,
                 double* trace, double* final_locations, mdsx_hmc_stats* stats);

/* ---- Allocation-free variant (no counterpart in the reference) ----
 * For callers that cannot allocate device memory: hosts whose GPU memory is
 * owned by another allocator (a JVM or R process sharing the device with a
 * framework that has reserved it) and sampler loops that must not call
 * cudaMalloc/cudaFree, which can fail at run time and synchronise the device.
 *
 * One fused FP32 sweep (the MDSX_FLAG_FLOAT arithmetic) over caller-owned
 * device buffers: d_delta is N x N float, row stride delta_ld floats (a
 * multiple of 4, >= N, 16-byte aligned base; NaN = missing); d_locations is
 * N*P row-major doubles; writes getSumOfIncrements() to *d_sum_of_increments
 * and the N*P gradient to d_gradient (device doubles). Synchronous on `stream`
 * (a cudaStream_t; NULL = the legacy default stream).
 *
 * All scratch lives in one static device array of MDSX_NOALLOC_SCRATCH_BYTES,
 * held on every GPU that loads the library until the process exits. The first
 * call on a device resolves that array's address (cudaGetSymbolAddress), so
 * make it before any stream capture. Calls share the array: calls that overlap
 * on the GPU race and must be serialised. Problems whose scratch does not fit
 * (N above MDSX_NOALLOC_MAX_LOCATIONS, or a plan too large) return MDSX_EINVAL;
 * mdsx_last_error(NULL) then gives the message. No cudaMalloc, cudaFree or
 * allocating library routine is called. */
#define MDSX_NOALLOC_SCRATCH_BYTES (8u << 20)
#define MDSX_NOALLOC_MAX_LOCATIONS 32768
int mdsx_sweep_f32_noalloc(const float* d_delta, long long delta_ld, const double* d_locations,
                           int location_count, int embedding_dimension, double precision, int truncation,
                           double* d_sum_of_increments, double* d_gradient, void* stream);

/* Library version string. */
const char* mdsx_version(void);

#ifdef __cplusplus
}  /* extern "C" */
#endif

#endif /* MDSX_H */
