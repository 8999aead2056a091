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
/* FP64-accurate sweep in double-float arithmetic on the FP32 pipes (not with
 * MDSX_FLAG_FLOAT; with MDSX_FLAG_DELTA_F32 over FP32-stored delta). P <= 6,
 * whole-matrix engines, unordered-pair schedule; not for the HMC driver. */
#define MDSX_FLAG_DOUBLE_FLOAT (1L << 12)

/* Largest embedding dimension the CUDA kernels are built for. */
#define MDSX_MAX_DIMENSION 10

typedef struct mdsx_engine mdsx_engine;

/* Replaces mds::factory(dim, N, flags, device, threads) (src/factory.cpp:32) for
 * the GPU branch and the engine constructor
 * NewMultiDimensionalScaling(embeddingDimension, locationCount, flags, threads)
 * (src/NewMultiDimensionalScaling.hpp:79). device < 0 selects the current device. */
int mdsx_create(int embedding_dimension, int location_count, long flags, int device,
                mdsx_engine** out);

/* A row range of one problem, for splitting a sweep across GPUs: the engine
 * holds and sweeps rows [row_begin, row_end) of the N x N delta only. This is
 * the reference's own parallel split -- its TBB engine partitions the rows i
 * of both passes (parallel_reduce / parallel_for over i,
 * src/NewMultiDimensionalScaling.hpp:708-744) -- across devices instead of
 * threads. Differences from mdsx_create: setPairwiseData takes the range's
 * rows, (row_end - row_begin) * N values; updateLocations still takes all N
 * locations; getSumOfIncrements returns the range's share (the sum over
 * ranges is the whole matrix's value); getLogLikelihood the range's share of
 * R/mds.R:24-28 (observation count (row_end - row_begin)(N - 1)/2);
 * getLogLikelihoodGradient the range's rows, (row_end - row_begin) * P values
 * (row i of the gradient reads only row i of delta, :421-461). Row ranges use
 * the row-block schedule; the HMC driver and the surrogate need a whole-matrix
 * engine. */
int mdsx_create_rows(int embedding_dimension, int location_count, long flags, int device, int row_begin,
                     int row_end, mdsx_engine** out);
/* [row_begin, row_end) of an engine: [0, N) unless made by mdsx_create_rows. */
int mdsx_get_row_range(const mdsx_engine* engine, int* row_begin, int* row_end);

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

/* Sweep schedule (no counterpart in the reference; results agree within the
 * FP32 tolerance, the summation order differs):
 *   MDSX_SWEEP_ROWS  - one pass per ordered pair, row blocks x 128-column stages;
 *   MDSX_SWEEP_PAIRS - each unordered pair {i, j} once: distance and Phi shared
 *                      by (i, j) and (j, i), each direction with its own delta;
 *                      a sweep kernel plus a finish kernel, for P <= 6 in
 *                      every precision mode (FP64 results within 1e-10 of
 *                      the row-block schedule's).
 * New engines use MDSX_SWEEP_PAIRS where it is built, in the FP64 modes and in
 * FP32 with truncation (the pair math dominates there), else MDSX_SWEEP_ROWS
 * (untruncated FP32, at the memory bound with one kernel).
 * Setting MDSX_SWEEP_PAIRS where it is not built returns MDSX_EUNSUPPORTED. */
#define MDSX_SWEEP_ROWS 0
#define MDSX_SWEEP_PAIRS 1
int mdsx_set_sweep_schedule(mdsx_engine* engine, int schedule);
int mdsx_get_sweep_schedule(mdsx_engine* engine, int* out);

/* Self-test of the bounded device waits (no counterpart in the reference): a
 * one-thread kernel on `device` (< 0: current) waits on a barrier that never
 * completes, gives up after limit_seconds (0 < limit <= 10) and records the
 * timeout. Returns MDSX_ETIMEOUT with *device_code = 1 when the wait gave up as
 * designed (the context stays usable), MDSX_ECUDA otherwise. */
int mdsx_selftest_bounded_wait(double limit_seconds, int device, int* device_code);

/* Self-test of the FP64 pair-math helpers (no counterpart in the reference):
 * for each of the n host values x[i] writes out[4i .. 4i+3] = the sweep's
 * Newton-refined 1/x and 1/sqrt(x), and its normal CDF and density at z = x
 * (the FP64 sweeps' Phi and phi), computed on `device` (< 0: current).
 * Returns MDSX_OK, MDSX_EINVAL (n = 0 or > 2^24), MDSX_ENOMEM or MDSX_ECUDA. */
int mdsx_selftest_math_f64(const double* x, size_t n, double* out, int device);

/* ---- Learned gradient surrogate (no counterpart in the reference) ----
 * g_i ~= s * sum_k alpha_ik (x_i - x_{l_k}) over K landmark locations (a
 * seeded random subset), alpha_i = MLP(features_i) with rotation-invariant
 * features [d(x_i, x_{l_k}) - delta_{i, l_k} (scaled), delta_{i, l_k}
 * (standardised)]. The MLP
 * (2K -> width x layers, SiLU -> K) runs forward and backward on BF16 tensor
 * cores with FP32 accumulation and is trained with Adam on rows (features,
 * landmark directions, exact log-likelihood gradient) harvested from exact
 * states. Used by mdsx_hmc_run inside trajectories only; every accept is
 * judged with the exact potential. Requires landmarks and width multiples of
 * 64; the surrogate reads the engine's delta and lives on its GPU and stream,
 * and must be destroyed before the engine. */
typedef struct mdsx_surrogate mdsx_surrogate;

int mdsx_surrogate_create(mdsx_engine* engine, int landmarks, int hidden_width, int hidden_layers,
                          int max_training_rows, unsigned long long seed, mdsx_surrogate** out);
void mdsx_surrogate_destroy(mdsx_surrogate* surrogate);
const char* mdsx_surrogate_last_error(const mdsx_surrogate* surrogate);
/* ints[8]: N, P, landmarks, width, layers, harvested rows, max rows, Adam steps;
 * reals[5]: delta-feature mean and 1/sd, contraction scale, target scale,
 * 1/scale of the residual features. */
int mdsx_surrogate_info(const mdsx_surrogate* surrogate, int* ints, double* reals);
int mdsx_surrogate_landmarks(const mdsx_surrogate* surrogate, int* out);
/* which: 0 read, 1 write the FP32 weight [out][in] and bias of `layer`
 * (0 .. layers; `layers` is the output layer), 2 read their gradients. */
int mdsx_surrogate_parameters(mdsx_surrogate* surrogate, int layer, int which, float* weight, float* bias);
/* Harvest `rows` rows at random locations of one exact state (host N*P doubles). */
int mdsx_surrogate_add_state(mdsx_surrogate* surrogate, const double* locations, const double* gradient, int rows,
                             unsigned long long seed);
int mdsx_surrogate_training_rows(mdsx_surrogate* surrogate, int first, int count, float* features,
                                 float* directions, float* targets);
/* Adam steps on seeded uniform batches (batch a multiple of 64); loss_trace
 * (steps doubles, may be NULL) gets each step's mean squared error in units
 * of the target scale. */
int mdsx_surrogate_train(mdsx_surrogate* surrogate, int steps, int batch, double learning_rate,
                         unsigned long long seed, double* loss_trace);
/* Loss and parameter gradients of the given training rows, without update. */
int mdsx_surrogate_batch_gradient(mdsx_surrogate* surrogate, const int* rows, int count, double* loss);
/* Surrogate log-likelihood gradient at host locations (N*P) into host gradient. */
int mdsx_surrogate_gradient(mdsx_surrogate* surrogate, const double* locations, double* gradient);
/* Test hook: C[m x n] = op(A) op(B) with the MLP's tensor-core GEMM (BF16 bit
 * patterns in, FP32 out, host buffers). a_t: A stored [k][m]; b_t: B stored
 * [k][n] (else [n][k]); m, n multiples of 64, k of 32. */
int mdsx_test_gemm_bf16(int a_t, int b_t, int m, int n, int k, const unsigned short* a, const unsigned short* b,
                        float* c);

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
 * difference, 1 if the trajectory used the surrogate) followed by the traced pair distances and location norms. */
#define MDSX_HMC_TRACE_BASE 8
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
    /* Surrogate phase (surrogate == NULL: exact gradients throughout). The
     * first harvest_iterations iterations use exact gradients; iterations
     * harvest_start .. harvest_iterations - 1 harvest harvest_rows rows from
     * the chain's state after the accept step (finite by construction); the
     * surrogate is then trained (train_steps Adam steps, train_batch rows,
     * train_learning_rate) and drives the leapfrog steps. When the acceptance
     * rate over the last fallback_window surrogate iterations drops below
     * fallback_accept the chain returns to exact gradients for good. */
    mdsx_surrogate* surrogate;
    int harvest_iterations;
    int harvest_start;
    int harvest_rows;
    int train_steps;
    int train_batch;
    double train_learning_rate;
    double fallback_accept;      /* 0.6 */
    int fallback_window;         /* e.g. 50 */
    /* Checkpoint and resume of exact-gradient chains (no surrogate), so a long
     * run can stop and continue: `checkpoint` (capacity checkpoint_capacity
     * >= MDSX_HMC_CHECKPOINT_BYTES(N, P); NULL for none) receives the chain's
     * state after its last iteration -- next iteration index, locations and
     * their exact gradient, log-likelihood, log prior, potential, X'X, tau,
     * trait precision, step size and step-size adaptation state, and the host
     * random generator; stats->checkpoint_bytes gives its size. `resume`
     * (NULL for a fresh chain) continues the chain such a checkpoint holds,
     * with the same seed, engine dimensions and delta: initial_locations is
     * ignored, `iterations` counts further iterations, burn_in stays counted
     * from the chain's first iteration. A chain run in pieces this way gives
     * the same trace, bit for bit, as the chain run in one call. */
    const void* resume;
    size_t resume_bytes;
    void* checkpoint;
    size_t checkpoint_capacity;
    /* Nonzero: during burn-in the half-width of the precision proposal adapts
     * toward 44 % acceptance (log half-width += (accepted - 0.44) / sqrt(t)),
     * then stays fixed. The reference keeps it at 0.01, which at N = 50 000
     * moves tau far too slowly; off by default. */
    int adapt_precision_proposal;
} mdsx_hmc_config;

#define MDSX_HMC_CHECKPOINT_BYTES(n, p) \
    (112 + 16 * (size_t)(p) * (size_t)(p) + 16 * (size_t)(n) * (size_t)(p) + 8192)

typedef struct {
    double accept_rate;              /* after burn-in */
    double step_size;                /* final */
    double seconds;                  /* wall time of the iterations after burn-in */
    long long gradient_evaluations;  /* fused sweeps run */
    double precision;                /* final tau */
    long long surrogate_evaluations; /* surrogate gradients evaluated */
    int fallback_iteration;          /* iteration of the fallback to exact gradients, -1 if none */
    double train_seconds;            /* wall time of surrogate training */
    double train_loss;               /* mean loss over the last 10% of training steps */
    long long checkpoint_bytes;      /* bytes written to config->checkpoint, 0 if none */
} mdsx_hmc_stats;

/* initial_locations: N*P host doubles; trace: iterations * (MDSX_HMC_TRACE_BASE +
 * n_traced_pairs + n_traced_locations) host doubles; final_locations (N*P) and
 * stats may be NULL. The engine is left at the final locations and precision. */
int mdsx_hmc_run(mdsx_engine* engine, const mdsx_hmc_config* config, const double* initial_locations,
                 double* trace, double* final_locations, mdsx_hmc_stats* stats);

/* ---- Batched multi-instance engine (replaces the reference's many-engines
 * pattern: the JNI singleton's vector of engines addressed by index,
 * src/jni/dr_inference_multidimensionalscaling_NativeMDSSingleton.cpp:10-100) ----
 * Many independent MDS problems (any mix of N and P) on one GPU, evaluated by
 * one persistent stream-K launch per embedding dimension, captured as a CUDA
 * graph. FP32 pair arithmetic with FP64 reductions (flags must include
 * MDSX_FLAG_FLOAT; MDSX_FLAG_LEFT_TRUNCATION applies to every instance).
 * Instance calls keep the reference's names and lazy semantics: a getter
 * evaluates the whole batch when any instance changed since the last
 * evaluation. Adding an instance, setting its data or forcing a shape
 * re-plans the batch at the next evaluation. */
typedef struct mdsx_batch mdsx_batch;

int mdsx_batch_create(long flags, int device, mdsx_batch** out);
void mdsx_batch_destroy(mdsx_batch* batch);
const char* mdsx_batch_last_error(const mdsx_batch* batch);
int mdsx_batch_instance_count(const mdsx_batch* batch);
/* JNI initialize(embeddingDimension, locationCount): *instance = new index. */
int mdsx_batch_add_instance(mdsx_batch* batch, int embedding_dimension, int location_count, int* instance);
int mdsx_batch_set_pairwise_data(mdsx_batch* batch, int instance, const double* data, size_t length);
int mdsx_batch_set_pairwise_data_f32(mdsx_batch* batch, int instance, const float* data, size_t length);
int mdsx_batch_set_parameters(mdsx_batch* batch, int instance, const double* parameters, size_t length);
int mdsx_batch_update_locations(mdsx_batch* batch, int instance, int location_index, const double* locations,
                                size_t length);
int mdsx_batch_make_dirty(mdsx_batch* batch);
int mdsx_batch_get_sum_of_increments(mdsx_batch* batch, int instance, double* out);
int mdsx_batch_get_log_likelihood(mdsx_batch* batch, int instance, double* out);
int mdsx_batch_get_log_likelihood_gradient(mdsx_batch* batch, int instance, double* out, size_t length);
/* One evaluation of every instance, results read back to the host. */
int mdsx_batch_evaluate(mdsx_batch* batch);
/* One evaluation left on the device, enqueued without synchronising: d_sums
 * gets [count][4] doubles (sum r^2, sum log Phi, getSumOfIncrements(),
 * unused), d_gradients the instances' N*P gradients concatenated in instance
 * order; either may be NULL. */
int mdsx_batch_evaluate_device(mdsx_batch* batch, double* d_sums, double* d_gradients);
/* Shapes: schedule 0 = stream-K over (row block x 128 columns) units of all
 * instances, 1 = queue of whole row blocks (largest instance first, each CTA
 * owning the row blocks it takes); rows per warp (1, 2, 4 as built for P);
 * CTAs per SM. Autotuner: times every built shape of each dimension group on
 * this batch and caches the fastest per (P, N-bucket = floor(log2 mean N),
 * truncation), in process and in the file named by the environment variable
 * MDSX_TUNE_CACHE. *candidates (may be NULL) = shapes timed. */
int mdsx_batch_tune(mdsx_batch* batch, int repetitions, int* candidates);
/* Shape in use for dimension p (plans the batch if needed). */
int mdsx_batch_group_shape(mdsx_batch* batch, int p, int* schedule, int* rows_per_warp, int* ctas_per_sm,
                           int* grid);
/* Fixes the shape of dimension p's group (rows_per_warp 0 removes it). */
int mdsx_batch_force_shape(mdsx_batch* batch, int p, int schedule, int rows_per_warp, int ctas_per_sm);

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
 * held until the process exits on each device where the entry point has been
 * called (on every device the process uses under CUDA_MODULE_LOADING=EAGER).
 * Each call resolves that array's address in the current context
 * (cudaGetSymbolAddress) and returns after the results are in the caller's
 * buffers. Delta is read once when it holds no NaN; with NaN pairs the call
 * scans delta for them and sweeps a second time. Calls share the array: calls
 * that overlap on the GPU race and must be serialised. Problems whose scratch does not fit
 * (N above MDSX_NOALLOC_MAX_LOCATIONS, or a plan too large) return MDSX_EINVAL;
 * mdsx_last_error(NULL) then gives the message. No cudaMalloc, cudaFree or
 * allocating library routine is called. */
#define MDSX_NOALLOC_SCRATCH_BYTES (8u << 20)
#define MDSX_NOALLOC_MAX_LOCATIONS 32768
int mdsx_sweep_f32_noalloc(const float* d_delta, long long delta_ld, const double* d_locations,
                           int location_count, int embedding_dimension, double precision, int truncation,
                           double* d_sum_of_increments, double* d_gradient, void* stream);

/* ---- Host-side fault injection (no counterpart in the reference, which
 * asserts or exits on errors) ----
 * For tests of the failure paths: arms one host-side call of `site` to fail
 * after `after` further calls at that site succeed; the failing call is not
 * made and the hook returns what the CUDA runtime would (out of memory, or a
 * non-sticky launch failure), so no GPU fault occurs and the context stays
 * usable. The engine and batch calls then return MDSX_ENOMEM or MDSX_ECUDA.
 * One-shot: the hook disarms itself when it fires; MDSX_FAULT_NONE disarms.
 * *fired (may be NULL) = faults fired so far in this process. */
#define MDSX_FAULT_NONE 0
#define MDSX_FAULT_DEVICE_ALLOC 1 /* cudaMalloc in engine and batch set-up */
#define MDSX_FAULT_HOST_ALLOC 2   /* cudaMallocHost (pinned result mirrors) */
#define MDSX_FAULT_LAUNCH 3       /* the enqueue of a sweep (engine) or of the batch graph */
int mdsx_inject_fault(int site, long long after, long long* fired);

/* Library version string. */
const char* mdsx_version(void);

#ifdef __cplusplus
}  /* extern "C" */
#endif

#endif /* MDSX_H */
