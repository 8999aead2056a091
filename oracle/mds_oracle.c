/*
 * Test infrastructure: the oracle. Not product code.
 *
 * An independent FP64 restatement of the MassiveMDS likelihood and gradient
 * sweep (suchard-group/MassiveMDS), used only by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg as the checker.
 * The CUDA engine never calls it.
 *
 * Semantics followed, by reference file:line:
 *   - A pair (i,j) is missing when i == j or delta_ij is NaN; missing pairs
 *     add nothing (src/NewMultiDimensionalScaling.hpp:402-410, :431-433, :504-506).
 *   - d_ij = ||x_i - x_j||_2 summed over dimensions in order
 *     (src/Distance.hpp:78-88, :142-151).
 *   - With truncation the increment of an ordered pair is
 *       0.5*tau*(delta - d)^2 + log(0.5*erfc(-d*sqrt(tau)/sqrt(2)))
 *     (src/NewMultiDimensionalScaling.hpp:508-514 with scale = 0.5*precision
 *     at :527 and oneOverSd = sqrt(precision) at :265; logPhi is
 *     src/CDF.h:583-592). Without truncation it is (delta - d)^2.
 *   - The sum runs over all ordered pairs of the full N x N matrix and is then
 *     halved (:529-557). getSumOfIncrements returns that total with
 *     truncation, and 0.5*tau*total without (:193-203).
 *   - The gradient row i reads only row i of delta (:421-461):
 *       g_i = sum_j tau * r_ij / d_ij * (x_i - x_j),
 *       r_ij = (delta_ij - d_ij) - [trunc] phi(z)/(Phi(z)*sqrt(tau)), z = d_ij*sqrt(tau)
 *     with phi(z) = exp(-z^2/2)/sqrt(2*pi) (src/CDF.h:608-616). The reference
 *     writes Phi(z) as exp(logPhi(z)); here it is 0.5*erfc(-z/sqrt(2))
 *     directly, which differs by at most a rounding.
 *   - The R log-likelihood is 0.5*(log tau - log 2pi)*N(N-1)/2 - sumOfIncrements
 *     (R/mds.R:24-28).
 *
 * Unlike the reference (which accumulates naively in RealType and stores an
 * N x N increments array), every sum here is Neumaier-compensated in FP64,
 * row results are combined in row order (so the answer does not depend on the
 * thread count), indices are 64-bit, and no N x N scratch is kept, so the
 * oracle also runs at N = 50 000.
 *
 * delta may be given as double or as float (FP32-rounded and promoted, the
 * form the FP32-stored configurations use).
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define MDSO_SQRT1_2 0.70710678118654752440
#define MDSO_1_SQRT_2PI 0.39894228040143267794

typedef struct {
    double s, c; /* Neumaier sum and compensation */
} nsum;

static inline void nsum_add(nsum* a, double v) {
    double t = a->s + v;
    if (fabs(a->s) >= fabs(v))
        a->c += (a->s - t) + v;
    else
        a->c += (v - t) + a->s;
    a->s = t;
}
static inline double nsum_get(const nsum* a) { return a->s + a->c; }

typedef struct {
    const void* delta;
    int delta_is_f32;
    const double* x;
    int64_t n;
    int p;
    double tau;
    int truncation;
    int want_sum, want_grad;
    int64_t row_begin, row_end; /* rows this call covers */
    double* row_sum;            /* [row_end-row_begin] per-row increment sums */
    double* grad;               /* [(row_end-row_begin)*p] */
    int64_t t_begin, t_end;     /* rows of one worker */
} job;

static inline double delta_at(const job* jb, int64_t i, int64_t j) {
    if (jb->delta_is_f32) return (double)((const float*)jb->delta)[i * jb->n + j];
    return ((const double*)jb->delta)[i * jb->n + j];
}

static inline double distance(const double* xi, const double* xj, int p) {
    double s = 0.0;
    for (int k = 0; k < p; ++k) {
        double df = xi[k] - xj[k];
        s += df * df;
    }
    return sqrt(s);
}

static void sweep_row(const job* jb, int64_t i) {
    const int p = jb->p;
    const double* xi = jb->x + i * p;
    const double sqrt_tau = sqrt(jb->tau);
    nsum rs = {0.0, 0.0};
    nsum g[64];
    int pp = p < 64 ? p : 64;
    for (int k = 0; k < pp; ++k) g[k].s = g[k].c = 0.0;

    for (int64_t j = 0; j < jb->n; ++j) {
        const double obs = delta_at(jb, i, j);
        if (i == j || isnan(obs)) continue;
        const double* xj = jb->x + j * p;
        const double d = distance(xi, xj, p);
        const double resid = obs - d;
        if (jb->want_sum) {
            double inc;
            if (jb->truncation) {
                const double z = d * sqrt_tau;
                inc = 0.5 * jb->tau * resid * resid + log(0.5 * erfc(-z * MDSO_SQRT1_2));
            } else {
                inc = resid * resid;
            }
            nsum_add(&rs, inc);
        }
        if (jb->want_grad) {
            double r = resid;
            if (jb->truncation) {
                const double z = d * sqrt_tau;
                const double pdf = MDSO_1_SQRT_2PI * exp(-0.5 * z * z);
                const double cdf = 0.5 * erfc(-z * MDSO_SQRT1_2);
                r -= pdf / (cdf * sqrt_tau);
            }
            const double c = r * jb->tau / d;
            for (int k = 0; k < pp; ++k) nsum_add(&g[k], c * (xi[k] - xj[k]));
        }
    }
    const int64_t local = i - jb->row_begin;
    if (jb->want_sum) jb->row_sum[local] = nsum_get(&rs);
    if (jb->want_grad)
        for (int k = 0; k < pp; ++k) jb->grad[local * p + k] = nsum_get(&g[k]);
}

static void* worker(void* arg) {
    job* jb = (job*)arg;
    for (int64_t i = jb->t_begin; i < jb->t_end; ++i) sweep_row(jb, i);
    return NULL;
}

/* Runs the sweep over rows [row_begin, row_end) on `threads` threads. */
static int run(job* base, int threads) {
    int64_t rows = base->row_end - base->row_begin;
    if (rows <= 0) return 0;
    if (threads < 1) threads = 1;
    if (threads > rows) threads = (int)rows;
    job* jobs = (job*)malloc(sizeof(job) * (size_t)threads);
    pthread_t* tid = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)threads);
    if (!jobs || !tid) {
        free(jobs);
        free(tid);
        return -1;
    }
    int64_t chunk = rows / threads, extra = rows % threads, start = base->row_begin;
    for (int t = 0; t < threads; ++t) {
        jobs[t] = *base;
        jobs[t].t_begin = start;
        start += chunk + (t < extra ? 1 : 0);
        jobs[t].t_end = start;
    }
    for (int t = 1; t < threads; ++t) pthread_create(&tid[t], NULL, worker, &jobs[t]);
    worker(&jobs[0]);
    for (int t = 1; t < threads; ++t) pthread_join(tid[t], NULL);
    free(jobs);
    free(tid);
    return 0;
}

/*
 * Sweep rows [row_begin, row_end). Outputs (either may be NULL):
 *   row_sum[r - row_begin]   = sum over j of the ordered-pair increments of row r
 *                              (not halved, not scaled)
 *   grad[(r - row_begin)*p + k] = gradient component k of location r
 * Returns 0 on success.
 */
int mdso_sweep_rows(const void* delta, int delta_is_f32, const double* x, int64_t n, int p,
                    double tau, int truncation, int64_t row_begin, int64_t row_end,
                    double* row_sum, double* grad, int threads) {
    if (p < 1 || p > 64 || n < 0 || row_begin < 0 || row_end > n) return -1;
    job base;
    memset(&base, 0, sizeof(base));
    base.delta = delta;
    base.delta_is_f32 = delta_is_f32;
    base.x = x;
    base.n = n;
    base.p = p;
    base.tau = tau;
    base.truncation = truncation;
    base.want_sum = row_sum != NULL;
    base.want_grad = grad != NULL;
    base.row_begin = row_begin;
    base.row_end = row_end;
    base.row_sum = row_sum;
    base.grad = grad;
    return run(&base, threads);
}

/*
 * getSumOfIncrements() of the reference engine for the full matrix
 * (src/NewMultiDimensionalScaling.hpp:193-203, :524-561).
 */
double mdso_sum_of_increments(const void* delta, int delta_is_f32, const double* x, int64_t n,
                              int p, double tau, int truncation, int threads) {
    double* rows = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    if (!rows) return NAN;
    if (mdso_sweep_rows(delta, delta_is_f32, x, n, p, tau, truncation, 0, n, rows, NULL, threads)) {
        free(rows);
        return NAN;
    }
    nsum total = {0.0, 0.0};
    for (int64_t i = 0; i < n; ++i) nsum_add(&total, rows[i]);
    free(rows);
    double half = nsum_get(&total) / 2.0;
    return truncation ? half : 0.5 * tau * half;
}

/*
 * getLogLikelihoodGradient() of the reference engine
 * (src/NewMultiDimensionalScaling.hpp:281-334, :421-461); out has n*p entries.
 */
int mdso_gradient(const void* delta, int delta_is_f32, const double* x, int64_t n, int p,
                  double tau, int truncation, double* out, int threads) {
    return mdso_sweep_rows(delta, delta_is_f32, x, n, p, tau, truncation, 0, n, NULL, out, threads);
}

/* R/mds.R:24-28: log-likelihood from the sum of increments. */
double mdso_log_likelihood(double sum_of_increments, int64_t n, double tau) {
    const double observation_count = (double)n * (double)(n - 1) / 2.0;
    return 0.5 * (log(tau) - log(2.0 * M_PI)) * observation_count - sum_of_increments;
}

/*
 * The reference's own per-evaluation work order, restated for timing as the
 * CPU baseline port: for each row a likelihood pass (src/NewMultiDimensionalScaling.hpp:494-522)
 * and then a separate gradient pass (:421-461), both with libm transcendentals
 * and plain (uncompensated) accumulation in double. Covers rows
 * [row_begin, row_end) so a bounded sample of a large matrix can be timed.
 * Returns the (unhalved) partial sum of increments over those rows; writes the
 * gradient rows into grad.
 */
typedef struct {
    const void* delta;
    int delta_is_f32;
    const double* x;
    int64_t n;
    int p;
    double tau;
    int truncation;
    int64_t t_begin, t_end, row_begin;
    double* grad;
    double partial;
} port_job;

static void* port_worker(void* arg) {
    port_job* jb = (port_job*)arg;
    const int p = jb->p;
    const double sqrt_tau = sqrt(jb->tau), scale = 0.5 * jb->tau;
    double total = 0.0;
    for (int64_t i = jb->t_begin; i < jb->t_end; ++i) {
        const double* xi = jb->x + i * p;
        double row = 0.0;
        for (int64_t j = 0; j < jb->n; ++j) {
            double obs = jb->delta_is_f32 ? (double)((const float*)jb->delta)[i * jb->n + j]
                                          : ((const double*)jb->delta)[i * jb->n + j];
            if (i == j || isnan(obs)) continue;
            double d = distance(xi, jb->x + j * p, p);
            double r = obs - d, sq = r * r;
            if (jb->truncation) sq = sq * scale + log(0.5 * erfc(-d * sqrt_tau * MDSO_SQRT1_2));
            row += sq;
        }
        total += row;
        double* g = jb->grad + (i - jb->row_begin) * p;
        for (int k = 0; k < p; ++k) g[k] = 0.0;
        for (int64_t j = 0; j < jb->n; ++j) {
            double obs = jb->delta_is_f32 ? (double)((const float*)jb->delta)[i * jb->n + j]
                                          : ((const double*)jb->delta)[i * jb->n + j];
            if (i == j || isnan(obs)) continue;
            const double* xj = jb->x + j * p;
            double d = distance(xi, xj, p);
            double r = obs - d;
            if (jb->truncation) {
                double z = d * sqrt_tau;
                r -= MDSO_1_SQRT_2PI * exp(-0.5 * z * z) /
                     (exp(log(0.5 * erfc(-z * MDSO_SQRT1_2))) * sqrt_tau);
            }
            double c = r * jb->tau / d;
            for (int k = 0; k < p; ++k) g[k] += c * (xi[k] - xj[k]);
        }
    }
    jb->partial = total;
    return NULL;
}

double mdso_port_eval_rows(const void* delta, int delta_is_f32, const double* x, int64_t n, int p,
                           double tau, int truncation, int64_t row_begin, int64_t row_end,
                           double* grad, int threads) {
    int64_t rows = row_end - row_begin;
    if (rows <= 0) return 0.0;
    if (threads < 1) threads = 1;
    if (threads > rows) threads = (int)rows;
    port_job* jobs = (port_job*)calloc((size_t)threads, sizeof(port_job));
    pthread_t* tid = (pthread_t*)calloc((size_t)threads, sizeof(pthread_t));
    if (!jobs || !tid) {
        free(jobs);
        free(tid);
        return NAN;
    }
    int64_t chunk = rows / threads, extra = rows % threads, start = row_begin;
    for (int t = 0; t < threads; ++t) {
        port_job* jb = &jobs[t];
        jb->delta = delta;
        jb->delta_is_f32 = delta_is_f32;
        jb->x = x;
        jb->n = n;
        jb->p = p;
        jb->tau = tau;
        jb->truncation = truncation;
        jb->row_begin = row_begin;
        jb->grad = grad;
        jb->t_begin = start;
        start += chunk + (t < extra ? 1 : 0);
        jb->t_end = start;
    }
    for (int t = 1; t < threads; ++t) pthread_create(&tid[t], NULL, port_worker, &jobs[t]);
    port_worker(&jobs[0]);
    for (int t = 1; t < threads; ++t) pthread_join(tid[t], NULL);
    double total = 0.0;
    for (int t = 0; t < threads; ++t) total += jobs[t].partial;
    free(jobs);
    free(tid);
    return total;
}

/*
 * The reference's FLOAT engine (NewMultiDimensionalScaling<FloatNoSimdTypeInfo, ...>,
 * src/factory.cpp:42-62) per-evaluation work order, restated for timing as
 * the single-precision CPU baseline: the same likelihood pass and gradient
 * pass as mdso_port_eval_rows, with delta, locations, distances, residuals and
 * sums in float. As in the reference, logPhi and phi take a float argument
 * but evaluate erfc, log and exp in double (src/CDF.h:583-616: the constants
 * M_SQRT1_2 and M_1_SQRT_2PI are double) and round the result to float.
 * delta must be float. Returns the (unhalved) partial sum over the rows.
 */
typedef struct {
    const float* delta;
    const float* x;
    int64_t n;
    int p;
    float tau;
    int truncation;
    int64_t t_begin, t_end, row_begin;
    float* grad;
    double partial;
} port32_job;

static inline float distance_f32(const float* xi, const float* xj, int p) {
    float s = 0.0f;
    for (int k = 0; k < p; ++k) {
        float df = xi[k] - xj[k];
        s += df * df;
    }
    return sqrtf(s);
}

static void* port32_worker(void* arg) {
    port32_job* jb = (port32_job*)arg;
    const int p = jb->p;
    const float sqrt_tau = sqrtf(jb->tau), scale = 0.5f * jb->tau;
    float total = 0.0f;
    for (int64_t i = jb->t_begin; i < jb->t_end; ++i) {
        const float* xi = jb->x + i * p;
        float row = 0.0f;
        for (int64_t j = 0; j < jb->n; ++j) {
            const float obs = jb->delta[i * jb->n + j];
            if (i == j || isnan(obs)) continue;
            const float d = distance_f32(xi, jb->x + j * p, p);
            const float r = obs - d;
            float sq = r * r;
            if (jb->truncation) sq = sq * scale + (float)log(0.5 * erfc(-(d * sqrt_tau) * MDSO_SQRT1_2));
            row += sq;
        }
        total += row;
        float* g = jb->grad + (i - jb->row_begin) * p;
        for (int k = 0; k < p; ++k) g[k] = 0.0f;
        for (int64_t j = 0; j < jb->n; ++j) {
            const float obs = jb->delta[i * jb->n + j];
            if (i == j || isnan(obs)) continue;
            const float* xj = jb->x + j * p;
            const float d = distance_f32(xi, xj, p);
            float r = obs - d;
            if (jb->truncation) {
                const float z = d * sqrt_tau;
                const float pdf = (float)(MDSO_1_SQRT_2PI * exp(-0.5 * z * z));
                const float lphi = (float)log(0.5 * erfc(-z * MDSO_SQRT1_2));
                r -= pdf / (expf(lphi) * sqrt_tau);
            }
            const float c = r * jb->tau / d;
            for (int k = 0; k < p; ++k) g[k] += c * (xi[k] - xj[k]);
        }
    }
    jb->partial = total;
    return NULL;
}

double mdso_port_eval_rows_f32(const float* delta, const float* x, int64_t n, int p, float tau, int truncation,
                               int64_t row_begin, int64_t row_end, float* grad, int threads) {
    int64_t rows = row_end - row_begin;
    if (rows <= 0) return 0.0;
    if (threads < 1) threads = 1;
    if (threads > rows) threads = (int)rows;
    port32_job* jobs = (port32_job*)calloc((size_t)threads, sizeof(port32_job));
    pthread_t* tid = (pthread_t*)calloc((size_t)threads, sizeof(pthread_t));
    if (!jobs || !tid) {
        free(jobs);
        free(tid);
        return NAN;
    }
    int64_t chunk = rows / threads, extra = rows % threads, start = row_begin;
    for (int t = 0; t < threads; ++t) {
        port32_job* jb = &jobs[t];
        jb->delta = delta;
        jb->x = x;
        jb->n = n;
        jb->p = p;
        jb->tau = tau;
        jb->truncation = truncation;
        jb->row_begin = row_begin;
        jb->grad = grad;
        jb->t_begin = start;
        start += chunk + (t < extra ? 1 : 0);
        jb->t_end = start;
    }
    for (int t = 1; t < threads; ++t) pthread_create(&tid[t], NULL, port32_worker, &jobs[t]);
    port32_worker(&jobs[0]);
    for (int t = 1; t < threads; ++t) pthread_join(tid[t], NULL);
    double total = 0.0;
    for (int t = 0; t < threads; ++t) total += jobs[t].partial;
    free(jobs);
    free(tid);
    return total;
}
