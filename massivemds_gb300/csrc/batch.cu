// Batched multi-instance engine (mdsx_batch_* of the C ABI).
//
// Replaces the reference's many-engines pattern, a process-wide vector of
// independent engines addressed by index (src/jni/dr_inference_
// multidimensionalscaling_NativeMDSSingleton.cpp:10-100: initialize,
// updateLocations, getSumOfIncrements, getLogLikelihoodGradient,
// setPairwiseData, setParameters, makeDirty), by one object that owns every
// instance's data on one GPU and evaluates all of them with one persistent
// launch per (P, truncation) group, the launches captured once as a CUDA
// graph. Three schedules: stream-K over (row block x 128 columns) units of all
// instances (batch_kernel.cuh), a queue of whole row blocks taken
// dynamically, largest instance first (batch_queue.cuh), and stream-K over the
// unordered-pair units of all instances with a finish kernel (batch_pairs.cuh,
// P <= 6). Results of all instances come back in one
// device-to-host copy. Instance calls keep the reference's names and lazy
// semantics: a getter evaluates the batch when any instance changed.
//
// Location updates go to a pinned host copy per instance and reach the device
// with the next evaluation, so a caller updating every instance pays no
// synchronisation per call.
// Shapes (schedule, rows per warp, CTAs per SM) come from an autotuner that times
// the candidates on the batch itself and caches the winner per (P, N-bucket,
// truncation), in process and, when MDSX_TUNE_CACHE names a file, on disk.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/mdsx.h"
#include "batch_sweep.h"
#include "normal_rational.h"
#include "pair_plan.h"
#include "sweep.h"
#include "fault.h"

namespace mdsx {
namespace batch {

bool rw_built(int p, int rw) {
    if (p < 1 || p > 10) return false;
    return rw == 1 || (rw == 2 && p <= 8) || (rw == 4 && p <= 4);
}

// Shapes the kernels are built for: schedules 0 and 1 with rw_built rows per
// warp; schedule 2 (unordered pairs) with 4 rows per warp and P <= kPairMaxP.
bool shape_built(int p, int schedule, int rw) {
    if (schedule == 2) return rw == 4 && p >= 1 && p <= kPairMaxP;
    return (schedule == 0 || schedule == 1) && rw_built(p, rw);
}

int smem_bytes(int p, int rw) {
    const int rb = 8 * rw;
    return kStages * (rb * kStepCols * 4 + p * kStepCols * 4) + 2 * kStages * 8 + 128;
}

cudaError_t occupancy(int p, bool trunc, int rw, int* ctas, size_t* local_bytes) {
    return p <= 4 ? occupancy_lo(p, trunc, rw, ctas, local_bytes) : occupancy_hi(p, trunc, rw, ctas, local_bytes);
}

cudaError_t launch(int p, bool trunc, int rw, const BatchArgs& a, cudaStream_t st) {
    return p <= 4 ? launch_lo(p, trunc, rw, a, st) : launch_hi(p, trunc, rw, a, st);
}

cudaError_t occupancy_queue(int p, bool trunc, int rw, int* ctas) {
    return p <= 4 ? occupancy_queue_lo(p, trunc, rw, ctas) : occupancy_queue_hi(p, trunc, rw, ctas);
}

cudaError_t launch_queue(int p, bool trunc, int rw, const QueueArgs& a, int grid, cudaStream_t st) {
    return p <= 4 ? launch_queue_lo(p, trunc, rw, a, grid, st) : launch_queue_hi(p, trunc, rw, a, grid, st);
}

namespace {

// ------------------------------------------------------------ tuning cache

struct TuneKey {
    int p, bucket, trunc;
    bool operator<(const TuneKey& o) const { return std::tie(p, bucket, trunc) < std::tie(o.p, o.bucket, o.trunc); }
};
struct TuneValue {
    int schedule, rw, ctas_per_sm;  // schedule 0: stream-K (batch_kernel.cuh), 1: row-block queue (batch_queue.cuh)
    double us;
};

std::mutex g_tune_mu;
std::map<TuneKey, TuneValue> g_tune;
bool g_tune_loaded = false;

// N-bucket: floor(log2(mean N)).
int n_bucket(double mean_n) { return mean_n < 1.0 ? 0 : (int)std::floor(std::log2(mean_n)); }

void load_cache_locked() {
    if (g_tune_loaded) return;
    g_tune_loaded = true;
    const char* path = std::getenv("MDSX_TUNE_CACHE");
    if (!path) return;
    FILE* f = std::fopen(path, "r");
    if (!f) return;
    int p, b, t, sc, rw, c;
    double us;
    while (std::fscanf(f, "%d %d %d %d %d %d %lf", &p, &b, &t, &sc, &rw, &c, &us) == 7)
        if (shape_built(p, sc, rw) && c >= 1 && c <= 4) g_tune[{p, b, t}] = {sc, rw, c, us};
    std::fclose(f);
}

void save_cache_locked() {
    const char* path = std::getenv("MDSX_TUNE_CACHE");
    if (!path) return;
    FILE* f = std::fopen(path, "w");
    if (!f) return;
    for (const auto& kv : g_tune)
        std::fprintf(f, "%d %d %d %d %d %d %.3f\n", kv.first.p, kv.first.bucket, kv.first.trunc, kv.second.schedule,
                     kv.second.rw, kv.second.ctas_per_sm, kv.second.us);
    std::fclose(f);
}

// Default shape: the single-instance kernel's rows per warp, two CTAs per SM.
int default_rw(int p) { return p <= 4 ? 4 : (p <= 6 ? 2 : 1); }

PFN_cuTensorMapEncodeTiled_v12000 encode_tiled() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void* ptr = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(ptr);
    }
    return fn;
}

long long round_up(long long v, long long m) { return (v + m - 1) / m * m; }

}  // namespace
}  // namespace batch
}  // namespace mdsx

// ------------------------------------------------------------------ state

struct BatchInst {
    int p = 0, n = 0;
    double tau = 0.0;
    bool data_set = false;
    float* d_delta = nullptr;  // [n][ld]
    long long ld = 0;
    float* d_x = nullptr;      // SoA [p + 1][x_ld]; row p: missing-row flags
    int x_ld = 0;
    double* d_xin = nullptr;   // row-major [n][p] staging
    double* h_x = nullptr;     // pinned host copy of the locations, row-major [n][p]
    bool x_dirty = false;      // h_x changed since the last upload
    // plan-dependent
    int* d_row_nan = nullptr;
    int rows_padded = 0, n_row_blocks = 0;
    float* d_gpart = nullptr;
    double* d_lpart = nullptr;
    double* d_lrow = nullptr;
    unsigned* d_counts = nullptr;  // [R] row-block counters + [1] done counter
    double* d_qlpart = nullptr;    // queue schedule: [R][warps][2] likelihood partials
    unsigned* d_qdone = nullptr;   // queue schedule: row blocks finished
    float* d_prow = nullptr;       // pair schedule: row partials [units][32][P]
    float* d_pcol = nullptr;       // pair schedule: column partials [nb][max_slots][8][P][128]
    double* d_plp = nullptr;       // pair schedule: likelihood partials [CTAs meeting it][8][2]
    int* d_pjfirst = nullptr;      // pair schedule: first CTA per column block
    int* d_pjslots = nullptr;      // pair schedule: CTAs per column block
    long long grad_off = 0;        // offset (doubles) in the concatenated gradients
};

struct Shape {
    int schedule = 1, rw = 0, ctas = 0;
};

struct BatchGroup {
    int p = 0;
    bool trunc = false;
    int schedule = 1, rw = 0, ctas_per_sm = 0;
    std::vector<int> members;
    long long n_units = 0;
    int grid = 0;
    std::vector<mdsx::batch::BatchInstance> h_desc;
    mdsx::batch::BatchInstance* d_desc = nullptr;
    // queue schedule
    std::vector<int> order;  // members, largest N first (queue item order)
    std::vector<mdsx::batch::QueueInstance> h_qdesc;
    mdsx::batch::QueueInstance* d_qdesc = nullptr;
    unsigned long long* d_next = nullptr;
    long long n_items = 0;
    // unordered-pair schedule
    std::vector<mdsx::batch::PairInstance> h_pdesc;  // in member order
    mdsx::batch::PairInstance* d_pdesc = nullptr;
    long long* d_pbegin = nullptr;  // [grid + 1] global units per CTA
    int finish_blocks = 0;
    double work = 0.0;  // modelled cost: sum of N^2 x (16 + 3P) instructions per pair
};

struct mdsx_batch {
    int device = 0;
    long flags = 0;
    bool trunc = false;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    std::vector<BatchInst> inst;
    std::vector<BatchGroup> groups;
    bool planned = false, desc_dirty = true, graph_dirty = true, results_known = false;
    double* d_grad_all = nullptr;  // concatenated gradients
    double* d_sums_all = nullptr;  // [count][4]
    int* d_err = nullptr;
    double* h_results = nullptr;   // pinned: sums [count][4], then gradients
    long long grad_total = 0;
    cudaEvent_t uploaded = nullptr;  // recorded after the location uploads of an evaluation
    bool upload_pending = false;     // an upload from the pinned copies may still be in flight
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<cudaStream_t> aux;     // one branch stream per dimension group (graph capture)
    std::vector<cudaEvent_t> aux_ev;   // [0] fork, [1 + g] join of group g
    long long evaluations = 0;
    std::map<std::pair<int, int>, Shape> forced;  // (p, trunc) -> shape
    std::string last_error;
};

namespace {

using mdsx::batch::BatchArgs;
using mdsx::batch::BatchInstance;

int bfail(mdsx_batch* b, int code, const std::string& msg) {
    if (b) b->last_error = msg;
    return code;
}
#define BCUDA(b, call)                                                                                  \
    do {                                                                                                \
        cudaError_t _e = (call);                                                                        \
        if (_e != cudaSuccess)                                                                          \
            return bfail(b, _e == cudaErrorMemoryAllocation ? MDSX_ENOMEM : MDSX_ECUDA,                 \
                         std::string(#call) + ": " + cudaGetErrorString(_e));                           \
    } while (0)

struct Guard {
    int prev = -1;
    explicit Guard(int dev) {
        cudaGetDevice(&prev);
        if (prev != dev) cudaSetDevice(dev);
    }
    ~Guard() {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

void free_plan_scratch(BatchInst& in) {
    cudaFree(in.d_prow);
    cudaFree(in.d_pcol);
    cudaFree(in.d_plp);
    cudaFree(in.d_pjfirst);
    cudaFree(in.d_pjslots);
    in.d_prow = in.d_pcol = nullptr;
    in.d_plp = nullptr;
    in.d_pjfirst = in.d_pjslots = nullptr;
    cudaFree(in.d_qlpart);
    cudaFree(in.d_qdone);
    in.d_qlpart = nullptr;
    in.d_qdone = nullptr;
    cudaFree(in.d_row_nan);
    cudaFree(in.d_gpart);
    cudaFree(in.d_lpart);
    cudaFree(in.d_lrow);
    cudaFree(in.d_counts);
    in.d_row_nan = nullptr;
    in.d_gpart = nullptr;
    in.d_lpart = nullptr;
    in.d_lrow = nullptr;
    in.d_counts = nullptr;
}

void drop_graph(mdsx_batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    b->graph_dirty = true;
}

void free_plan(mdsx_batch* b) {
    drop_graph(b);
    for (auto& g : b->groups) {
        cudaFree(g.d_desc);
        cudaFree(g.d_qdesc);
        cudaFree(g.d_next);
        cudaFree(g.d_pdesc);
        cudaFree(g.d_pbegin);
    }
    b->groups.clear();
    for (auto& in : b->inst) free_plan_scratch(in);
    cudaFree(b->d_grad_all);
    cudaFree(b->d_sums_all);
    if (b->h_results) cudaFreeHost(b->h_results);
    b->d_grad_all = nullptr;
    b->d_sums_all = nullptr;
    b->h_results = nullptr;
    b->planned = false;
}

int make_tmap(mdsx_batch* b, CUtensorMap* map, void* base, long long cols, long long rows, long long ld,
              unsigned box_cols, unsigned box_rows, CUtensorMapSwizzle swizzle = CU_TENSOR_MAP_SWIZZLE_NONE) {
    auto fn = mdsx::batch::encode_tiled();
    if (!fn) return bfail(b, MDSX_ECUDA, "cuTensorMapEncodeTiled unavailable from the driver");
    cuuint64_t gdim[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t gstride[1] = {(cuuint64_t)(ld * 4)};
    cuuint32_t box[2] = {box_cols, box_rows};
    cuuint32_t estride[2] = {1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, base, gdim, gstride, box, estride,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return bfail(b, MDSX_ECUDA, "cuTensorMapEncodeTiled failed");
    return MDSX_OK;
}

// Precision constants of one instance (the single-instance engine's make_args).
template <typename D>
void set_precision_constants(D& d, double tau) {
    const double s = std::sqrt(tau);
    d.tau = tau;
    d.k_e = (float)(-0.5 * tau * 1.4426950408889634074);
    d.log2_k2 = (float)std::log2(1.0 / std::sqrt(2.0 * M_PI * tau));
    d.tp0 = (float)(mdsx::kTailP0 / tau);
    d.tp1 = (float)(mdsx::kTailP1 / s);
    d.tp2 = (float)mdsx::kTailP2;
    d.ts0 = (float)(mdsx::kTailS0 / (s * s * s));
    d.ts1 = (float)(mdsx::kTailS1 / (s * s));
    d.ts2 = (float)(mdsx::kTailS2 / s);
}

// Unordered-pair schedule of one group: the members' unit lists (pair_kernel.cuh)
// concatenated in member order and split over the group's CTAs (all SMs at the
// group's occupancy) by modelled cost (pair_unit_cost); per member the slot
// tables of its column blocks, its partial buffers, tensor maps and a PairArgs
// descriptor.
int plan_pairs_group(mdsx_batch* b, BatchGroup& g) {
    std::vector<int> ns;
    for (int k : g.members) ns.push_back(b->inst[k].n);
    const mdsx::PairPlan plan = mdsx::pair_plan(ns, (long long)b->sm_count * g.ctas_per_sm);
    g.n_units = plan.units;
    g.grid = plan.grid;
    const int G = plan.grid;
    const std::vector<long long>& begin = plan.cta_begin;
    cudaStream_t st = b->stream;
    int finish = 0;
    for (size_t m = 0; m < g.members.size(); ++m) {
        BatchInst& in = b->inst[g.members[m]];
        const mdsx::PairInstancePlan& q = plan.inst[m];
        const std::vector<int>& jfirst = q.j_first;
        const std::vector<int>& jslots = q.j_slots;
        const int max_slots = q.max_slots;
        const int first_cta = q.first_cta;
        const int islots = q.ctas;
        BCUDA(b, mdsx::device_malloc(&in.d_prow, (size_t)q.units * mdsx::kPairRows * g.p * sizeof(float)));
        BCUDA(b, mdsx::device_malloc(&in.d_pcol,
                            (size_t)q.nb * max_slots * mdsx::kPairWarps * g.p * mdsx::kPairCols * sizeof(float)));
        BCUDA(b, mdsx::device_malloc(&in.d_plp, (size_t)islots * mdsx::kPairWarps * 2 * sizeof(double)));
        BCUDA(b, mdsx::device_malloc(&in.d_pjfirst, (size_t)q.nb * sizeof(int)));
        BCUDA(b, mdsx::device_malloc(&in.d_pjslots, (size_t)q.nb * sizeof(int)));
        BCUDA(b, cudaMemcpyAsync(in.d_pjfirst, jfirst.data(), (size_t)q.nb * sizeof(int), cudaMemcpyHostToDevice, st));
        BCUDA(b, cudaMemcpyAsync(in.d_pjslots, jslots.data(), (size_t)q.nb * sizeof(int), cudaMemcpyHostToDevice, st));
        BCUDA(b, cudaStreamSynchronize(st));  // the host tables go out of scope
        mdsx::batch::PairInstance d{};
        int rc = make_tmap(b, &d.tmap_a, in.d_delta, in.n, in.n, in.ld, mdsx::kPairCols, mdsx::kPairRows);
        if (!rc)
            rc = make_tmap(b, &d.tmap_b, in.d_delta, in.n, in.n, in.ld, mdsx::kPairRows, mdsx::kPairCols,
                           CU_TENSOR_MAP_SWIZZLE_128B);
        // the location maps span x_ld columns, so the flags past N are read from memory (1), not filled
        if (!rc) rc = make_tmap(b, &d.tmap_xi, in.d_x, in.x_ld, g.p + 1, in.x_ld, mdsx::kPairRows, g.p + 1);
        if (!rc) rc = make_tmap(b, &d.tmap_xj, in.d_x, in.x_ld, g.p + 1, in.x_ld, mdsx::kPairCols, g.p + 1);
        if (rc) return rc;
        mdsx::PairArgs& a = d.args;
        a.n = in.n;
        a.nb = q.nb;
        a.nc = q.nc;
        a.grid = islots;
        a.max_slots = max_slots;
        a.truncation = g.trunc ? 1 : 0;
        a.n_units = q.units;
        set_precision_constants(a, in.tau);
        a.sqrt_tau = std::sqrt(in.tau);
        a.rowpart = in.d_prow;
        a.colpart = in.d_pcol;
        a.lpart = in.d_plp;
        a.j_first_cta = in.d_pjfirst;
        a.j_slots = in.d_pjslots;
        d.unit_begin = q.unit_begin;
        d.first_cta = first_cta;
        d.finish_begin = finish;
        finish += q.nc + 1;
        g.h_pdesc.push_back(d);
    }
    g.finish_blocks = finish;
    BCUDA(b, mdsx::device_malloc(&g.d_pdesc, g.h_pdesc.size() * sizeof(mdsx::batch::PairInstance)));
    BCUDA(b, mdsx::device_malloc(&g.d_pbegin, (size_t)(G + 1) * sizeof(long long)));
    BCUDA(b, cudaMemcpy(g.d_pbegin, begin.data(), (size_t)(G + 1) * sizeof(long long), cudaMemcpyHostToDevice));
    return MDSX_OK;
}

// Shape of a group: the override, else the tuning cache, else the default: with
// truncation and P <= 6 the unordered-pair schedule (the single-instance
// engine's choice), otherwise the row-block queue with the single-instance rows
// per warp; full occupancy.
Shape group_shape(const mdsx_batch* b, int p, double mean_n, const std::map<std::pair<int, int>, Shape>* force) {
    Shape sh;
    sh.rw = mdsx::batch::default_rw(p);
    if (b->trunc && p <= mdsx::kPairMaxP) {
        sh.schedule = 2;
        sh.rw = 4;
    }
    {
        std::lock_guard<std::mutex> lock(mdsx::batch::g_tune_mu);
        mdsx::batch::load_cache_locked();
        auto it = mdsx::batch::g_tune.find({p, mdsx::batch::n_bucket(mean_n), b->trunc ? 1 : 0});
        if (it != mdsx::batch::g_tune.end()) sh = {it->second.schedule, it->second.rw, it->second.ctas_per_sm};
    }
    if (force) {
        auto it = force->find({p, b->trunc ? 1 : 0});
        if (it != force->end()) sh = it->second;
    }
    return sh;
}

// Builds the groups, scratch, descriptors and result buffers. `force` maps a
// group key (p, trunc) to a shape that overrides the cache.
int plan(mdsx_batch* b, const std::map<std::pair<int, int>, Shape>* force = nullptr) {
    if (b->inst.empty()) return bfail(b, MDSX_ESTATE, "batch has no instances");
    for (size_t k = 0; k < b->inst.size(); ++k) {
        if (!b->inst[k].data_set) return bfail(b, MDSX_ESTATE, "instance " + std::to_string(k) + ": no pairwise data");
        if (!(b->inst[k].tau > 0.0)) return bfail(b, MDSX_ESTATE, "instance " + std::to_string(k) + ": precision not set");
    }
    free_plan(b);
    cudaStream_t st = b->stream;
    // gradients concatenated in instance order
    long long grad_off = 0;
    for (auto& in : b->inst) {
        in.grad_off = grad_off;
        grad_off += (long long)in.n * in.p;
    }
    // groups by P (one truncation mode per batch); they run concurrently as graph branches
    std::map<int, std::vector<int>> by_p;
    for (size_t k = 0; k < b->inst.size(); ++k) by_p[b->inst[k].p].push_back((int)k);
    double total_work = 0.0;
    for (const auto& in : b->inst) total_work += (double)in.n * in.n * (16.0 + 3.0 * in.p);
    const bool concurrent = by_p.size() > 1;
    for (auto& kv : by_p) {
        BatchGroup g;
        g.p = kv.first;
        g.trunc = b->trunc;
        g.members = kv.second;
        double mean_n = 0.0;
        for (int k : g.members) mean_n += b->inst[k].n;
        mean_n /= g.members.size();
        const Shape sh = group_shape(b, g.p, mean_n, force);
        int occ = 0;
        size_t local = 0;
        if (sh.schedule == 0)
            BCUDA(b, mdsx::batch::occupancy(g.p, g.trunc, sh.rw, &occ, &local));
        else if (sh.schedule == 1)
            BCUDA(b, mdsx::batch::occupancy_queue(g.p, g.trunc, sh.rw, &occ));
        else
            BCUDA(b, mdsx::batch::occupancy_pairs(g.p, g.trunc, &occ));
        if (occ < 1) return bfail(b, MDSX_ECUDA, "batched sweep kernel cannot be resident");
        g.schedule = sh.schedule;
        g.rw = sh.rw;
        g.ctas_per_sm = sh.ctas >= 1 ? std::min(sh.ctas, occ) : occ;
        const int rb = 8 * g.rw;
        g.work = 0.0;
        for (int k : g.members) g.work += (double)b->inst[k].n * b->inst[k].n * (16.0 + 3.0 * g.p);
        // per instance: row blocks, missing-row marks and flags
        for (int k : g.members) {
            BatchInst& in = b->inst[k];
            in.n_row_blocks = (in.n + rb - 1) / rb;
            in.rows_padded = in.n_row_blocks * rb;
            BCUDA(b, mdsx::device_malloc(&in.d_row_nan, (size_t)in.rows_padded * sizeof(int)));
            BCUDA(b, mdsx::mark_nan_rows(in.d_delta, true, in.n, in.ld, in.d_row_nan, in.rows_padded, st));
            // flag row: 1 for rows with a NaN and for columns n .. x_ld (read by the pair schedule)
            BCUDA(b, mdsx::write_flag_row(in.d_row_nan, in.n, in.rows_padded, in.d_x + (size_t)g.p * in.x_ld, true,
                                          in.x_ld, st));
        }
        if (g.schedule == 0) {
            // stream-K: global units, slots, scratch
            for (int k : g.members) {
                BatchInst& in = b->inst[k];
                BatchInstance d{};
                d.unit_begin = g.n_units;
                d.n = in.n;
                d.n_row_blocks = in.n_row_blocks;
                d.steps_per_row = (in.n + mdsx::kStepCols - 1) / mdsx::kStepCols;
                d.x_ld = in.x_ld;
                d.truncation = g.trunc ? 1 : 0;
                set_precision_constants(d, in.tau);
                g.n_units += (long long)d.n_row_blocks * d.steps_per_row;
                g.h_desc.push_back(d);
            }
            long long slots = (long long)b->sm_count * g.ctas_per_sm;
            if (concurrent) slots = std::max<long long>(1, std::llround(slots * g.work / total_work));
            g.grid = (int)std::min<long long>(g.n_units, slots);
            for (size_t m = 0; m < g.members.size(); ++m) {
                BatchInst& in = b->inst[g.members[m]];
                BatchInstance& d = g.h_desc[m];
                int max_slots = 1;
                for (int r = 0; r < d.n_row_blocks; ++r) {
                    const long long u0 = d.unit_begin + (long long)r * d.steps_per_row, u1 = u0 + d.steps_per_row - 1;
                    max_slots = std::max(max_slots, mdsx::cta_of_unit(u1, g.n_units, g.grid) -
                                                        mdsx::cta_of_unit(u0, g.n_units, g.grid) + 1);
                }
                d.max_slots = max_slots;
                BCUDA(b, mdsx::device_malloc(&in.d_gpart, (size_t)d.n_row_blocks * max_slots * rb * g.p * sizeof(float)));
                BCUDA(b, mdsx::device_malloc(&in.d_lpart,
                                    (size_t)d.n_row_blocks * max_slots * mdsx::kConsumerWarps * 2 * sizeof(double)));
                BCUDA(b, mdsx::device_malloc(&in.d_lrow, (size_t)d.n_row_blocks * 2 * sizeof(double)));
                BCUDA(b, mdsx::device_malloc(&in.d_counts, ((size_t)d.n_row_blocks + 1) * sizeof(unsigned)));
                BCUDA(b, cudaMemsetAsync(in.d_counts, 0, ((size_t)d.n_row_blocks + 1) * sizeof(unsigned), st));
                int rc = make_tmap(b, &d.tmap_delta, in.d_delta, in.n, in.n, in.ld, mdsx::kStepCols, rb);
                if (!rc) rc = make_tmap(b, &d.tmap_x, in.d_x, in.n, g.p, in.x_ld, mdsx::kStepCols, g.p);
                if (rc) return rc;
                d.x = in.d_x;
                d.row_nan = in.d_row_nan;
                d.gpart = in.d_gpart;
                d.lpart = in.d_lpart;
                d.lrow = in.d_lrow;
                d.rb_count = in.d_counts;
                d.done_count = in.d_counts + d.n_row_blocks;
            }
            BCUDA(b, mdsx::device_malloc(&g.d_desc, g.h_desc.size() * sizeof(BatchInstance)));
        } else if (g.schedule == 2) {
            // full residency, as the queue: the CTAs never wait on one another, so
            // concurrent groups simply share the SMs
            int rc = plan_pairs_group(b, g);
            if (rc) return rc;
        } else {
            // row-block queue: items ordered largest instance first
            g.order = g.members;
            std::stable_sort(g.order.begin(), g.order.end(),
                             [&](int x, int y) { return b->inst[x].n > b->inst[y].n; });
            for (int k : g.order) {
                BatchInst& in = b->inst[k];
                mdsx::batch::QueueInstance d{};
                d.n = in.n;
                d.n_row_blocks = in.n_row_blocks;
                d.steps_per_row = (in.n + mdsx::kStepCols - 1) / mdsx::kStepCols;
                d.truncation = g.trunc ? 1 : 0;
                d.item_begin = g.n_items;
                set_precision_constants(d, in.tau);
                g.n_items += in.n_row_blocks;
                BCUDA(b, mdsx::device_malloc(&in.d_qlpart, (size_t)in.n_row_blocks * mdsx::kConsumerWarps * 2 * sizeof(double)));
                BCUDA(b, mdsx::device_malloc(&in.d_qdone, sizeof(unsigned)));
                BCUDA(b, cudaMemsetAsync(in.d_qdone, 0, sizeof(unsigned), st));
                int rc = make_tmap(b, &d.tmap_delta, in.d_delta, in.n, in.n, in.ld, mdsx::kStepCols, rb);
                if (!rc) rc = make_tmap(b, &d.tmap_x, in.d_x, in.n, g.p + 1, in.x_ld, mdsx::kStepCols, g.p + 1);
                if (rc) return rc;
                d.lpart = in.d_qlpart;
                d.done_count = in.d_qdone;
                g.h_qdesc.push_back(d);
            }
            g.grid = (int)std::max<long long>(1, std::min<long long>(g.n_items, (long long)b->sm_count * g.ctas_per_sm));
            BCUDA(b, mdsx::device_malloc(&g.d_qdesc, g.h_qdesc.size() * sizeof(mdsx::batch::QueueInstance)));
            BCUDA(b, mdsx::device_malloc(&g.d_next, sizeof(unsigned long long)));
        }
        b->groups.push_back(std::move(g));
    }
    b->grad_total = grad_off;
    const size_t count = b->inst.size();
    BCUDA(b, mdsx::device_malloc(&b->d_grad_all, (size_t)std::max<long long>(1, grad_off) * sizeof(double)));
    BCUDA(b, mdsx::device_malloc(&b->d_sums_all, count * 4 * sizeof(double)));
    BCUDA(b, cudaMemsetAsync(b->d_sums_all, 0, count * 4 * sizeof(double), st));
    BCUDA(b, mdsx::host_malloc(&b->h_results, (count * 4 + (size_t)grad_off) * sizeof(double)));
    // output pointers (instance order in the sums array is the instance index)
    for (auto& g : b->groups) {
        for (size_t m = 0; m < g.h_desc.size(); ++m) {
            const int k = g.members[m];
            g.h_desc[m].grad_out = b->d_grad_all + b->inst[k].grad_off;
            g.h_desc[m].sums_out = b->d_sums_all + 4 * (size_t)k;
        }
        for (size_t m = 0; m < g.h_qdesc.size(); ++m) {
            const int k = g.order[m];
            g.h_qdesc[m].grad_out = b->d_grad_all + b->inst[k].grad_off;
            g.h_qdesc[m].sums_out = b->d_sums_all + 4 * (size_t)k;
        }
        for (size_t m = 0; m < g.h_pdesc.size(); ++m) {
            const int k = g.members[m];
            g.h_pdesc[m].args.grad_out = b->d_grad_all + b->inst[k].grad_off;
            g.h_pdesc[m].args.sums_out = b->d_sums_all + 4 * (size_t)k;
            g.h_pdesc[m].args.err = b->d_err;
        }
    }
    while (b->aux.size() < b->groups.size()) {  // branch streams for concurrent groups (created outside capture)
        cudaStream_t bs = nullptr;
        BCUDA(b, cudaStreamCreateWithFlags(&bs, cudaStreamNonBlocking));
        b->aux.push_back(bs);
    }
    while (b->aux_ev.size() < b->groups.size() + 1) {
        cudaEvent_t ev = nullptr;
        BCUDA(b, cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        b->aux_ev.push_back(ev);
    }
    b->planned = true;
    b->desc_dirty = true;
    b->graph_dirty = true;
    BCUDA(b, cudaStreamSynchronize(st));
    return MDSX_OK;
}

int upload_descriptors(mdsx_batch* b) {
    for (auto& g : b->groups) {
        if (!g.h_desc.empty())
            BCUDA(b, cudaMemcpyAsync(g.d_desc, g.h_desc.data(), g.h_desc.size() * sizeof(BatchInstance),
                                     cudaMemcpyHostToDevice, b->stream));
        if (!g.h_qdesc.empty())
            BCUDA(b, cudaMemcpyAsync(g.d_qdesc, g.h_qdesc.data(), g.h_qdesc.size() * sizeof(mdsx::batch::QueueInstance),
                                     cudaMemcpyHostToDevice, b->stream));
        if (!g.h_pdesc.empty())
            BCUDA(b, cudaMemcpyAsync(g.d_pdesc, g.h_pdesc.data(), g.h_pdesc.size() * sizeof(mdsx::batch::PairInstance),
                                     cudaMemcpyHostToDevice, b->stream));
    }
    BCUDA(b, cudaStreamSynchronize(b->stream));  // the host descriptors may change after return
    b->desc_dirty = false;
    return MDSX_OK;
}

BatchArgs group_args(const mdsx_batch* b, const BatchGroup& g) {
    BatchArgs a{};
    a.inst = g.d_desc;
    a.count = (int)g.members.size();
    a.n_units = g.n_units;
    a.grid = g.grid;
    a.err = b->d_err;
    return a;
}

// One group's launch on stream st (the queue schedule first resets its counter).
int launch_group(mdsx_batch* b, const BatchGroup& g, cudaStream_t st) {
    if (g.schedule == 0) {
        BCUDA(b, mdsx::batch::launch(g.p, g.trunc, g.rw, group_args(b, g), st));
        return MDSX_OK;
    }
    if (g.schedule == 2) {
        mdsx::batch::BatchPairArgs a{};
        a.inst = g.d_pdesc;
        a.count = (int)g.h_pdesc.size();
        a.cta_begin = g.d_pbegin;
        a.err = b->d_err;
        BCUDA(b, mdsx::batch::launch_pairs(g.p, g.trunc, a, g.grid, g.finish_blocks, st));
        return MDSX_OK;
    }
    mdsx::batch::QueueArgs a{};
    a.inst = g.d_qdesc;
    a.count = (int)g.h_qdesc.size();
    a.n_items = g.n_items;
    a.next = g.d_next;
    a.err = b->d_err;
    BCUDA(b, cudaMemsetAsync(g.d_next, 0, sizeof(unsigned long long), st));
    BCUDA(b, mdsx::batch::launch_queue(g.p, g.trunc, g.rw, a, g.grid, st));
    return MDSX_OK;
}

// The group launches: one group on the batch stream, several as concurrent
// branches (fork from and join back to the batch stream).
int enqueue_groups(mdsx_batch* b) {
    if (b->groups.size() == 1) return launch_group(b, b->groups[0], b->stream);
    if (b->aux.size() < b->groups.size() || b->aux_ev.size() < b->groups.size() + 1)
        return bfail(b, MDSX_ESTATE, "branch streams missing (plan)");
    BCUDA(b, cudaEventRecord(b->aux_ev[0], b->stream));
    for (size_t i = 0; i < b->groups.size(); ++i) {
        BCUDA(b, cudaStreamWaitEvent(b->aux[i], b->aux_ev[0], 0));
        const int rc = launch_group(b, b->groups[i], b->aux[i]);
        if (rc) return rc;
        BCUDA(b, cudaEventRecord(b->aux_ev[1 + i], b->aux[i]));
        BCUDA(b, cudaStreamWaitEvent(b->stream, b->aux_ev[1 + i], 0));
    }
    return MDSX_OK;
}

// Uploads the locations of every instance updated since the last upload (one
// copy from its pinned host copy and one layout conversion each) on the batch
// stream, and records `uploaded` behind them.
int flush_uploads(mdsx_batch* b) {
    bool any = false;
    for (auto& in : b->inst) {
        if (!in.x_dirty) continue;
        BCUDA(b, cudaMemcpyAsync(in.d_xin, in.h_x, (size_t)in.n * in.p * sizeof(double), cudaMemcpyHostToDevice,
                                 b->stream));
        BCUDA(b, mdsx::convert_locations(in.d_xin, in.n, in.p, in.d_x, in.x_ld, true, b->stream));
        in.x_dirty = false;
        any = true;
    }
    if (any) {
        BCUDA(b, cudaEventRecord(b->uploaded, b->stream));
        b->upload_pending = true;
    }
    return MDSX_OK;
}

// Enqueues one evaluation of every instance (graph launch); no synchronisation.
int enqueue_evaluation(mdsx_batch* b) {
    if (!b->planned) {
        int rc = plan(b, b->forced.empty() ? nullptr : &b->forced);
        if (rc) return rc;
    }
    if (b->desc_dirty) {
        int rc = upload_descriptors(b);
        if (rc) return rc;
    }
    {
        int rc = flush_uploads(b);
        if (rc) return rc;
    }
    if (b->graph_dirty) {
        drop_graph(b);
        BCUDA(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        const int rc = enqueue_groups(b);
        cudaGraph_t gr = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(b->stream, &gr);
        if (rc) {
            if (gr) cudaGraphDestroy(gr);
            return rc;
        }
        BCUDA(b, ce);
        b->graph = gr;
        BCUDA(b, cudaGraphInstantiate(&b->exec, gr, 0));
        b->graph_dirty = false;
    }
    BCUDA(b, mdsx::launch_fault());
    BCUDA(b, cudaGraphLaunch(b->exec, b->stream));
    ++b->evaluations;
    return MDSX_OK;
}

// Evaluates if needed and brings every instance's sums and gradient to the host.
int ensure_results(mdsx_batch* b) {
    if (b->results_known) return MDSX_OK;
    int rc = enqueue_evaluation(b);
    if (rc) return rc;
    const size_t count = b->inst.size();
    BCUDA(b, cudaMemcpyAsync(b->h_results, b->d_sums_all, count * 4 * sizeof(double), cudaMemcpyDeviceToHost,
                             b->stream));
    BCUDA(b, cudaMemcpyAsync(b->h_results + count * 4, b->d_grad_all, (size_t)b->grad_total * sizeof(double),
                             cudaMemcpyDeviceToHost, b->stream));
    int err = 0;
    BCUDA(b, cudaMemcpyAsync(&err, b->d_err, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
    BCUDA(b, cudaStreamSynchronize(b->stream));
    if (err) {
        cudaMemsetAsync(b->d_err, 0, sizeof(int), b->stream);
        for (auto& in : b->inst)
            if (in.d_counts)
                cudaMemsetAsync(in.d_counts, 0, ((size_t)in.n_row_blocks + 1) * sizeof(unsigned), b->stream);
        for (auto& in : b->inst)
            if (in.d_qdone) cudaMemsetAsync(in.d_qdone, 0, sizeof(unsigned), b->stream);
        cudaStreamSynchronize(b->stream);
        return bfail(b, MDSX_ETIMEOUT, "a bounded device wait in the batched sweep timed out");
    }
    b->results_known = true;
    return MDSX_OK;
}

int check_instance(mdsx_batch* b, int k) {
    if (k < 0 || k >= (int)b->inst.size()) return bfail(b, MDSX_EINVAL, "instance index out of range");
    return MDSX_OK;
}

}  // namespace

extern "C" {

int mdsx_batch_create(long flags, int device, mdsx_batch** out) {
    if (!out) return MDSX_EINVAL;
    *out = nullptr;
    if (!(flags & MDSX_FLAG_FLOAT)) return MDSX_EUNSUPPORTED;  // the batched path computes in FP32
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return MDSX_ECUDA;
    if (device < 0 && cudaGetDevice(&device) != cudaSuccess) device = 0;
    if (device >= count) return MDSX_EINVAL;
    Guard guard(device);
    auto* b = new mdsx_batch;
    b->device = device;
    b->flags = flags;
    b->trunc = (flags & MDSX_FLAG_LEFT_TRUNCATION) != 0;
    if (cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->uploaded, cudaEventDisableTiming) != cudaSuccess ||
        mdsx::device_malloc(&b->d_err, sizeof(int)) != cudaSuccess || cudaMemset(b->d_err, 0, sizeof(int)) != cudaSuccess) {
        if (b->stream) cudaStreamDestroy(b->stream);
        if (b->uploaded) cudaEventDestroy(b->uploaded);
        cudaFree(b->d_err);
        delete b;
        return MDSX_ECUDA;
    }
    *out = b;
    return MDSX_OK;
}

void mdsx_batch_destroy(mdsx_batch* b) {
    if (!b) return;
    Guard guard(b->device);
    cudaStreamSynchronize(b->stream);
    free_plan(b);
    for (auto& in : b->inst) {
        cudaFree(in.d_delta);
        cudaFree(in.d_x);
        cudaFree(in.d_xin);
        if (in.h_x) cudaFreeHost(in.h_x);
    }
    if (b->uploaded) cudaEventDestroy(b->uploaded);
    cudaFree(b->d_err);
    for (cudaStream_t st : b->aux) cudaStreamDestroy(st);
    for (cudaEvent_t ev : b->aux_ev) cudaEventDestroy(ev);
    cudaStreamDestroy(b->stream);
    delete b;
}

const char* mdsx_batch_last_error(const mdsx_batch* b) { return b ? b->last_error.c_str() : "NULL batch"; }

int mdsx_batch_instance_count(const mdsx_batch* b) { return b ? (int)b->inst.size() : 0; }

// The reference's JNI initialize(dimension, locations, ...): returns the new instance's index.
int mdsx_batch_add_instance(mdsx_batch* b, int embedding_dimension, int location_count, int* instance) {
    if (!b) return MDSX_EINVAL;
    if (!instance) return bfail(b, MDSX_EINVAL, "instance is NULL");
    if (embedding_dimension < 1 || embedding_dimension > MDSX_MAX_DIMENSION)
        return bfail(b, MDSX_EUNSUPPORTED, "embedding dimension outside 1..MDSX_MAX_DIMENSION");
    if (location_count < 2 || location_count > (1 << 20)) return bfail(b, MDSX_EINVAL, "locationCount outside 2..2^20");
    Guard guard(b->device);
    BatchInst in;
    in.p = embedding_dimension;
    in.n = location_count;
    in.ld = mdsx::batch::round_up(in.n, 4);
    in.x_ld = (int)mdsx::batch::round_up(in.n, mdsx::kStepCols);
    const size_t xb = (size_t)(in.p + 1) * in.x_ld * sizeof(float);  // row P: missing-row flags
    if (mdsx::device_malloc(&in.d_delta, (size_t)in.n * in.ld * sizeof(float)) != cudaSuccess ||
        mdsx::device_malloc(&in.d_x, xb) != cudaSuccess ||
        mdsx::device_malloc(&in.d_xin, (size_t)in.n * in.p * sizeof(double)) != cudaSuccess ||
        mdsx::host_malloc(&in.h_x, (size_t)in.n * in.p * sizeof(double)) != cudaSuccess) {
        cudaFree(in.d_delta);
        cudaFree(in.d_x);
        cudaFree(in.d_xin);
        if (in.h_x) cudaFreeHost(in.h_x);
        return bfail(b, MDSX_ENOMEM, "instance allocation failed");
    }
    std::memset(in.h_x, 0, (size_t)in.n * in.p * sizeof(double));
    BCUDA(b, cudaMemsetAsync(in.d_x, 0, xb, b->stream));
    BCUDA(b, cudaStreamSynchronize(b->stream));
    *instance = (int)b->inst.size();
    b->inst.push_back(in);
    free_plan(b);  // the groups change
    b->results_known = false;
    return MDSX_OK;
}

static int set_delta(mdsx_batch* b, int k, const float* host_rows) {
    BatchInst& in = b->inst[k];
    BCUDA(b, cudaMemcpy2DAsync(in.d_delta, in.ld * sizeof(float), host_rows, (size_t)in.n * sizeof(float),
                               (size_t)in.n * sizeof(float), in.n, cudaMemcpyHostToDevice, b->stream));
    BCUDA(b, cudaStreamSynchronize(b->stream));
    in.data_set = true;
    free_plan(b);  // NaN rows and tensor maps are rebuilt by the next plan
    b->results_known = false;
    return MDSX_OK;
}

// setPairwiseData of one instance: N*N row-major doubles (NaN = missing), stored as FP32.
int mdsx_batch_set_pairwise_data(mdsx_batch* b, int k, const double* data, size_t length) {
    if (!b) return MDSX_EINVAL;
    int rc = check_instance(b, k);
    if (rc) return rc;
    const BatchInst& in = b->inst[k];
    if (!data || length != (size_t)in.n * in.n) return bfail(b, MDSX_EINVAL, "pairwise data must hold N*N values");
    Guard guard(b->device);
    std::vector<float> rows(length);
    for (size_t i = 0; i < length; ++i) rows[i] = (float)data[i];
    return set_delta(b, k, rows.data());
}

int mdsx_batch_set_pairwise_data_f32(mdsx_batch* b, int k, const float* data, size_t length) {
    if (!b) return MDSX_EINVAL;
    int rc = check_instance(b, k);
    if (rc) return rc;
    const BatchInst& in = b->inst[k];
    if (!data || length != (size_t)in.n * in.n) return bfail(b, MDSX_EINVAL, "pairwise data must hold N*N values");
    Guard guard(b->device);
    return set_delta(b, k, data);
}

// setParameters of one instance: parameters[0] = precision tau > 0.
int mdsx_batch_set_parameters(mdsx_batch* b, int k, const double* parameters, size_t length) {
    if (!b) return MDSX_EINVAL;
    int rc = check_instance(b, k);
    if (rc) return rc;
    if (!parameters || length < 1 || !(parameters[0] > 0.0) || !std::isfinite(parameters[0]))
        return bfail(b, MDSX_EINVAL, "precision must be finite and > 0");
    b->inst[k].tau = parameters[0];
    for (auto& g : b->groups) {
        for (size_t m = 0; m < g.h_desc.size(); ++m)
            if (g.members[m] == k) set_precision_constants(g.h_desc[m], parameters[0]);
        for (size_t m = 0; m < g.h_qdesc.size(); ++m)
            if (g.order[m] == k) set_precision_constants(g.h_qdesc[m], parameters[0]);
        for (size_t m = 0; m < g.h_pdesc.size(); ++m)
            if (g.members[m] == k) {
                set_precision_constants(g.h_pdesc[m].args, parameters[0]);
                g.h_pdesc[m].args.sqrt_tau = std::sqrt(parameters[0]);
            }
    }
    b->desc_dirty = true;
    b->results_known = false;
    return MDSX_OK;
}

// updateLocations of one instance: index -1 with N*P row-major doubles, or one location (P doubles).
int mdsx_batch_update_locations(mdsx_batch* b, int k, int index, const double* locations, size_t length) {
    if (!b) return MDSX_EINVAL;
    int rc = check_instance(b, k);
    if (rc) return rc;
    BatchInst& in = b->inst[k];
    if (!locations) return bfail(b, MDSX_EINVAL, "locations is NULL");
    if (index == -1) {
        if (length != (size_t)in.n * in.p) return bfail(b, MDSX_EINVAL, "locations must hold N*P values");
    } else if (index < 0 || index >= in.n || length != (size_t)in.p) {
        return bfail(b, MDSX_EINVAL, "location index out of range or length != P");
    }
    // The values go to the instance's pinned host copy now and to the device with
    // the next evaluation (one copy per changed instance, no synchronisation per
    // call). Wait only if an upload from the pinned copies may still be reading them.
    if (b->upload_pending) {
        Guard guard(b->device);
        BCUDA(b, cudaEventSynchronize(b->uploaded));
        b->upload_pending = false;
    }
    std::memcpy(in.h_x + (index == -1 ? 0 : (size_t)index * in.p), locations, length * sizeof(double));
    in.x_dirty = true;
    b->results_known = false;
    return MDSX_OK;
}

// makeDirty: forces the next getter to evaluate again.
int mdsx_batch_make_dirty(mdsx_batch* b) {
    if (!b) return MDSX_EINVAL;
    b->results_known = false;
    return MDSX_OK;
}

// One evaluation of every instance, results read back to the host.
int mdsx_batch_evaluate(mdsx_batch* b) {
    if (!b) return MDSX_EINVAL;
    Guard guard(b->device);
    b->results_known = false;
    return ensure_results(b);
}

// One evaluation of every instance left on the device (no synchronisation):
// *d_sums receives [count][4] doubles (sum r^2, sum log Phi, getSumOfIncrements(),
// unused) and d_gradients the concatenated N_k*P_k gradients, when non-NULL.
int mdsx_batch_evaluate_device(mdsx_batch* b, double* d_sums, double* d_gradients) {
    if (!b) return MDSX_EINVAL;
    Guard guard(b->device);
    int rc = enqueue_evaluation(b);
    if (rc) return rc;
    if (d_sums)
        BCUDA(b, cudaMemcpyAsync(d_sums, b->d_sums_all, b->inst.size() * 4 * sizeof(double),
                                 cudaMemcpyDeviceToDevice, b->stream));
    if (d_gradients)
        BCUDA(b, cudaMemcpyAsync(d_gradients, b->d_grad_all, (size_t)b->grad_total * sizeof(double),
                                 cudaMemcpyDeviceToDevice, b->stream));
    b->results_known = false;
    return MDSX_OK;
}

int mdsx_batch_get_sum_of_increments(mdsx_batch* b, int k, double* out) {
    if (!b) return MDSX_EINVAL;
    int rc = check_instance(b, k);
    if (rc) return rc;
    if (!out) return bfail(b, MDSX_EINVAL, "out is NULL");
    Guard guard(b->device);
    if ((rc = ensure_results(b))) return rc;
    *out = b->h_results[4 * (size_t)k + 2];
    return MDSX_OK;
}

// R/mds.R:24-28: 0.5 (log tau - log 2 pi) N (N - 1) / 2 - getSumOfIncrements().
int mdsx_batch_get_log_likelihood(mdsx_batch* b, int k, double* out) {
    double s = 0.0;
    int rc = mdsx_batch_get_sum_of_increments(b, k, &s);
    if (rc) return rc;
    const BatchInst& in = b->inst[k];
    *out = 0.5 * (std::log(in.tau) - std::log(2.0 * M_PI)) * ((double)in.n * (in.n - 1) / 2.0) - s;
    return MDSX_OK;
}

int mdsx_batch_get_log_likelihood_gradient(mdsx_batch* b, int k, double* out, size_t length) {
    if (!b) return MDSX_EINVAL;
    int rc = check_instance(b, k);
    if (rc) return rc;
    const BatchInst& in = b->inst[k];
    if (!out || length != (size_t)in.n * in.p) return bfail(b, MDSX_EINVAL, "gradient buffer must hold N*P values");
    Guard guard(b->device);
    if ((rc = ensure_results(b))) return rc;
    std::memcpy(out, b->h_results + 4 * b->inst.size() + in.grad_off, length * sizeof(double));
    return MDSX_OK;
}

// Shape chosen for the group of embedding dimension p: rows per warp, CTAs per SM, grid.
int mdsx_batch_group_shape(mdsx_batch* b, int p, int* schedule, int* rows_per_warp, int* ctas_per_sm, int* grid) {
    if (!b) return MDSX_EINVAL;
    Guard guard(b->device);
    if (!b->planned) {
        int rc = plan(b, b->forced.empty() ? nullptr : &b->forced);
        if (rc) return rc;
    }
    for (const auto& g : b->groups)
        if (g.p == p) {
            if (schedule) *schedule = g.schedule;
            if (rows_per_warp) *rows_per_warp = g.rw;
            if (ctas_per_sm) *ctas_per_sm = g.ctas_per_sm;
            if (grid) *grid = g.grid;
            return MDSX_OK;
        }
    return bfail(b, MDSX_EINVAL, "no instance of that embedding dimension");
}

}  // extern "C"

namespace {

// Mean device time (microseconds) of one group's launch over `reps` launches.
int time_group(mdsx_batch* b, const BatchGroup& g, int reps, double* us) {
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    BCUDA(b, cudaEventCreate(&e0));
    BCUDA(b, cudaEventCreate(&e1));
    int rc = MDSX_OK;
    for (int w = 0; w < 2 && !rc; ++w) rc = launch_group(b, g, b->stream);
    if (!rc && cudaEventRecord(e0, b->stream) != cudaSuccess) rc = bfail(b, MDSX_ECUDA, "event record");
    for (int r = 0; r < reps && !rc; ++r) rc = launch_group(b, g, b->stream);
    float ms = 0.f;
    if (!rc && (cudaEventRecord(e1, b->stream) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess))
        rc = bfail(b, MDSX_ECUDA, "timing events failed");
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    int err = 0;
    BCUDA(b, cudaMemcpy(&err, b->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (err) return bfail(b, MDSX_ETIMEOUT, "a bounded device wait timed out while tuning");
    *us = 1e3 * ms / reps;
    return MDSX_OK;
}

}  // namespace

extern "C" {

// Test and tuning hook: fixes the shape of the group of embedding dimension p:
// schedule (0 stream-K, 1 row-block queue, 2 unordered pairs with rows per warp 4,
// P <= 6), rows per warp, CTAs per SM; rows_per_warp 0 removes the override.
int mdsx_batch_force_shape(mdsx_batch* b, int p, int schedule, int rows_per_warp, int ctas_per_sm) {
    if (!b) return MDSX_EINVAL;
    const std::pair<int, int> key{p, b->trunc ? 1 : 0};
    if (rows_per_warp == 0) {
        b->forced.erase(key);
    } else {
        if (!mdsx::batch::shape_built(p, schedule, rows_per_warp) || ctas_per_sm < 1 || ctas_per_sm > 4)
            return bfail(b, MDSX_EINVAL,
                         "schedule not 0, 1 or 2, rows per warp not built for this dimension and schedule, or CTAs per "
                         "SM outside 1..4");
        b->forced[key] = Shape{schedule, rows_per_warp, ctas_per_sm};
    }
    free_plan(b);
    b->results_known = false;
    return MDSX_OK;
}

// Autotuner: times every built (schedule, rows per warp, CTAs per SM)
// candidate of each group on this batch (`repetitions` launches each, after two warm-ups) and
// caches the fastest per (P, N-bucket, truncation); later plans of any batch
// in this process (and in others, through MDSX_TUNE_CACHE) use it. Writes the
// number of candidates timed to *candidates when non-NULL.
int mdsx_batch_tune(mdsx_batch* b, int repetitions, int* candidates) {
    if (!b) return MDSX_EINVAL;
    if (repetitions < 1) return bfail(b, MDSX_EINVAL, "repetitions must be >= 1");
    Guard guard(b->device);
    int rc = plan(b);
    if (rc) return rc;
    if ((rc = flush_uploads(b))) return rc;  // time on the current locations
    struct Key {
        int p, trunc, bucket;
    };
    std::vector<Key> keys;
    for (const auto& g : b->groups) {
        double mean_n = 0.0;
        for (int k : g.members) mean_n += b->inst[k].n;
        keys.push_back({g.p, g.trunc ? 1 : 0, mdsx::batch::n_bucket(mean_n / g.members.size())});
    }
    int timed = 0;
    std::map<std::pair<int, int>, Shape> best_shape;
    std::map<std::pair<int, int>, double> best_us;
    for (int sched : {0, 1, 2})
        for (int rw : {1, 2, 4})
            for (int ctas : {1, 2}) {
                std::map<std::pair<int, int>, Shape> force;
                bool any = false;
                for (const auto& k : keys)
                    if (mdsx::batch::shape_built(k.p, sched, rw)) {
                        int occ = 0;
                        size_t local = 0;
                        const cudaError_t ce = sched == 0   ? mdsx::batch::occupancy(k.p, k.trunc != 0, rw, &occ, &local)
                                               : sched == 1 ? mdsx::batch::occupancy_queue(k.p, k.trunc != 0, rw, &occ)
                                                            : mdsx::batch::occupancy_pairs(k.p, k.trunc != 0, &occ);
                        if (ce != cudaSuccess || occ < ctas) continue;
                        force[{k.p, k.trunc}] = Shape{sched, rw, ctas};
                        any = true;
                    }
                if (!any) continue;
                if ((rc = plan(b, &force))) return rc;
                if ((rc = upload_descriptors(b))) return rc;
                for (const auto& g : b->groups) {
                    const std::pair<int, int> key{g.p, g.trunc ? 1 : 0};
                    if (!force.count(key) || g.schedule != sched || g.rw != rw || g.ctas_per_sm != ctas) continue;
                    double us = 0.0;
                    if ((rc = time_group(b, g, repetitions, &us))) return rc;
                    ++timed;
                    if (!best_us.count(key) || us < best_us[key]) {
                        best_us[key] = us;
                        best_shape[key] = Shape{sched, rw, ctas};
                    }
                }
            }
    {
        std::lock_guard<std::mutex> lock(mdsx::batch::g_tune_mu);
        mdsx::batch::load_cache_locked();
        for (const auto& k : keys) {
            const std::pair<int, int> key{k.p, k.trunc};
            if (!best_shape.count(key)) continue;
            const Shape& w = best_shape[key];
            mdsx::batch::g_tune[{k.p, k.bucket, k.trunc}] = {w.schedule, w.rw, w.ctas, best_us[key]};
        }
        mdsx::batch::save_cache_locked();
    }
    if (candidates) *candidates = timed;
    free_plan(b);  // the next evaluation plans with the tuned shapes
    b->results_known = false;
    return MDSX_OK;
}

}  // extern "C"
