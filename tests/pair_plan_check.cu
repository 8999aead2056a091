// Host-only check of the unordered-pair plan (massivemds_gb300/csrc/pair_plan.h),
// built and run by tests/test_pair_plan.py on the CPU. For random instance lists
// and grids it walks every CTA's range the way pair_kernel / batch_pair_kernel
// do (instance cursor, column block J, row chunk I) and checks:
//   - the CTA ranges are non-empty, increasing and cover all units;
//   - the producer's unit order equals the consumers' (J, I) walk;
//   - every column-block slot and likelihood slot a CTA writes lies in its table,
//     and every slot the finish kernel reads was written;
//   - every unordered pair i > j of every instance is covered exactly once
//     (instances up to 700 locations);
//   - the finish kernel's blocks (pair_finish_block, every FinishShape: P = 1..6,
//     FP32 and FP64 partials) read only inside the row- and column-partial
//     buffers as the engine sizes them, read every row partial and every column
//     partial of a real column once, and write every gradient entry once.
// Prints "ok" and exits 0, or prints the first failure and exits 1.
#include <cstdio>
#include <cstdlib>
#include <random>
#include <set>
#include <utility>
#include <vector>

#include "pair_plan.h"

using mdsx::kPairCols;
using mdsx::kPairRows;
using mdsx::pair_block_of_unit;
using mdsx::pair_units_before;

#define CHECK(cond, ...)                          \
    do {                                          \
        if (!(cond)) {                            \
            std::printf("FAILED %s: ", #cond);    \
            std::printf(__VA_ARGS__);             \
            std::printf("\n");                    \
            std::exit(1);                         \
        }                                         \
    } while (0)

static void check(const std::vector<int>& ns, long long max_grid) {
    const mdsx::PairPlan plan = mdsx::pair_plan(ns, max_grid);
    const int G = plan.grid;
    CHECK(G >= 1 && G <= max_grid && (long long)G <= plan.units, "grid %d", G);
    CHECK(plan.cta_begin[0] == 0 && plan.cta_begin[G] == plan.units, "range ends");
    for (int c = 0; c < G; ++c) CHECK(plan.cta_begin[c + 1] > plan.cta_begin[c], "empty range %d", c);

    std::vector<std::set<std::pair<int, int>>> col_written(ns.size());
    std::vector<std::set<int>> lik_written(ns.size());
    std::vector<std::vector<unsigned char>> cover(ns.size());
    for (size_t m = 0; m < ns.size(); ++m)
        if (ns[m] <= 700) cover[m].assign((size_t)ns[m] * ns[m], 0);

    for (int c = 0; c < G; ++c) {
        const long long ub = plan.cta_begin[c], ue = plan.cta_begin[c + 1];
        const int K = (int)(ue - ub);
        // producer walk
        size_t pk = 0;
        while (pk + 1 < plan.inst.size() && plan.inst[pk + 1].unit_begin <= ub) ++pk;
        std::vector<std::pair<size_t, std::pair<int, int>>> issued;
        {
            const auto* q = &plan.inst[pk];
            const long long lu = ub - q->unit_begin;
            int J = pair_block_of_unit(lu, q->nb, q->nc);
            int I = 4 * J + (int)(lu - pair_units_before(J, q->nc));
            for (int m = 0; m < K; ++m) {
                CHECK(J < q->nb && I >= 4 * J && I < q->nc, "producer unit out of range");
                issued.push_back({pk, {J, I}});
                if (++I == q->nc) {
                    ++J;
                    I = 4 * J;
                    if (J == q->nb && pk + 1 < plan.inst.size()) {
                        ++pk;
                        q = &plan.inst[pk];
                        J = I = 0;
                    }
                }
            }
        }
        // consumer walk
        size_t ik = 0;
        while (ik + 1 < plan.inst.size() && plan.inst[ik + 1].unit_begin <= ub) ++ik;
        int k = 0;
        for (; k < K; ++ik) {
            const auto& q = plan.inst[ik];
            const long long in_end = q.unit_begin + q.units;
            const int k_inst_end = (int)(std::min(ue, in_end) - ub);
            const long long lu0 = ub + k - q.unit_begin;
            for (int J = pair_block_of_unit(lu0, q.nb, q.nc); k < k_inst_end; ++J) {
                const long long before = pair_units_before(J, q.nc);
                const long long j_end = q.unit_begin + before + (q.nc - 4 * J);
                const int k_end = (int)(std::min(ue, j_end) - ub);
                const int slot = c - q.j_first[J];
                CHECK(slot >= 0 && slot < q.j_slots[J] && q.j_slots[J] <= q.max_slots, "slot %d J %d", slot, J);
                col_written[ik].insert({J, slot});
                int I = 4 * J + (int)(ub + k - q.unit_begin - before);
                for (; k < k_end; ++k, ++I) {
                    CHECK(issued[k].first == ik && issued[k].second == std::make_pair(J, I), "order at unit %d", k);
                    if (!cover[ik].empty()) {
                        const int n = ns[ik];
                        for (int i = I * kPairRows; i < I * kPairRows + kPairRows && i < n; ++i)
                            for (int j = J * kPairCols; j < J * kPairCols + kPairCols && j < n; ++j)
                                if (i > j) ++cover[ik][(size_t)i * n + j];
                    }
                }
            }
            const int e = c - q.first_cta;
            CHECK(e >= 0 && e < q.ctas, "likelihood slot %d", e);
            lik_written[ik].insert(e);
        }
    }
    for (size_t m = 0; m < ns.size(); ++m) {
        const auto& q = plan.inst[m];
        for (int J = 0; J < q.nb; ++J)
            for (int s = 0; s < q.j_slots[J]; ++s) CHECK(col_written[m].count({J, s}), "slot (%d, %d) unwritten", J, s);
        CHECK((int)lik_written[m].size() == q.ctas, "likelihood slots");
        if (!cover[m].empty()) {
            const int n = ns[m];
            for (int i = 0; i < n; ++i)
                for (int j = 0; j < n; ++j)
                    CHECK(cover[m][(size_t)i * n + j] == (i > j ? 1 : 0), "pair (%d, %d) covered %d times", i, j,
                          (int)cover[m][(size_t)i * n + j]);
        }
    }
}

// The finish of one sweep over an N-location instance, replaying the index
// arithmetic of pair_finish_block (pair_kernel.cuh) for every block and thread.
template <int P, typename Part>
static void check_finish(int n, long long max_grid) {
    using FS = mdsx::FinishShape<P, Part>;
    static_assert(FS::kGroups * FS::kOut <= FS::kThreads, "finish block holds its groups");
    static_assert(FS::kRows * FS::kSplit == kPairRows, "row split covers a chunk");
    const mdsx::PairPlan plan = mdsx::pair_plan({n}, max_grid);
    const mdsx::PairInstancePlan& q = plan.inst[0];
    const int nc = q.nc, nb = q.nb;
    const size_t row_size = (size_t)q.units * kPairRows * P;  // engine.cu's allocations
    const size_t col_size = (size_t)nb * q.max_slots * mdsx::kPairWarps * P * kPairCols;
    std::vector<unsigned char> row_read(row_size, 0), col_read(col_size, 0), grad_written((size_t)n * P, 0);
    const int blocks = mdsx::pair_finish_blocks<P, Part>(nc);
    CHECK(blocks == 1 + nc * FS::kSplit, "finish grid");
    for (int blk = 1; blk < blocks; ++blk) {
        const int ci = (blk - 1) / FS::kSplit;
        const int I = nc - 1 - ci;
        const int h0 = (blk - 1 - ci * FS::kSplit) * FS::kRows;
        CHECK(I >= 0 && I < nc && h0 >= 0 && h0 + FS::kRows <= kPairRows, "block %d", blk);
        for (int t = 0; t < FS::kThreads; ++t) {
            const int g = t / FS::kOut, o = t - g * FS::kOut;
            if (g < FS::kGroups) {
                const int j_max = I >> 2;
                for (int J0 = g; J0 <= j_max; J0 += FS::kGroups * FS::kChunk)
                    for (int k = 0; k < FS::kChunk; ++k) {
                        const int J = J0 + FS::kGroups * k;
                        if (J > j_max) continue;
                        const long long u = pair_units_before(J, nc) + (I - 4 * J);
                        const size_t idx = (size_t)u * (kPairRows * P) + h0 * P + o;
                        CHECK(u >= 0 && u < q.units && idx < row_size, "row partial (%d, %d) P %d", J, I, P);
                        ++row_read[idx];
                    }
                const int J = I >> 2, r = o / P, qd = o - r * P, jj = (I & 3) * kPairRows + h0 + r;
                CHECK(J < nb && jj < kPairCols, "column block %d", J);
                const int n_e = q.j_slots[J] * mdsx::kPairWarps;
                CHECK(q.j_slots[J] <= q.max_slots, "slots of %d", J);
                for (int e0 = g; e0 < n_e; e0 += FS::kGroups * FS::kColChunk)
                    for (int k = 0; k < FS::kColChunk; ++k) {
                        const int e = e0 + FS::kGroups * k;
                        if (e >= n_e) continue;
                        const size_t idx = ((size_t)J * q.max_slots * mdsx::kPairWarps + e) * (P * kPairCols) +
                                           qd * kPairCols + jj;
                        CHECK(idx < col_size, "column partial J %d e %d", J, e);
                        ++col_read[idx];
                    }
            }
            if (t < FS::kOut) {
                const int row = I * kPairRows + h0 + t / P;
                if (row < n) {
                    const size_t idx = (size_t)(I * kPairRows + h0) * P + t;
                    CHECK(idx < (size_t)n * P, "gradient index");
                    ++grad_written[idx];
                }
            }
        }
    }
    for (size_t i = 0; i < row_size; ++i) CHECK(row_read[i] == 1, "row partial %zu read %d times", i, row_read[i]);
    for (int J = 0; J < nb; ++J)
        for (int e = 0; e < q.max_slots * mdsx::kPairWarps; ++e)
            for (int qd = 0; qd < P; ++qd)
                for (int jj = 0; jj < kPairCols; ++jj) {
                    const size_t idx = ((size_t)J * q.max_slots * mdsx::kPairWarps + e) * (P * kPairCols) +
                                       qd * kPairCols + jj;
                    const bool real = e < q.j_slots[J] * mdsx::kPairWarps && J * kPairCols + jj < nc * kPairRows;
                    CHECK(col_read[idx] == (real ? 1 : 0), "column partial (J %d, e %d, q %d, col %d) read %d times", J,
                          e, qd, jj, col_read[idx]);
                }
    for (size_t i = 0; i < grad_written.size(); ++i)
        CHECK(grad_written[i] == 1, "gradient entry %zu written %d times", i, grad_written[i]);
}

template <typename Part>
static void check_finish_all(int n, long long max_grid) {
    check_finish<1, Part>(n, max_grid);
    check_finish<2, Part>(n, max_grid);
    check_finish<3, Part>(n, max_grid);
    check_finish<4, Part>(n, max_grid);
    check_finish<5, Part>(n, max_grid);
    check_finish<6, Part>(n, max_grid);
}

int main() {
    std::mt19937 rng(7);
    for (int n : {1, 2, 31, 32, 33, 127, 128, 129, 300, 641, 1000, 4099})
        for (long long g : {1LL, 17LL, 152LL, 304LL}) {
            check_finish_all<float>(n, g);
            check_finish_all<double>(n, g);
        }
    const long long grids[] = {1, 2, 5, 17, 152, 304};
    for (int n : {1, 2, 31, 32, 33, 127, 128, 129, 300, 641, 700})
        for (long long g : grids) check({n}, g);
    for (int t = 0; t < 300; ++t) {
        std::vector<int> ns(1 + rng() % 8);
        for (int& n : ns) n = 1 + (int)(rng() % 2000);
        check(ns, grids[rng() % 6]);
    }
    check({20000}, 304);
    std::vector<int> c3(64);
    for (int& n : c3) n = 500 + (int)(rng() % 7501);
    check(c3, 304);
    std::printf("ok\n");
    return 0;
}
