// Host-side plan of the unordered-pair schedule (pair_kernel.cuh), shared by the
// single-instance engine (one instance) and the batch (the instances of one
// dimension group): the units of every instance concatenated in order, split
// into contiguous CTA ranges of equal modelled cost, and per instance the slot
// tables the kernels and the finish use.
#pragma once

#include <algorithm>
#include <vector>

#include "pair_kernel.cuh"

namespace mdsx {

struct PairInstancePlan {
    int nb = 0, nc = 0;          // column blocks, row chunks
    long long units = 0;         // units of the instance
    long long unit_begin = 0;    // first global unit
    int first_cta = 0;           // first CTA whose range meets the instance
    int ctas = 0;                // CTAs whose ranges meet the instance
    int max_slots = 1;           // most CTAs meeting one column block
    std::vector<int> j_first;    // [nb] first CTA meeting column block J (absolute)
    std::vector<int> j_slots;    // [nb] CTAs meeting column block J
};

struct PairPlan {
    int grid = 0;
    long long units = 0;
    std::vector<long long> cta_begin;  // [grid + 1]
    std::vector<PairInstancePlan> inst;
};

// Plans instances of sizes ns over at most max_grid CTAs. CTA c starts at the
// first unit whose cumulative modelled cost (pair_unit_cost) reaches c / G of
// the total; every range keeps at least one unit (G <= total units).
inline PairPlan pair_plan(const std::vector<int>& ns, long long max_grid) {
    PairPlan plan;
    double total = 0.0;
    for (int n : ns) {
        PairInstancePlan q;
        q.nb = (n + kPairCols - 1) / kPairCols;
        q.nc = (n + kPairRows - 1) / kPairRows;
        q.units = pair_units_before(q.nb, q.nc);
        q.unit_begin = plan.units;
        plan.units += q.units;
        for (int J = 0; J < q.nb; ++J)
            for (int I = 4 * J; I < q.nc; ++I) total += pair_unit_cost(I, J);
        plan.inst.push_back(std::move(q));
    }
    const long long U = plan.units;
    const int G = (int)std::max<long long>(1, std::min<long long>(U, max_grid));
    plan.grid = G;
    std::vector<long long>& begin = plan.cta_begin;
    begin.assign(G + 1, 0);
    {
        int c = 1;
        double cum = 0.0;
        long long u = 0;
        for (size_t m = 0; m < plan.inst.size() && c < G; ++m)
            for (int J = 0; J < plan.inst[m].nb && c < G; ++J)
                for (int I = 4 * J; I < plan.inst[m].nc && c < G; ++I, ++u) {
                    while (c < G && cum >= total * c / G) begin[c++] = u;
                    cum += pair_unit_cost(I, J);
                }
        while (c < G) begin[c++] = U;
        begin[G] = U;
        // strictly increasing with room for the ranges after each
        for (int k = 1; k < G; ++k) begin[k] = std::min(std::max(begin[k], begin[k - 1] + 1), U - (G - k));
    }
    auto cta_of = [&](long long u) {  // CTA whose range holds global unit u
        return (int)(std::upper_bound(begin.begin(), begin.end(), u) - begin.begin()) - 1;
    };
    for (auto& q : plan.inst) {
        q.j_first.resize(q.nb);
        q.j_slots.resize(q.nb);
        q.max_slots = 1;
        for (int J = 0; J < q.nb; ++J) {
            const long long u0 = q.unit_begin + pair_units_before(J, q.nc);
            const long long u1 = u0 + (q.nc - 4 * J) - 1;
            q.j_first[J] = cta_of(u0);
            q.j_slots[J] = cta_of(u1) - q.j_first[J] + 1;
            q.max_slots = std::max(q.max_slots, q.j_slots[J]);
        }
        q.first_cta = cta_of(q.unit_begin);
        q.ctas = cta_of(q.unit_begin + q.units - 1) - q.first_cta + 1;
    }
    return plan;
}

}  // namespace mdsx
