// Test scaffolding, not product code.
//
// Minimal stand-ins for the four Intel TBB headers that the MassiveMDS CPU
// engine includes unconditionally (USE_TBB is forced on in
// src/AbstractMultiDimensionalScaling.hpp:23). Real TBB is not installed on
// either build machine, so these shims let the reference's own serial engine
// (NewMultiDimensionalScaling<...NoSimd..., CpuAccumulate>) compile from its
// sources for use as the oracle. The TbbAccumulate instantiations also compile
// and run: parallel_reduce / parallel_for below split the range into one
// contiguous chunk per worker on std::thread and combine the chunk results in
// chunk order. That is "the reference TBB code path on a std::thread shim",
// not Intel TBB's work-stealing scheduler.
#ifndef MDSX_ORACLE_TBB_SHIM_COMMON_H
#define MDSX_ORACLE_TBB_SHIM_COMMON_H

#include <algorithm>
#include <atomic>
#include <cstddef>
#include <thread>
#include <vector>

namespace tbb {

namespace detail {
inline std::atomic<std::size_t>& parallelism_limit() {
    static std::atomic<std::size_t> limit{0};  // 0 = hardware concurrency
    return limit;
}
inline std::size_t worker_count() {
    std::size_t hw = std::max<std::size_t>(1, std::thread::hardware_concurrency());
    std::size_t lim = parallelism_limit().load();
    return lim == 0 ? hw : std::max<std::size_t>(1, lim);
}
}  // namespace detail

template <typename Value>
class blocked_range {
public:
    blocked_range(Value begin, Value end, std::size_t grain = 1)
        : begin_(begin), end_(end), grain_(grain) {}
    Value begin() const { return begin_; }
    Value end() const { return end_; }
    bool empty() const { return !(begin_ < end_); }
    std::size_t size() const { return static_cast<std::size_t>(end_ - begin_); }
    std::size_t grainsize() const { return grain_; }

private:
    Value begin_, end_;
    std::size_t grain_;
};

namespace this_task_arena {
inline int max_concurrency() { return static_cast<int>(detail::worker_count()); }
}  // namespace this_task_arena

class global_control {
public:
    enum parameter { max_allowed_parallelism, thread_stack_size };
    global_control(parameter p, std::size_t value) : p_(p), previous_(detail::parallelism_limit().load()) {
        if (p_ == max_allowed_parallelism) detail::parallelism_limit().store(value);
    }
    ~global_control() {
        if (p_ == max_allowed_parallelism) detail::parallelism_limit().store(previous_);
    }
    static std::size_t active_value(parameter p) {
        return p == max_allowed_parallelism ? detail::worker_count() : 0;
    }

private:
    parameter p_;
    std::size_t previous_;
};

namespace detail {
// Split [b, e) into at most `workers` contiguous chunks.
template <typename Value>
std::vector<blocked_range<Value>> split(const blocked_range<Value>& r, std::size_t workers) {
    std::vector<blocked_range<Value>> parts;
    const std::size_t n = r.size();
    if (n == 0) return parts;
    workers = std::min(workers, n);
    const std::size_t base = n / workers, extra = n % workers;
    Value start = r.begin();
    for (std::size_t w = 0; w < workers; ++w) {
        const std::size_t len = base + (w < extra ? 1 : 0);
        Value stop = start + static_cast<Value>(len);
        parts.emplace_back(start, stop, r.grainsize());
        start = stop;
    }
    return parts;
}
}  // namespace detail

template <typename Range, typename Value, typename Body, typename Reduction>
Value parallel_reduce(const Range& range, const Value& identity, const Body& body,
                      const Reduction& reduction) {
    auto parts = detail::split(range, detail::worker_count());
    if (parts.size() <= 1) return parts.empty() ? identity : body(parts[0], identity);
    std::vector<Value> partial(parts.size(), identity);
    std::vector<std::thread> threads;
    for (std::size_t w = 1; w < parts.size(); ++w)
        threads.emplace_back([&, w] { partial[w] = body(parts[w], identity); });
    partial[0] = body(parts[0], identity);
    for (auto& t : threads) t.join();
    Value total = partial[0];
    for (std::size_t w = 1; w < parts.size(); ++w) total = reduction(total, partial[w]);
    return total;
}

template <typename Range, typename Body>
void parallel_for(const Range& range, const Body& body) {
    auto parts = detail::split(range, detail::worker_count());
    if (parts.size() <= 1) {
        if (!parts.empty()) body(parts[0]);
        return;
    }
    std::vector<std::thread> threads;
    for (std::size_t w = 1; w < parts.size(); ++w) threads.emplace_back([&, w] { body(parts[w]); });
    body(parts[0]);
    for (auto& t : threads) t.join();
}

}  // namespace tbb

#endif  // MDSX_ORACLE_TBB_SHIM_COMMON_H
