// Minimal stand-in for the parts of oneTBB that the reference permanent
// calculators use, so that their sources compile and run without TBB.
// Oracle-only test infrastructure: it never ships in the product library.
//
// parallel_for runs its body on std::thread workers at the outermost level
// (work items are handed out through an atomic counter) and serially when
// called from inside a worker, so the reference's nested task trees do not
// oversubscribe.  combinable<T> keeps one slot per OS thread.
#pragma once
#include <atomic>
#include <cstdint>
#include <cstdlib>
#include <functional>
#include <map>
#include <mutex>
#include <thread>
#include <vector>
#include "scalable_allocator.h"
#include "spin_mutex.h"
#include "cache_aligned_allocator.h"
#include "concurrent_vector.h"

namespace tbb {

namespace shim {
inline int& depth() { thread_local int d = 0; return d; }
inline unsigned workers() {
    const char* env = std::getenv("PQB_REF_THREADS");
    if (env && std::atoi(env) > 0) return (unsigned)std::atoi(env);
    unsigned h = std::thread::hardware_concurrency();
    return h ? h : 1;
}
// Run job(i) for i in [0, count) on the worker pool (or inline when nested).
inline void run_items(int64_t count, const std::function<void(int64_t)>& job) {
    if (count <= 0) return;
    unsigned nw = workers();
    if (depth() > 0 || nw <= 1 || count == 1) {
        ++depth();
        for (int64_t i = 0; i < count; ++i) job(i);
        --depth();
        return;
    }
    std::atomic<int64_t> next{0};
    auto worker = [&]() {
        ++depth();
        for (;;) {
            int64_t i = next.fetch_add(1);
            if (i >= count) break;
            job(i);
        }
        --depth();
    };
    unsigned nt = (unsigned)std::min<int64_t>(nw, count);
    std::vector<std::thread> pool;
    for (unsigned t = 1; t < nt; ++t) pool.emplace_back(worker);
    worker();
    for (auto& th : pool) th.join();
}
}  // namespace shim

template <typename T>
class blocked_range {
public:
    blocked_range(T b, T e, size_t grain = 1) : b_(b), e_(e) { (void)grain; }
    T begin() const { return b_; }
    T end() const { return e_; }
    bool empty() const { return !(b_ < e_); }
    size_t size() const { return (size_t)(e_ - b_); }
private:
    T b_, e_;
};

template <typename Index, typename Func>
void parallel_for(Index first, Index last, Index step, const Func& f) {
    if (step <= 0 || !(first < last)) return;
    int64_t count = (int64_t)((last - first + step - 1) / step);
    shim::run_items(count, [&](int64_t i) { f((Index)(first + (Index)i * step)); });
}

template <typename Index, typename Func>
void parallel_for(Index first, Index last, const Func& f) {
    parallel_for(first, last, (Index)1, f);
}

template <typename T, typename Func>
void parallel_for(const blocked_range<T>& r, const Func& f) {
    if (r.empty()) return;
    // one sub-range per element at the outermost level
    int64_t count = (int64_t)(r.end() - r.begin());
    shim::run_items(count, [&](int64_t i) {
        T b = (T)(r.begin() + (T)i);
        f(blocked_range<T>(b, (T)(b + 1)));
    });
}

template <typename T>
class combinable {
public:
    combinable() : init_([]() { return T(); }) {}
    template <typename F>
    explicit combinable(F f) : init_(f) {}
    combinable(const combinable& o) : init_(o.init_) {}
    combinable& operator=(const combinable& o) {
        std::lock_guard<std::mutex> g(m_);
        init_ = o.init_;
        slots_.clear();
        return *this;
    }
    T& local() {
        std::lock_guard<std::mutex> g(m_);
        auto id = std::this_thread::get_id();
        auto it = slots_.find(id);
        if (it == slots_.end()) it = slots_.emplace(id, init_()).first;
        return it->second;
    }
    template <typename F>
    void combine_each(F f) {
        std::lock_guard<std::mutex> g(m_);
        for (auto& kv : slots_) f(kv.second);
    }
    void clear() { std::lock_guard<std::mutex> g(m_); slots_.clear(); }
private:
    std::function<T()> init_;
    std::map<std::thread::id, T> slots_;  // node-based: references stay valid
    std::mutex m_;
};

class task_group {
public:
    template <typename F> void run(const F& f) { f(); }
    void wait() {}
};

class tick_count {
public:
    static tick_count now() { return tick_count(); }
    struct interval_t { double seconds() const { return 0.0; } };
    interval_t operator-(const tick_count&) const { return interval_t(); }
};

inline void parallel_invoke() {}
template <typename F, typename... R>
void parallel_invoke(const F& f, const R&... r) { f(); parallel_invoke(r...); }

}  // namespace tbb
