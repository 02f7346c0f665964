// host_pool.h -- a fixed pool of host threads for the set-up and transfer
// loops (FP64 -> FP32 rounding of model arrays, FP32 -> FP64 widening of
// results, model scans).  A large FP32 transfer runs one such loop per
// 32 MiB chunk, a 352^3 model about two hundred of them; creating and
// joining fifteen threads for each cost about as much as the loop itself.
// The workers start on first use and live as long as the process (the pool
// is never destroyed, so nothing joins them at exit).  A process forked
// after they started has none of them, so a call from a different process
// than the creator's runs its ranges on fresh threads.
#pragma once
#include <unistd.h>

#include <algorithm>
#include <condition_variable>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace seidart_host {

class HostPool {
  public:
    static HostPool& get() {
        static HostPool* pool = new HostPool;
        return *pool;
    }
    // threads a call may use (workers + the caller)
    int size() const { return (int)workers_.size() + 1; }
    // f(w) for w in [0, n): w = 0 (and any w beyond the workers) on the
    // caller, the rest on the workers; returns when all are done.  Calls
    // from several threads take turns; a call made from inside a range (a
    // nested loop) runs all its ranges on the calling thread.
    void run(int n, const std::function<void(int)>& f) {
        if (n <= 1 || in_range()) {
            for (int w = 0; w < n; ++w) f(w);
            return;
        }
        if (getpid() != pid_) {  // forked child: the workers live in the parent only
            std::vector<std::thread> t;
            for (int w = 1; w < n; ++w) t.emplace_back([&f, w] { f(w); });
            f(0);
            for (auto& x : t) x.join();
            return;
        }
        std::lock_guard<std::mutex> turn(run_mu_);
        const int nw = std::min(n, size());
        {
            std::lock_guard<std::mutex> l(mu_);
            job_ = &f;
            njob_ = nw;
            pending_ = nw - 1;
            ++gen_;
        }
        cv_.notify_all();
        {
            RangeFlag inside;
            f(0);
            for (int w = nw; w < n; ++w) f(w);
        }
        std::unique_lock<std::mutex> l(mu_);
        done_cv_.wait(l, [&] { return pending_ == 0; });
        job_ = nullptr;
    }

  private:
    // set on a thread while it runs a range
    static bool& in_range() {
        static thread_local bool flag = false;
        return flag;
    }
    struct RangeFlag {
        RangeFlag() { in_range() = true; }
        ~RangeFlag() { in_range() = false; }
    };
    HostPool() : pid_(getpid()) {
        const unsigned hw = std::thread::hardware_concurrency();
        const int n = (int)std::max(1u, std::min(hw, 16u));
        for (int w = 1; w < n; ++w) workers_.emplace_back([this, w] { loop(w); });
    }
    void loop(int w) {
        unsigned seen = 0;
        for (;;) {
            const std::function<void(int)>* f = nullptr;
            {
                std::unique_lock<std::mutex> l(mu_);
                cv_.wait(l, [&] { return gen_ != seen; });
                seen = gen_;
                if (w >= njob_) continue;
                f = job_;
            }
            {
                RangeFlag inside;
                (*f)(w);
            }
            std::lock_guard<std::mutex> l(mu_);
            if (--pending_ == 0) done_cv_.notify_one();
        }
    }

    const pid_t pid_;
    std::vector<std::thread> workers_;
    std::mutex run_mu_, mu_;
    std::condition_variable cv_, done_cv_;
    const std::function<void(int)>* job_ = nullptr;
    int njob_ = 0, pending_ = 0;
    unsigned gen_ = 0;
};

// body(lo, hi) over [0, m) in contiguous ranges, on up to 16 host threads
// (one range per 256 Ki elements at least)
template <typename F>
void host_parallel(size_t m, F body) {
    HostPool& pool = HostPool::get();
    const size_t nth = std::max<size_t>(1, std::min<size_t>((size_t)pool.size(), m >> 18));
    if (nth <= 1) {
        body(0, m);
        return;
    }
    pool.run((int)nth, [&](int w) { body(m * w / nth, m * (w + 1) / nth); });
}

}  // namespace seidart_host
