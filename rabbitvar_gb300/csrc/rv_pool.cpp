// Host worker pool (see rv_pool.h).
#include "rv_pool.h"

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <exception>
#include <mutex>
#include <thread>
#include <vector>

namespace rv {

namespace {

thread_local bool t_in_section = false;

class Pool {
  public:
    Pool() {
        // leaves two cores to the threads outside the pool (the caller's other
        // host work, a record-formatting thread, the CUDA runtime's threads):
        // an oversubscribed core would stall a whole parallel section
        unsigned hw = std::thread::hardware_concurrency();
        int n = (int)std::min(hw ? hw : 1u, 32u) - 3;
        if (n < 0) n = 0;
        for (int i = 0; i < n; i++) workers_.emplace_back([this] { loop(); });
    }
    int threads() const { return (int)workers_.size() + 1; }

    void run(int64_t n, const std::function<void(int64_t)> &fn) {
        if (n <= 0) return;
        if (t_in_section || n == 1 || workers_.empty()) {
            for (int64_t i = 0; i < n; i++) fn(i);
            return;
        }
        std::lock_guard<std::mutex> one(run_mu_);  // one section at a time
        {
            std::lock_guard<std::mutex> lk(mu_);
            job_ = &fn;
            n_ = n;
            next_.store(0);
            busy_ = (int)workers_.size();
            error_ = nullptr;
            gen_++;
        }
        cv_work_.notify_all();
        work();
        std::unique_lock<std::mutex> lk(mu_);
        cv_done_.wait(lk, [this] { return busy_ == 0; });
        job_ = nullptr;
        if (error_) {
            std::exception_ptr e = error_;
            error_ = nullptr;
            std::rethrow_exception(e);
        }
    }

  private:
    void work() {
        t_in_section = true;
        for (int64_t i; (i = next_.fetch_add(1)) < n_;) {
            try {
                (*job_)(i);
            } catch (...) {
                std::lock_guard<std::mutex> lk(mu_);
                if (!error_) error_ = std::current_exception();
            }
        }
        t_in_section = false;
    }
    void loop() {
        uint64_t seen = 0;
        for (;;) {
            {
                std::unique_lock<std::mutex> lk(mu_);
                cv_work_.wait(lk, [&] { return gen_ != seen; });
                seen = gen_;
            }
            work();
            std::lock_guard<std::mutex> lk(mu_);
            if (--busy_ == 0) cv_done_.notify_all();
        }
    }

    std::vector<std::thread> workers_;
    std::mutex mu_, run_mu_;
    std::condition_variable cv_work_, cv_done_;
    const std::function<void(int64_t)> *job_ = nullptr;
    int64_t n_ = 0;
    std::atomic<int64_t> next_{0};
    uint64_t gen_ = 0;
    int busy_ = 0;
    std::exception_ptr error_;
};

// never destroyed: the workers stay parked on their condition variable until
// the process exits
Pool &pool() {
    static Pool *p = new Pool();
    return *p;
}

}  // namespace

void parallel_for(int64_t n, const std::function<void(int64_t)> &fn) { pool().run(n, fn); }

int pool_threads() { return pool().threads(); }

int64_t parallel_chunks(int64_t n, int64_t min_per_chunk, const std::function<void(int64_t, int64_t, int64_t)> &fn) {
    const int64_t c = chunks_for(n, min_per_chunk);
    const int64_t per = (n + c - 1) / c;
    parallel_for(c, [&](int64_t k) {
        int64_t a = std::min(n, k * per), b = std::min(n, (k + 1) * per);
        fn(k, a, b);
    });
    return c;
}

}  // namespace rv
