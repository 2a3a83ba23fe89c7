// Worker pool behind symgb::parallelFor (include/symgb/parallel.hpp).
#include "symgb/parallel.hpp"

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstdlib>
#include <mutex>
#include <thread>
#include <vector>

namespace symgb {

namespace {

thread_local bool t_inWorker = false;

class Pool {
public:
    explicit Pool(int threads) {
        for (int i = 1; i < threads; ++i) workers_.emplace_back([this] { loop(); });
    }
    ~Pool() {
        {
            std::lock_guard<std::mutex> g(m_);
            stop_ = true;
        }
        cv_.notify_all();
        for (auto& t : workers_) t.join();
    }
    int size() const { return (int)workers_.size() + 1; }

    void run(std::size_t n, std::size_t chunk, const std::function<void(std::size_t, std::size_t)>& fn) {
        std::lock_guard<std::mutex> serial(runMutex_);  // one loop at a time
        {
            std::lock_guard<std::mutex> g(m_);
            fn_ = &fn;
            n_ = n;
            chunk_ = chunk;
            next_.store(0);
            pending_ = workers_.size();
            ++generation_;
        }
        cv_.notify_all();
        work();
        std::unique_lock<std::mutex> g(m_);
        done_.wait(g, [this] { return pending_ == 0; });
        fn_ = nullptr;
    }

private:
    void work() {
        for (;;) {
            const std::size_t b = next_.fetch_add(chunk_);
            if (b >= n_) return;
            (*fn_)(b, std::min(n_, b + chunk_));
        }
    }
    void loop() {
        t_inWorker = true;
        std::size_t seen = 0;
        for (;;) {
            {
                std::unique_lock<std::mutex> g(m_);
                cv_.wait(g, [&] { return stop_ || generation_ != seen; });
                if (stop_) return;
                seen = generation_;
            }
            work();
            std::lock_guard<std::mutex> g(m_);
            if (--pending_ == 0) done_.notify_one();
        }
    }

    std::vector<std::thread> workers_;
    std::mutex m_, runMutex_;
    std::condition_variable cv_, done_;
    const std::function<void(std::size_t, std::size_t)>* fn_ = nullptr;
    std::size_t n_ = 0, chunk_ = 1, pending_ = 0, generation_ = 0;
    std::atomic<std::size_t> next_{0};
    bool stop_ = false;
};

int configuredThreads() {
    if (const char* e = std::getenv("SYMGB_THREADS")) {
        const int v = std::atoi(e);
        if (v >= 1) return std::min(v, 256);
    }
    const unsigned h = std::thread::hardware_concurrency();
    return h ? (int)std::min(h, 256u) : 1;
}

Pool& pool() {
    static Pool p(configuredThreads());
    return p;
}

}  // namespace

int frontEndThreads() { return pool().size(); }

void parallelFor(std::size_t n, std::size_t grain, const std::function<void(std::size_t, std::size_t)>& fn) {
    if (n == 0) return;
    grain = std::max<std::size_t>(grain, 1);
    if (t_inWorker || n < 2 * grain || pool().size() == 1) {
        fn(0, n);
        return;
    }
    // Many small chunks, taken dynamically: per-item costs are uneven (the
    // output blocks of a decomposition, which come last, cost the most), and a
    // few large chunks left one thread with most of the work.
    const std::size_t chunks = std::min<std::size_t>((std::size_t)pool().size() * 64, (n + grain - 1) / grain);
    pool().run(n, (n + chunks - 1) / chunks, fn);
}

}  // namespace symgb
