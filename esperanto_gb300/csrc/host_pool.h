// host_pool.h -- persistent host worker threads for the batch entry points'
// input scans.  Starting a thread costs tens of microseconds on the host,
// as much as scanning a 64K-pair batch; the pool's workers are started once
// per handle and woken per call.
#pragma once

#include <condition_variable>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

class HostPool {
public:
    explicit HostPool(unsigned workers) {
        for (unsigned i = 0; i < workers; i++) th_.emplace_back([this, i] { loop(i + 1); });
    }
    ~HostPool() {
        {
            std::lock_guard<std::mutex> g(mu_);
            stop_ = true;
        }
        cv_.notify_all();
        for (auto &t : th_) t.join();
    }
    HostPool(const HostPool &) = delete;
    HostPool &operator=(const HostPool &) = delete;

    // Threads a call can use: the caller plus the workers.
    unsigned size() const { return (unsigned)th_.size() + 1; }

    // fn(t) for t in [0, T): the caller runs t = 0, workers 1..T-1; returns
    // when all have finished.  One run at a time (a handle serves one host
    // thread at a time).
    void run(unsigned T, const std::function<void(unsigned)> &fn) {
        if (T > size()) T = size();
        if (T <= 1) {
            fn(0);
            return;
        }
        {
            std::lock_guard<std::mutex> g(mu_);
            job_ = &fn;
            T_ = T;
            pending_ = T - 1;
            gen_++;
        }
        cv_.notify_all();
        fn(0);
        std::unique_lock<std::mutex> g(mu_);
        done_.wait(g, [this] { return pending_ == 0; });
        job_ = nullptr;
    }

private:
    void loop(unsigned id) {
        unsigned seen = 0;
        for (;;) {
            const std::function<void(unsigned)> *job;
            {
                std::unique_lock<std::mutex> g(mu_);
                cv_.wait(g, [&] { return stop_ || gen_ != seen; });
                if (stop_) return;
                seen = gen_;
                if (id >= T_) continue;  // not needed for this run
                job = job_;
            }
            (*job)(id);
            {
                std::lock_guard<std::mutex> g(mu_);
                if (--pending_ == 0) done_.notify_one();
            }
        }
    }

    std::vector<std::thread> th_;
    std::mutex mu_;
    std::condition_variable cv_, done_;
    const std::function<void(unsigned)> *job_ = nullptr;
    unsigned T_ = 0, gen_ = 0, pending_ = 0;
    bool stop_ = false;
};
