// serve_sched.h -- admission and batching of the serving loop (host only, no
// CUDA: the decisions are tested on the CPU by tests/serve_sched_check.cpp).
//
// Requests queue FIFO as jobs.  A launch takes reads from the head of the
// queue -- the rest of the head request, then the next requests of the same
// CIGAR stride -- up to max_batch reads, so small requests share one launch
// and a request larger than max_batch runs over several.  Every launch is
// charged the DP scratch it needs (traceback words dominate) from one shared
// pool of the memory budget: when the pool cannot hold the launch, it is cut
// to the longest prefix whose scratch fits the largest free block, and when
// not even min_batch reads fit, the head request waits until a running
// launch returns its scratch.
#pragma once

#include <algorithm>
#include <cstdint>
#include <deque>
#include <functional>
#include <map>
#include <vector>

namespace serve {

inline uint64_t al256(uint64_t x) { return (x + 255) / 256 * 256; }

// First-fit allocator of one region [0, size) in 256-byte units; freed
// blocks coalesce with free neighbours.
class ScratchPool {
  public:
    void reset(uint64_t size) {
        size_ = size / 256 * 256;
        free_.clear();
        if (size_) free_[0] = size_;
        used_ = peak_ = 0;
    }
    bool alloc(uint64_t bytes, uint64_t &off) {
        bytes = al256(std::max<uint64_t>(bytes, 1));
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < bytes) continue;
            off = it->first;
            const uint64_t rest = it->second - bytes;
            free_.erase(it);
            if (rest) free_[off + bytes] = rest;
            used_ += bytes;
            peak_ = std::max(peak_, used_);
            return true;
        }
        return false;
    }
    void release(uint64_t off, uint64_t bytes) {
        bytes = al256(std::max<uint64_t>(bytes, 1));
        used_ -= bytes;
        auto nx = free_.lower_bound(off);
        if (nx != free_.end() && off + bytes == nx->first) {  // merge the next block
            bytes += nx->second;
            nx = free_.erase(nx);
        }
        if (nx != free_.begin()) {  // merge into the previous block
            auto pv = std::prev(nx);
            if (pv->first + pv->second == off) {
                pv->second += bytes;
                return;
            }
        }
        free_[off] = bytes;
    }
    uint64_t largest_free() const {
        uint64_t m = 0;
        for (auto &kv : free_) m = std::max(m, kv.second);
        return m;
    }
    uint64_t size() const { return size_; }
    uint64_t used() const { return used_; }
    uint64_t peak() const { return peak_; }

  private:
    std::map<uint64_t, uint64_t> free_;  // offset -> length
    uint64_t size_ = 0, used_ = 0, peak_ = 0;
};

// A queued request as the scheduler sees it.
struct Job {
    uint64_t n = 0;                 // reads
    uint64_t next = 0;              // first read not yet given to a launch
    uint64_t done = 0;              // reads whose launch has completed
    uint32_t max_m = 0, max_n = 0;  // longest read and window (scratch sizing)
    uint32_t group = 0;             // only jobs of one group share a launch
    uint32_t launches = 0;          // launches its reads were given to
    bool held = false;              // waited at the head of the queue for scratch
    void *user = nullptr;
};

struct Piece {
    Job *job;
    uint64_t first, count;  // reads [first, first + count) of the job
};

struct Launch {
    std::vector<Piece> pieces;
    uint64_t n = 0;
    uint32_t max_m = 0, max_n = 0;
    uint64_t off = 0, bytes = 0;  // scratch carved from the pool
};

struct Stats {
    uint64_t launches = 0;      // launches completed
    uint64_t reads = 0;         // reads in them
    uint64_t merged = 0;        // launches holding reads of more than one request
    uint64_t split_jobs = 0;    // requests whose reads ran in more than one launch
    uint64_t budget_waits = 0;  // requests held at the head of the queue for scratch
    uint64_t cuts = 0;          // launches cut short to fit the free scratch
};

// DP scratch bytes of one launch of n reads of at most max_m x max_n bases.
using NeedFn = std::function<uint64_t(uint64_t n, uint32_t max_m, uint32_t max_n)>;

class Scheduler {
  public:
    Scheduler() = default;
    Scheduler(uint64_t pool_bytes, uint64_t max_batch, uint64_t min_batch, NeedFn need)
        : max_batch_(max_batch), min_batch_(std::min(min_batch, max_batch)), need_(std::move(need)) {
        pool_.reset(pool_bytes);
    }

    // Whether the job can ever run: its smallest launch fits the whole pool.
    bool admissible(const Job &j) const {
        return j.n == 0 || need_(std::min(j.n, min_batch_), j.max_m, j.max_n) <= pool_.size();
    }
    void push(Job *j) { q_.push_back(j); }
    bool empty() const { return q_.empty(); }
    size_t queued() const { return q_.size(); }

    // The next launch (see the file comment).  False when the queue is empty
    // or the scratch is short (the head request then counts once in
    // budget_waits, however often it is retried).
    bool next(Launch &L) {
        L = Launch{};
        if (q_.empty()) return false;
        const uint32_t group = q_.front()->group;
        uint64_t cap = max_batch_;
        for (Job *j : q_) {
            if (cap == 0 || j->group != group) break;
            const uint64_t take = std::min(j->n - j->next, cap);
            L.pieces.push_back({j, j->next, take});
            L.n += take;
            cap -= take;
        }
        shape(L);
        if (!pool_.alloc(L.bytes, L.off)) {
            // cut to the longest prefix that fits; failing that, the head
            // request's piece alone (its own scratch shape) cut the same way
            const uint64_t gathered = L.n;
            if (!fit_prefix(L)) {
                L.pieces.resize(1);
                L.n = L.pieces[0].count;
                shape(L);
                if (!fit_prefix(L)) {
                    Job *head = q_.front();
                    if (!head->held) stats_.budget_waits++;
                    head->held = true;
                    L = Launch{};
                    return false;
                }
            }
            if (L.n < gathered) stats_.cuts++;
        }
        for (const Piece &p : L.pieces) {
            p.job->next += p.count;
            p.job->launches++;
        }
        while (!q_.empty() && q_.front()->next == q_.front()->n) q_.pop_front();
        return true;
    }

    // Return a finished launch's scratch; jobs whose every read is now done
    // are appended to `completed`.
    void finish(const Launch &L, std::vector<Job *> &completed) {
        pool_.release(L.off, L.bytes);
        stats_.launches++;
        stats_.reads += L.n;
        if (L.pieces.size() > 1) stats_.merged++;
        for (const Piece &p : L.pieces) {
            p.job->done += p.count;
            if (p.job->done == p.job->n) {
                if (p.job->launches > 1) stats_.split_jobs++;
                completed.push_back(p.job);
            }
        }
    }

    // Remove the queued jobs none of whose reads was launched (closing).
    void drop_unstarted(std::vector<Job *> &dropped) {
        std::deque<Job *> keep;
        for (Job *j : q_) {
            if (j->next == 0) dropped.push_back(j);
            else keep.push_back(j);
        }
        q_.swap(keep);
    }

    const Stats &stats() const { return stats_; }
    const ScratchPool &pool() const { return pool_; }

  private:
    // Cut L to the longest prefix whose scratch fits the largest free block
    // and carve it; false when that prefix is shorter than min_batch reads
    // (or than L itself, when L is shorter).
    bool fit_prefix(Launch &L) {
        const uint64_t F = pool_.largest_free();
        uint64_t lo = 0, hi = L.n;
        while (lo < hi) {
            const uint64_t mid = lo + (hi - lo + 1) / 2;
            if (need_(mid, L.max_m, L.max_n) <= F) lo = mid;
            else hi = mid - 1;
        }
        if (lo == 0 || lo < std::min(L.n, min_batch_)) return false;
        truncate(L, lo);
        shape(L);  // a shorter prefix needs at most need(lo) <= F
        return pool_.alloc(L.bytes, L.off);
    }
    void shape(Launch &L) const {
        L.max_m = L.max_n = 0;
        for (const Piece &p : L.pieces) {
            L.max_m = std::max(L.max_m, p.job->max_m);
            L.max_n = std::max(L.max_n, p.job->max_n);
        }
        L.bytes = need_(L.n, L.max_m, L.max_n);
    }
    static void truncate(Launch &L, uint64_t n) {
        uint64_t left = n;
        std::vector<Piece> kept;
        for (const Piece &p : L.pieces) {
            if (left == 0) break;
            kept.push_back({p.job, p.first, std::min(p.count, left)});
            left -= kept.back().count;
        }
        L.pieces.swap(kept);
        L.n = n;
    }

    ScratchPool pool_;
    std::deque<Job *> q_;
    uint64_t max_batch_ = 1, min_batch_ = 1;
    NeedFn need_;
    Stats stats_;
};

}  // namespace serve
