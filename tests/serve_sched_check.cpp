// CPU check of the serving loop's admission and batching decisions
// (esperanto_gb300/csrc/serve_sched.h) with a synthetic scratch-need
// function and launches completed in chosen orders: merging of small
// requests, splitting of large ones, a request held back by the memory
// budget and admitted when a launch returns its scratch, FIFO order, the
// pool never over-committed, and every read launched exactly once.
#include <cstdio>
#include <random>
#include <vector>

#include "serve_sched.h"

using namespace serve;

#define CHECK(c)                                                      \
    do {                                                              \
        if (!(c)) {                                                   \
            std::printf("line %d: check failed: %s\n", __LINE__, #c); \
            return 1;                                                 \
        }                                                             \
    } while (0)

// 1 KiB of scratch per warp of 32 reads, at most 64 warps (full
// residency), per-warp bytes growing with the longest read
static uint64_t need(uint64_t n, uint32_t m, uint32_t) {
    uint64_t warps = std::min<uint64_t>(64, (n + 31) / 32);
    return warps * (m <= 150 ? 1024 : 2048);
}

static int pool_checks() {
    ScratchPool p;
    p.reset(1 << 20);
    std::mt19937_64 rng(7);
    std::vector<std::pair<uint64_t, uint64_t>> live;
    for (int it = 0; it < 20000; it++) {
        if (live.empty() || rng() % 3) {
            uint64_t b = 1 + rng() % 40000, off;
            if (p.alloc(b, off)) {
                for (auto &l : live)  // no overlap with a live block
                    CHECK(off + al256(b) <= l.first || l.first + al256(l.second) <= off);
                CHECK(off + al256(b) <= p.size());
                live.push_back({off, b});
            }
        } else {
            size_t k = rng() % live.size();
            p.release(live[k].first, live[k].second);
            live.erase(live.begin() + k);
        }
        CHECK(p.used() <= p.size());
    }
    for (auto &l : live) p.release(l.first, l.second);
    CHECK(p.used() == 0 && p.largest_free() == p.size());
    return 0;
}

static int merge_split_checks() {
    Scheduler s(1 << 30, 1000, 256, need);
    Job a, b, c, d;
    a.n = 100; b.n = 200; c.n = 2500; d.n = 50;
    for (Job *j : {&a, &b, &c, &d}) { j->max_m = 150; j->max_n = 214; s.push(j); }
    Launch L1, L2, L3, L4;
    CHECK(s.next(L1) && L1.n == 1000 && L1.pieces.size() == 3);  // a, b and 700 of c
    CHECK(L1.pieces[2].job == &c && L1.pieces[2].first == 0 && L1.pieces[2].count == 700);
    CHECK(s.next(L2) && L2.n == 1000 && L2.pieces.size() == 1 && L2.pieces[0].first == 700);
    CHECK(s.next(L3) && L3.n == 850 && L3.pieces.size() == 2);  // rest of c, then d
    CHECK(!s.next(L4) && s.empty());
    std::vector<Job *> done;
    s.finish(L2, done);
    CHECK(done.empty());
    s.finish(L1, done);
    CHECK(done.size() == 2 && done[0] == &a && done[1] == &b);
    s.finish(L3, done);
    CHECK(done.size() == 4 && done[2] == &c && done[3] == &d);
    CHECK(s.stats().merged == 2 && s.stats().split_jobs == 1 && s.stats().launches == 3);
    CHECK(s.stats().reads == 2850 && s.stats().budget_waits == 0);
    // requests of another CIGAR stride (group) do not share a launch
    Scheduler t(1 << 30, 1000, 256, need);
    Job e, f;
    e.n = 10; f.n = 10; f.group = 1;
    t.push(&e);
    t.push(&f);
    Launch M;
    CHECK(t.next(M) && M.n == 10 && M.pieces.size() == 1 && M.pieces[0].job == &e);
    return 0;
}

static int budget_checks() {
    // room for 100 warps: one full launch (64 warps) and 36 warps more
    Scheduler s(100 * 1024, 4096, 512, need);
    Job a, b, c;
    a.n = 4096; b.n = 4096; c.n = 600;
    for (Job *j : {&a, &b, &c}) { j->max_m = 150; j->max_n = 214; j->group = 0; }
    s.push(&a);
    s.push(&b);
    s.push(&c);
    Launch La, Lb, Lc, Lx;
    CHECK(s.next(La) && La.n == 4096 && La.bytes == 64 * 1024);
    // b is cut to the 36 warps left: 1152 reads
    CHECK(s.next(Lb) && Lb.n == 1152 && Lb.bytes == 36 * 1024 && s.stats().cuts == 1);
    CHECK(s.pool().used() <= s.pool().size());
    // nothing left: the rest of b waits for memory, not for a slot
    CHECK(!s.next(Lx) && s.stats().budget_waits == 1 && !s.empty());
    CHECK(!s.next(Lx) && s.stats().budget_waits == 1);  // a retry is the same wait
    std::vector<Job *> done;
    s.finish(La, done);
    CHECK(done.size() == 1 && done[0] == &a);
    // the freed scratch admits the rest of b (FIFO: before c)
    CHECK(s.next(Lc) && Lc.pieces[0].job == &b && Lc.pieces[0].first == 1152);
    CHECK(s.pool().used() <= s.pool().size());
    // a request whose smallest launch cannot fit the whole pool is refused
    Job huge;
    huge.n = 100000; huge.max_m = 300;
    Scheduler u(10 * 1024, 4096, 512, need);
    CHECK(!u.admissible(huge));
    huge.max_m = 150;
    CHECK(!u.admissible(huge));  // 512 reads = 16 warps > 10
    Scheduler v(16 * 1024, 4096, 512, need);
    CHECK(v.admissible(huge));
    return 0;
}

static int random_simulation() {
    std::mt19937_64 rng(11);
    for (int round = 0; round < 200; round++) {
        const uint64_t pool = (20 + rng() % 200) * 1024;
        Scheduler s(pool, 256 + rng() % 4000, 64 + rng() % 256, need);
        std::vector<Job> jobs(1 + rng() % 40);
        uint64_t expect = 0;
        for (auto &j : jobs) {
            j.n = 1 + rng() % 6000;
            j.max_m = (rng() & 1) ? 150 : 300;
            j.max_n = j.max_m + 64;
            j.group = rng() % 3 == 0;
            if (!s.admissible(j)) { j.n = 0; continue; }
            expect += j.n;
            s.push(&j);
        }
        std::vector<Launch> running;
        std::vector<Job *> done;
        uint64_t launched = 0, order_job = 0, order_read = 0;
        int guard = 0;
        while (!s.empty() || !running.empty()) {
            CHECK(++guard < 1000000);
            Launch L;
            const size_t slots = 1 + rng() % 4;
            if (running.size() < slots && s.next(L)) {
                // reads are launched in submission order
                for (auto &p : L.pieces) {
                    uint64_t ji = (uint64_t)(p.job - jobs.data());
                    while (order_job < jobs.size() && (jobs[order_job].n == 0 ||
                                                       order_read == jobs[order_job].n)) {
                        order_job++;
                        order_read = 0;
                    }
                    CHECK(ji == order_job && p.first == order_read);
                    order_read += p.count;
                }
                launched += L.n;
                running.push_back(L);
                CHECK(s.pool().used() <= s.pool().size());
                continue;
            }
            // nothing admitted: some launch must be running to free memory
            CHECK(!running.empty());
            size_t k = rng() % running.size();
            s.finish(running[k], done);
            running.erase(running.begin() + k);
        }
        CHECK(launched == expect && s.stats().reads == expect);
        size_t nz = 0;
        for (auto &j : jobs) nz += j.n > 0;
        CHECK(done.size() == nz);
        for (auto &j : jobs) CHECK(j.done == j.n && j.next == j.n);
        CHECK(s.pool().used() == 0);
    }
    return 0;
}

static int close_checks() {
    Scheduler s(1 << 30, 1000, 100, need);
    Job a, b, c;
    a.n = 1500; b.n = 10; c.n = 20;
    s.push(&a);
    s.push(&b);
    s.push(&c);
    Launch L;
    CHECK(s.next(L) && L.n == 1000);  // a has started
    std::vector<Job *> dropped;
    s.drop_unstarted(dropped);
    CHECK(dropped.size() == 2 && dropped[0] == &b && dropped[1] == &c);
    Launch L2;
    CHECK(s.next(L2) && L2.n == 500 && L2.pieces.size() == 1);  // a finishes its reads
    CHECK(s.empty());
    return 0;
}

int main() {
    if (pool_checks() || merge_split_checks() || budget_checks() || random_simulation() ||
        close_checks())
        return 1;
    std::printf("ok\n");
    return 0;
}
