// Stress check of the batch entry points' host worker pool: every index of
// every run executes exactly once, runs of different widths follow each
// other without a lost wake-up, and destruction joins the workers.
#include <atomic>
#include <cstdio>
#include <vector>

#include "host_pool.h"

int main() {
    for (unsigned workers : {0u, 1u, 3u, 15u}) {
        HostPool pool(workers);
        if (pool.size() != workers + 1) {
            std::printf("size %u != %u\n", pool.size(), workers + 1);
            return 1;
        }
        for (int rep = 0; rep < 2000; rep++) {
            const unsigned T = 1 + (unsigned)(rep * 7 % (workers + 3));  // may exceed size()
            const unsigned ran = T < pool.size() ? T : pool.size();
            std::vector<std::atomic<int>> hits(ran);
            for (auto &h : hits) h = 0;
            pool.run(T, [&](unsigned t) { hits[t]++; });
            for (unsigned t = 0; t < ran; t++)
                if (hits[t] != 1) {
                    std::printf("workers %u rep %d index %u ran %d times\n", workers, rep, t,
                                (int)hits[t]);
                    return 1;
                }
        }
    }
    std::printf("ok\n");
    return 0;
}
