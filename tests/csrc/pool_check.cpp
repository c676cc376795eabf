// Checks wlg::WorkerPool (qec_pf_wang_landau_gb300/csrc/wlg_pool.h) on the
// CPU: every index runs exactly once per job, across many jobs and sizes,
// and an exception thrown by one index reaches the caller, after which the
// pool keeps working.  Prints "ok" and exits 0 on success.
#include <atomic>
#include <cstdio>
#include <stdexcept>
#include <vector>

#include "wlg_pool.h"

int main()
{
  for (int threads : {1, 2, 5, 16}) {
    wlg::WorkerPool pool(threads);
    for (int job = 0; job < 200; ++job) {
      const int n = (job * 37) % 1000;
      std::vector<std::atomic<int>> hits(static_cast<size_t>(n));
      for (auto& h : hits) h.store(0);
      pool.run(n, 1 + job % 9, [&](int i) { hits[static_cast<size_t>(i)].fetch_add(1); });
      for (int i = 0; i < n; ++i)
        if (hits[static_cast<size_t>(i)].load() != 1) {
          std::printf("index %d ran %d times (threads %d, job %d)\n", i, hits[static_cast<size_t>(i)].load(), threads,
                      job);
          return 1;
        }
    }
    bool caught = false;
    try {
      pool.run(500, 4, [](int i) {
        if (i == 333) throw std::runtime_error("planted");
      });
    } catch (const std::runtime_error&) {
      caught = true;
    }
    if (!caught) {
      std::printf("exception lost (threads %d)\n", threads);
      return 1;
    }
    std::atomic<int> sum{0};
    pool.run(100, 3, [&](int i) { sum.fetch_add(i); });
    if (sum.load() != 4950) {
      std::printf("pool unusable after an exception (threads %d)\n", threads);
      return 1;
    }
  }
  std::printf("ok\n");
  return 0;
}
