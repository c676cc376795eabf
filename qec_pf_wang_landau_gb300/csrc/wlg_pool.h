// A persistent pool of host worker threads for the per-problem host phases
// of a batch (hand-off, stitching).  Starting a thread costs tens of
// microseconds, comparable to those phases' whole work for a bench-sized
// batch, so the threads are started once per context and wait on a
// condition variable between jobs.  The calling thread works too.  One job
// at a time: a pool belongs to one context, which serves one host thread.
#pragma once

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <exception>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace wlg {

class WorkerPool {
 public:
  // `threads` in total, the caller included (at least 1).
  explicit WorkerPool(int threads)
  {
    for (int w = 1; w < threads; ++w) workers_.emplace_back([this] { work(); });
  }
  ~WorkerPool()
  {
    {
      std::lock_guard<std::mutex> lk(mu_);
      stop_ = true;
    }
    cv_.notify_all();
    for (std::thread& t : workers_) t.join();
  }
  WorkerPool(const WorkerPool&) = delete;
  WorkerPool& operator=(const WorkerPool&) = delete;

  int threads() const { return static_cast<int>(workers_.size()) + 1; }

  // f(i) for every i in [0, n), indices taken in chunks of `chunk` by the
  // caller and the workers; returns when all are done and rethrows the
  // first exception f threw.
  void run(int n, int chunk, const std::function<void(int)>& f)
  {
    if (n <= 0) return;
    chunk = std::max(chunk, 1);
    if (workers_.empty() || n <= chunk) {
      for (int i = 0; i < n; ++i) f(i);
      return;
    }
    {
      std::lock_guard<std::mutex> lk(mu_);
      job_ = &f;
      n_ = n;
      chunk_ = chunk;
      next_.store(0);
      busy_ = static_cast<int>(workers_.size());
      err_ = nullptr;
      ++gen_;
    }
    cv_.notify_all();
    drain();
    std::unique_lock<std::mutex> lk(mu_);
    done_cv_.wait(lk, [&] { return busy_ == 0; });
    job_ = nullptr;
    if (err_) std::rethrow_exception(err_);
  }

 private:
  void drain()
  {
    try {
      for (;;) {
        const int i0 = next_.fetch_add(chunk_);
        if (i0 >= n_) break;
        const int i1 = std::min(n_, i0 + chunk_);
        for (int i = i0; i < i1; ++i) (*job_)(i);
      }
    } catch (...) {
      next_.store(n_);  // stop handing out work
      std::lock_guard<std::mutex> lk(mu_);
      if (!err_) err_ = std::current_exception();
    }
  }

  void work()
  {
    long seen = 0;
    for (;;) {
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return stop_ || gen_ != seen; });
        if (stop_) return;
        seen = gen_;
      }
      drain();
      std::lock_guard<std::mutex> lk(mu_);
      if (--busy_ == 0) done_cv_.notify_all();
    }
  }

  std::vector<std::thread> workers_;
  std::mutex mu_;
  std::condition_variable cv_, done_cv_;
  const std::function<void(int)>* job_ = nullptr;
  int n_ = 0, chunk_ = 1, busy_ = 0;
  long gen_ = 0;
  bool stop_ = false;
  std::atomic<int> next_{0};
  std::exception_ptr err_;
};

}  // namespace wlg
