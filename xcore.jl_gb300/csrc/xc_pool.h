// A fixed pool of host threads for running one job per index, used by the
// ensemble step to drive the members' Stokes solves concurrently.  Host code
// only (the threads make `device` current before their first job).
#pragma once

#include <atomic>
#include <condition_variable>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

namespace xc {

// A fixed set of host threads running job(i) for i in [0, n), each thread
// taking the next index until none is left; run() returns when all are done.
class WorkerPool {
 public:
  WorkerPool(int nthreads, int device) : device_(device) {
    for (int t = 0; t < nthreads; ++t) th_.emplace_back([this] { loop(); });
  }
  ~WorkerPool() {
    {
      std::lock_guard<std::mutex> l(mu_);
      quit_ = true;
    }
    go_.notify_all();
    for (auto& t : th_) t.join();
  }
  void run(int n, const std::function<void(int)>& job) {
    {
      std::lock_guard<std::mutex> l(mu_);
      job_ = &job;
      n_ = n;
      next_.store(0);
      busy_ = (int)th_.size();
      ++gen_;
    }
    go_.notify_all();
    std::unique_lock<std::mutex> l(mu_);
    done_.wait(l, [this] { return busy_ == 0; });
  }

 private:
  void loop() {
    cudaSetDevice(device_);
    int seen = 0;
    for (;;) {
      const std::function<void(int)>* job;
      int n;
      {
        std::unique_lock<std::mutex> l(mu_);
        go_.wait(l, [&] { return quit_ || gen_ != seen; });
        if (quit_) return;
        seen = gen_;
        job = job_;
        n = n_;
      }
      for (int i; (i = next_.fetch_add(1)) < n;) (*job)(i);
      {
        std::lock_guard<std::mutex> l(mu_);
        if (--busy_ == 0) done_.notify_all();
      }
    }
  }
  std::vector<std::thread> th_;
  std::mutex mu_;
  std::condition_variable go_, done_;
  const std::function<void(int)>* job_ = nullptr;
  int n_ = 0, gen_ = 0, busy_ = 0;
  std::atomic<int> next_{0};
  bool quit_ = false;
  int device_;
};

}  // namespace xc
