// Batch gate of the solve server's block solves (host only, no CUDA).
//
// Large requests are solved whole by the block PCG on worker threads, one
// batch of iterations (one graph launch and its poll) at a time.  Two block
// solves side by side fill the GPU, and the small requests' admissions
// (uploads, assembly) and packed iterations then wait for them: on a
// 512-request stream their mean latency went from 0.13 s with one worker to
// 0.82 s with two.  The gate lets all workers run batches while no small
// request is being admitted or iterating, and one at a time while one is.
//
// A batch waits only while another batch runs, and every batch ends (its
// kernels finish and the worker calls leave()), so every wait ends.
#pragma once

#include <condition_variable>
#include <mutex>

namespace elx {

class BatchGate {
 public:
  explicit BatchGate(int workers = 2) : workers_(workers < 1 ? 1 : workers) {}

  // Before a batch: waits until fewer batches run than the current limit
  // (1 while small work is present, else the number of workers).
  void enter() {
    std::unique_lock<std::mutex> lk(mu_);
    cv_.wait(lk, [&] { return running_ < limit(); });
    running_++;
  }
  // After a batch (also when it failed).
  void leave() {
    {
      std::lock_guard<std::mutex> lk(mu_);
      running_--;
    }
    cv_.notify_all();
  }
  // Small requests entering (+1: admission starts) or leaving (-1: retired
  // or failed) the GPU.
  void small(int delta) {
    {
      std::lock_guard<std::mutex> lk(mu_);
      small_ += delta;
    }
    if (delta < 0) cv_.notify_all();
  }
  void set_workers(int workers) {
    {
      std::lock_guard<std::mutex> lk(mu_);
      workers_ = workers < 1 ? 1 : workers;
    }
    cv_.notify_all();
  }
  int running() {
    std::lock_guard<std::mutex> lk(mu_);
    return running_;
  }
  int small_count() {
    std::lock_guard<std::mutex> lk(mu_);
    return small_;
  }

 private:
  int limit() const { return small_ > 0 ? 1 : workers_; }
  std::mutex mu_;
  std::condition_variable cv_;
  int workers_;
  int small_ = 0, running_ = 0;
};

}  // namespace elx
