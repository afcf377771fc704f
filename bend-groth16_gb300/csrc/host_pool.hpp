// A process-wide pool of host worker threads for the serial host steps of an MSM that split
// into independent pieces (the per-window part sums of msm_finish).  parallel_for runs
// f(0..n-1) on the pool's idle workers and on the calling thread, so it completes even when
// every worker is busy with another caller's work; calls from several threads (batch lanes,
// the serving loop) interleave freely.
#pragma once
#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <deque>
#include <exception>
#include <functional>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

namespace bg {

class HostPool {
 public:
  // the shared pool: min(hardware threads - 1, 7) workers, created on first use
  static HostPool& get() {
    static HostPool pool(std::min(7u, std::max(1u, std::thread::hardware_concurrency()) - 1u));
    return pool;
  }

  unsigned workers() const { return (unsigned)threads_.size(); }

  void parallel_for(int n, const std::function<void(int)>& f) {
    if (n <= 0) return;
    const unsigned helpers = std::min<unsigned>(workers(), (unsigned)n - 1u);
    if (helpers == 0) {
      for (int i = 0; i < n; i++) f(i);
      return;
    }
    auto job = std::make_shared<Job>();
    job->n = n;
    job->f = &f;
    job->pending = helpers;
    {
      std::lock_guard<std::mutex> lk(mu_);
      for (unsigned h = 0; h < helpers; h++) queue_.push_back(job);
    }
    cv_.notify_all();
    job->run();
    // helpers that start after the indices are gone return at once; wait for all of them
    // (they read `f`, which lives in the caller's frame)
    std::unique_lock<std::mutex> lk(job->mu);
    job->cv.wait(lk, [&] { return job->pending == 0; });
    if (job->error) std::rethrow_exception(job->error);
  }

  ~HostPool() {
    {
      std::lock_guard<std::mutex> lk(mu_);
      stop_ = true;
    }
    cv_.notify_all();
    for (auto& t : threads_) t.join();
  }

 private:
  struct Job {
    int n = 0;
    const std::function<void(int)>* f = nullptr;
    std::atomic<int> next{0};
    unsigned pending = 0;  // helper runs not finished yet (guarded by mu)
    std::exception_ptr error;
    std::mutex mu;
    std::condition_variable cv;
    void run() {
      try {
        for (int i; (i = next.fetch_add(1)) < n;) (*f)(i);
      } catch (...) {
        std::lock_guard<std::mutex> lk(mu);
        if (!error) error = std::current_exception();
        next.store(n);
      }
    }
  };

  explicit HostPool(unsigned n) {
    for (unsigned i = 0; i < n; i++) threads_.emplace_back([this] { loop(); });
  }

  void loop() {
    for (;;) {
      std::shared_ptr<Job> job;
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return stop_ || !queue_.empty(); });
        if (stop_ && queue_.empty()) return;
        job = queue_.front();
        queue_.pop_front();
      }
      job->run();
      {
        std::lock_guard<std::mutex> lk(job->mu);
        job->pending--;
      }
      job->cv.notify_all();
    }
  }

  std::vector<std::thread> threads_;
  std::deque<std::shared_ptr<Job>> queue_;
  std::mutex mu_;
  std::condition_variable cv_;
  bool stop_ = false;
};

}  // namespace bg
