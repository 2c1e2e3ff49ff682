// Host-side data parallelism for the scene upload: fn(begin, end) over contiguous ranges of
// [0, n), each at least `grain` items, on a pool of worker threads started at the first use
// (one per hardware thread but the caller's, at most 63) so that the many small parallel
// steps of an upload do not each pay for starting threads. The caller takes ranges too and
// returns when all are done; calls from several threads run one after another.
#pragma once
#include <stddef.h>

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace nehost {

class WorkerPool {
 public:
  static WorkerPool& get() {
    // never destroyed: the workers wait on the condition variable until the process ends
    static WorkerPool* pool = new WorkerPool(
        (size_t)std::max(1u, std::min(64u, std::thread::hardware_concurrency())) - 1);
    return *pool;
  }
  size_t threads() const { return workers_.size() + 1; }
  // job(p) for p in [0, parts); returns once every part is done and no worker is inside the job
  void run(size_t parts, const std::function<void(size_t)>& job) {
    std::lock_guard<std::mutex> one(runLock_);
    {
      std::lock_guard<std::mutex> g(m_);
      job_ = &job;
      parts_ = parts;
      next_.store(0);
      left_ = parts;
      gen_++;
    }
    cv_.notify_all();
    work(job, parts);
    std::unique_lock<std::mutex> g(m_);
    done_.wait(g, [&] { return left_ == 0 && active_ == 0; });
    job_ = nullptr;
  }

 private:
  explicit WorkerPool(size_t n) {
    for (size_t i = 0; i < n; i++) workers_.emplace_back([this] { loop(); });
  }
  void work(const std::function<void(size_t)>& job, size_t parts) {
    for (;;) {
      const size_t p = next_.fetch_add(1);
      if (p >= parts) return;
      job(p);
      std::lock_guard<std::mutex> g(m_);
      if (--left_ == 0) done_.notify_all();
    }
  }
  void loop() {
    unsigned long long seen = 0;
    for (;;) {
      const std::function<void(size_t)>* job;
      size_t parts;
      {
        std::unique_lock<std::mutex> g(m_);
        cv_.wait(g, [&] { return gen_ != seen; });
        seen = gen_;
        if (left_ == 0 || !job_) continue;  // that job is already done
        job = job_;
        parts = parts_;
        active_++;
      }
      work(*job, parts);
      std::lock_guard<std::mutex> g(m_);
      if (--active_ == 0) done_.notify_all();
    }
  }
  std::vector<std::thread> workers_;
  std::mutex runLock_, m_;
  std::condition_variable cv_, done_;
  const std::function<void(size_t)>* job_ = nullptr;
  size_t parts_ = 0, left_ = 0, active_ = 0;
  std::atomic<size_t> next_{0};
  unsigned long long gen_ = 0;
};

template <class F>
void parallelFor(size_t n, size_t grain, F fn) {
  if (n == 0) return;
  WorkerPool& pool = WorkerPool::get();
  const size_t parts = std::max<size_t>(1, std::min(pool.threads(), (n + grain - 1) / std::max<size_t>(1, grain)));
  const size_t step = (n + parts - 1) / parts;
  if (parts == 1) {
    fn(0, n);
    return;
  }
  pool.run(parts, [&](size_t p) {
    const size_t b = p * step, e = std::min(n, b + step);
    if (b < e) fn(b, e);
  });
}

}  // namespace nehost
