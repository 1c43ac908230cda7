// mcba_host_pool.h -- a small persistent pool of host threads for the bulk
// copies and checks of the host-side entry points (problem load, pinned
// staging of the raw graph).  Those passes are bound by one core's memory
// bandwidth; spread over a few cores they run several times faster.
//
// run(n, fn) calls fn(0) .. fn(n-1), the calling thread taking part, and
// returns when all have returned.  One job runs at a time (callers from
// several threads queue on a mutex).  Workers start on first use and wait on
// a condition variable between jobs.
#pragma once

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstddef>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace mcba {

class HostPool {
 public:
  static HostPool& get() {
    static HostPool* p = new HostPool();  // never destroyed: workers outlive static teardown
    return *p;
  }

  void run(int n, const std::function<void(int)>& fn) {
    if (n <= 0) return;
    if (n == 1 || workers_.empty()) {
      for (int i = 0; i < n; ++i) fn(i);
      return;
    }
    std::lock_guard<std::mutex> job_lock(job_mu_);
    {
      std::lock_guard<std::mutex> lk(mu_);
      job_ = &fn;
      n_ = n;
      pending_ = n;
      ++gen_;
      next_.store((unsigned long long)(unsigned)gen_ << 32);
    }
    cv_.notify_all();
    work();
    std::unique_lock<std::mutex> lk(mu_);
    done_cv_.wait(lk, [&] { return pending_ == 0; });
    job_ = nullptr;
  }

  int size() const { return (int)workers_.size() + 1; }

 private:
  HostPool() {
    const unsigned hc = std::thread::hardware_concurrency();
    const int nw = (int)std::min<unsigned>(hc > 1 ? hc - 1 : 0, 7);
    for (int i = 0; i < nw; ++i) workers_.emplace_back([this] { loop(); });
    for (auto& t : workers_) t.detach();
  }

  // Claims task indices of the job with tag g: the counter carries the job's
  // tag in its high half, so a thread that read an older job never claims a
  // task of a newer one.
  int claim(unsigned g, int n) {
    unsigned long long v = next_.load();
    for (;;) {
      if ((unsigned)(v >> 32) != g || (int)(v & 0xffffffffu) >= n) return -1;
      if (next_.compare_exchange_weak(v, v + 1)) return (int)(v & 0xffffffffu);
    }
  }

  void work() {
    const std::function<void(int)>* fn;
    int n;
    unsigned g;
    {
      std::lock_guard<std::mutex> lk(mu_);
      fn = job_;
      n = n_;
      g = (unsigned)gen_;
    }
    if (!fn) return;
    int done = 0;
    for (int i = claim(g, n); i >= 0; i = claim(g, n)) {
      (*fn)(i);
      ++done;
    }
    if (done) {
      std::lock_guard<std::mutex> lk(mu_);
      pending_ -= done;
      if (pending_ == 0) done_cv_.notify_all();
    }
  }

  void loop() {
    unsigned long long seen = 0;
    for (;;) {
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return gen_ != seen; });
        seen = gen_;
      }
      work();
    }
  }

  std::mutex job_mu_;
  std::mutex mu_;
  std::condition_variable cv_, done_cv_;
  const std::function<void(int)>* job_ = nullptr;
  int n_ = 0;
  std::atomic<unsigned long long> next_{0};
  int pending_ = 0;
  unsigned long long gen_ = 0;
  std::vector<std::thread> workers_;
};

// Chunk [0, n) into at most `parts` ranges of at least `min_chunk` items and
// run fn(begin, end) on each through the pool.
inline void host_parallel_ranges(size_t n, size_t min_chunk, const std::function<void(size_t, size_t)>& fn) {
  HostPool& pool = HostPool::get();
  const size_t parts = std::max<size_t>(1, std::min<size_t>((size_t)pool.size(), n / std::max<size_t>(min_chunk, 1)));
  const size_t per = (n + parts - 1) / parts;
  pool.run((int)parts, [&](int i) {
    const size_t b = (size_t)i * per, e = std::min(n, b + per);
    if (b < e) fn(b, e);
  });
}

}  // namespace mcba
