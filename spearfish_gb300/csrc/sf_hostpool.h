// The host thread pool the plan build and result conversion split their work over.
#pragma once

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

#include <unistd.h>

namespace sfe {

// Host worker threads for the plan build, started on first use and kept for the process:
// starting threads per call would cost more than small batches save.  A process that forks
// gets a fresh pool in the child (the parent's threads do not exist there).
class HostPool {
 public:
  static HostPool& get() {
    static std::mutex mu;
    static HostPool* pool = nullptr;
    std::lock_guard<std::mutex> g(mu);
    if (!pool || pool->pid_ != getpid()) pool = new HostPool();  // a child's old pool is abandoned
    return *pool;
  }
  size_t workers() const { return threads_.size(); }
  // Queues fn; returns false if it could not be queued.
  bool post(std::function<void()> fn) {
    try {
      std::lock_guard<std::mutex> g(m_);
      q_.push_back(std::move(fn));
      queued_.fetch_add(1, std::memory_order_release);
    } catch (...) {
      return false;
    }
    cv_.notify_one();
    return true;
  }
  // How long a worker (or a caller waiting for its chunks) polls before it sleeps: a plan
  // build posts its phases back to back, and a sleeping thread takes tens of microseconds
  // to wake.
  static constexpr std::chrono::microseconds kSpin{200};

 private:
  HostPool() : pid_(getpid()) {
    const unsigned hw = std::thread::hardware_concurrency();
    const unsigned n = std::min(15u, hw > 1 ? hw - 1 : 0u);
    try {
      for (unsigned k = 0; k < n; ++k) threads_.emplace_back([this] { loop(); });
    } catch (...) {
    }
    for (auto& t : threads_) t.detach();
  }
  void loop() {
    for (;;) {
      const auto t0 = std::chrono::steady_clock::now();
      while (queued_.load(std::memory_order_acquire) == 0 &&
             std::chrono::steady_clock::now() - t0 < kSpin) {
      }
      std::function<void()> fn;
      {
        std::unique_lock<std::mutex> g(m_);
        cv_.wait(g, [this] { return !q_.empty(); });
        fn = std::move(q_.front());
        q_.pop_front();
        queued_.fetch_sub(1, std::memory_order_relaxed);
      }
      fn();
    }
  }
  pid_t pid_;
  std::vector<std::thread> threads_;
  std::mutex m_;
  std::condition_variable cv_;
  std::deque<std::function<void()>> q_;
  std::atomic<size_t> queued_{0};  // q_.size(), readable without the lock
};

// f(begin, end, k) for the k-th of up to max_threads contiguous chunks of [0, n), chunks 1..
// on the host pool's threads, when every chunk gets at least min_per_thread items (else one
// chunk on the calling thread).  The same (n, min_per_thread, max_threads) always gives the
// same chunks; a chunk the pool cannot take runs on the calling thread.
// How many chunks parallel_chunks(n, min_per_thread, max_threads, ...) makes.
inline size_t chunks_for(size_t n, size_t min_per_thread, int max_threads) {
  const size_t t = std::min<size_t>({HostPool::get().workers() + 1, (size_t)max_threads,
                                     min_per_thread ? n / min_per_thread : 1});
  return std::max<size_t>(t, 1);
}

template <class F>
void parallel_chunks(size_t n, size_t min_per_thread, int max_threads, F&& f) {
  HostPool& pool = HostPool::get();
  const size_t t = chunks_for(n, min_per_thread, max_threads);
  if (t <= 1) {
    f(size_t(0), n, 0);
    return;
  }
  const size_t chunk = (n + t - 1) / t;
  // `left` changes only under `m`, so that a worker is out of `done` once the caller has
  // taken `m` after seeing it reach zero.
  struct Done {
    std::mutex m;
    std::condition_variable cv;
    std::atomic<size_t> left{0};
  } done;
  for (size_t k = 1; k < t; ++k) {
    const size_t b = k * chunk, e = std::min(n, (k + 1) * chunk);
    {
      std::lock_guard<std::mutex> g(done.m);
      done.left.fetch_add(1, std::memory_order_relaxed);
    }
    const bool queued = pool.post([&f, &done, b, e, k] {
      f(b, e, (int)k);
      std::lock_guard<std::mutex> g(done.m);
      if (done.left.fetch_sub(1, std::memory_order_acq_rel) == 1) done.cv.notify_all();
    });
    if (!queued) {
      {
        std::lock_guard<std::mutex> g(done.m);
        done.left.fetch_sub(1, std::memory_order_relaxed);
      }
      f(b, e, (int)k);
    }
  }
  f(size_t(0), std::min(n, chunk), 0);
  const auto t0 = std::chrono::steady_clock::now();
  while (done.left.load(std::memory_order_acquire) != 0 &&
         std::chrono::steady_clock::now() - t0 < HostPool::kSpin) {
  }
  std::unique_lock<std::mutex> g(done.m);
  done.cv.wait(g, [&] { return done.left.load(std::memory_order_acquire) == 0; });
}

}  // namespace sfe
