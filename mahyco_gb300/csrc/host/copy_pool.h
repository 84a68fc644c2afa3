// Host copy threads of the field fetch (fetch.cu): plain C++, no CUDA.
#ifndef MAHYCO_GB300_COPY_POOL_H
#define MAHYCO_GB300_COPY_POOL_H

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstddef>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

namespace hydro {

// A few host threads that copy one buffer into another in pieces; the caller
// copies pieces too and returns once every piece is done.  The piece counter
// carries the job's number, so a thread still holding an earlier job takes
// no piece of a later one.
class CopyPool {
 public:
  explicit CopyPool(int workers) {
    for (int t = 0; t < workers; ++t) th_.emplace_back([this] { loop(); });
  }
  ~CopyPool() {
    {
      std::lock_guard<std::mutex> g(mu_);
      stop_ = true;
    }
    cv_.notify_all();
    for (auto& t : th_) t.join();
  }
  void copy(void* dst, const void* src, size_t bytes) {
    constexpr size_t kMinPiece = 1u << 20;
    int parts = (int)th_.size() + 1;
    while (parts > 1 && bytes / parts < kMinPiece) --parts;
    if (parts == 1) {
      std::memcpy(dst, src, bytes);
      return;
    }
    Job j{static_cast<char*>(dst), static_cast<const char*>(src), bytes,
          ((bytes + parts - 1) / parts + 63) / 64 * 64, parts};
    unsigned id;
    {
      std::lock_guard<std::mutex> g(mu_);
      job_ = j;
      id = ++job_id_;
      left_ = parts;
      next_.store((unsigned long long)id << 32, std::memory_order_release);
    }
    cv_.notify_all();
    work(j, id);
    std::unique_lock<std::mutex> l(mu_);
    done_.wait(l, [this] { return left_ == 0; });
  }

 private:
  struct Job {
    char* d;
    const char* s;
    size_t n, piece;
    int parts;
  };
  // takes pieces of job `id` until none is left (or another job started)
  void work(const Job& j, unsigned id) {
    for (;;) {
      unsigned long long v = next_.load(std::memory_order_acquire);
      do {
        if ((unsigned)(v >> 32) != id || (long long)(v & 0xffffffffull) >= j.parts) return;
      } while (!next_.compare_exchange_weak(v, v + 1, std::memory_order_acq_rel));
      const size_t a = (size_t)(v & 0xffffffffull) * j.piece;
      if (a < j.n) std::memcpy(j.d + a, j.s + a, std::min(j.piece, j.n - a));
      std::lock_guard<std::mutex> g(mu_);
      if (--left_ == 0) done_.notify_all();
    }
  }
  void loop() {
    unsigned seen = 0;
    for (;;) {
      Job j;
      {
        std::unique_lock<std::mutex> l(mu_);
        cv_.wait(l, [&] { return stop_ || job_id_ != seen; });
        if (stop_) return;
        seen = job_id_;
        j = job_;
      }
      work(j, seen);
    }
  }

  std::vector<std::thread> th_;
  std::mutex mu_;
  std::condition_variable cv_, done_;
  Job job_{};
  unsigned job_id_ = 0;
  int left_ = 0;
  std::atomic<unsigned long long> next_{0};
  bool stop_ = false;
};

}  // namespace hydro

#endif
