// Host-side data parallelism for the per-candidate work of a round (factor
// splitting, encoding): fn(begin, end) over contiguous slices of [0, n) on
// up to 16 host threads, the calling thread taking the first slice.  Each
// slice writes only its own outputs, so the results (and their order) are
// those of a sequential loop.  Rounds smaller than two slices run inline.
//
// The worker threads are started once per process and wait for slices on a
// shared queue (a local-search round is a few milliseconds of host work, so
// starting threads per call would cost a noticeable share of it).  Several
// callers (the serving loop's jobs) may share the pool: a caller whose slices
// are still queued runs them itself instead of waiting, so no call waits on
// another's work.
#pragma once
#include <algorithm>
#include <condition_variable>
#include <cstddef>
#include <deque>
#include <exception>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace rrh {

class SlicePool {
 public:
  static SlicePool& get() {
    // never destroyed: the workers stay blocked on the queue until the
    // process ends
    static SlicePool* pool = new SlicePool();
    return *pool;
  }
  size_t workers() const { return n_workers_; }

  struct Job {
    std::function<void()> fn;
    bool taken = false;
  };
  void push(Job* j) {
    {
      std::lock_guard<std::mutex> lk(mu_);
      q_.push_back(j);
    }
    cv_.notify_one();
  }
  // the caller runs its own job when no worker has taken it yet; a claimed
  // job leaves the queue, so no worker holds a pointer to it afterwards
  bool claim(Job* j) {
    std::lock_guard<std::mutex> lk(mu_);
    if (j->taken) return false;
    j->taken = true;
    q_.erase(std::find(q_.begin(), q_.end(), j));
    return true;
  }

 private:
  SlicePool() {
    const size_t hw = std::max<size_t>(1, std::thread::hardware_concurrency());
    n_workers_ = std::min<size_t>(hw, 16) - 1;
    for (size_t i = 0; i < n_workers_; ++i) std::thread([this] { loop(); }).detach();
  }
  void loop() {
    for (;;) {
      Job* j = nullptr;
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [this] { return !q_.empty(); });
        j = q_.front();
        q_.pop_front();
        if (j->taken) continue;
        j->taken = true;
      }
      j->fn();
    }
  }
  std::mutex mu_;
  std::condition_variable cv_;
  std::deque<Job*> q_;
  size_t n_workers_ = 0;
};

template <class F>
void parallel_slices(size_t n, size_t min_per_slice, F&& fn) {
  SlicePool& pool = SlicePool::get();
  const size_t t = std::min<size_t>(pool.workers() + 1, n / std::max<size_t>(1, min_per_slice));
  if (t <= 1) {
    fn(size_t(0), n);
    return;
  }
  std::exception_ptr err;
  std::mutex mu;
  std::condition_variable done_cv;
  size_t done = 0;
  auto run = [&](size_t b, size_t e) {
    try {
      fn(b, e);
    } catch (...) {
      std::lock_guard<std::mutex> lk(mu);
      if (!err) err = std::current_exception();
    }
  };
  std::vector<SlicePool::Job> jobs(t - 1);
  for (size_t i = 1; i < t; ++i) {
    const size_t b = n * i / t, e = n * (i + 1) / t;
    jobs[i - 1].fn = [&, b, e] {
      run(b, e);
      std::lock_guard<std::mutex> lk(mu);
      ++done;
      done_cv.notify_one();
    };
    pool.push(&jobs[i - 1]);
  }
  run(0, n / t);
  // slices no worker has started yet run here
  for (auto& j : jobs)
    if (pool.claim(&j)) j.fn();
  std::unique_lock<std::mutex> lk(mu);
  done_cv.wait(lk, [&] { return done == t - 1; });
  if (err) std::rethrow_exception(err);
}

}  // namespace rrh
