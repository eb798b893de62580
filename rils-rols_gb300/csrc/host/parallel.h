// Host-side data parallelism for the per-candidate work of a round (factor
// splitting, encoding): fn(begin, end) over contiguous slices of [0, n) on
// up to 16 host threads, the calling thread taking the first slice.  Each
// slice writes only its own outputs, so the results (and their order) are
// those of a sequential loop.  Rounds smaller than two slices run inline.
#pragma once
#include <algorithm>
#include <cstddef>
#include <exception>
#include <mutex>
#include <thread>
#include <vector>

namespace rrh {

template <class F>
void parallel_slices(size_t n, size_t min_per_slice, F&& fn) {
  const size_t hw = std::max<size_t>(1, std::thread::hardware_concurrency());
  const size_t t = std::min<size_t>(std::min<size_t>(hw, 16), n / std::max<size_t>(1, min_per_slice));
  if (t <= 1) {
    fn(size_t(0), n);
    return;
  }
  std::exception_ptr err;
  std::mutex mu;
  auto run = [&](size_t b, size_t e) {
    try {
      fn(b, e);
    } catch (...) {
      std::lock_guard<std::mutex> lk(mu);
      if (!err) err = std::current_exception();
    }
  };
  std::vector<std::thread> workers;
  workers.reserve(t - 1);
  for (size_t i = 1; i < t; ++i) workers.emplace_back(run, n * i / t, n * (i + 1) / t);
  run(0, n / t);
  for (auto& w : workers) w.join();
  if (err) std::rethrow_exception(err);
}

}  // namespace rrh
