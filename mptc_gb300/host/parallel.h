// Work sharing for the host stream writer and reader: a job index counter
// drained by a few threads, the calling thread included.
#pragma once
#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <cstddef>
#include <functional>
#include <thread>
#include <vector>

namespace mptc_host {

// Threads of the host coder: the host's hardware threads, or the positive
// integer in the environment variable MPTC_HOST_THREADS when it is set (a
// caller that shares the host with other work, or a test that wants small
// chunks).
inline size_t host_threads() {
  if (const char *e = std::getenv("MPTC_HOST_THREADS")) {
    const long v = std::strtol(e, nullptr, 10);
    if (v > 0) return (size_t)std::min(v, 4096L);
  }
  return std::max(1u, std::thread::hardware_concurrency());
}

// Runs job(i) for i in [0, count) on up to `threads` threads, the calling
// thread included (jobs of threads that could not be started run on the
// others). Returns false if a job threw (an allocation failed) or returned
// false.
inline bool parallel_for(size_t count, size_t threads, const std::function<bool(size_t)> &job) {
  std::atomic<size_t> next{0};
  std::atomic<bool> ok{true};
  auto worker = [&] {
    for (size_t i; (i = next.fetch_add(1)) < count;) {
      try {
        if (!job(i)) ok = false;
      } catch (...) {
        ok = false;
      }
    }
  };
  std::vector<std::thread> pool;
  const size_t extra = std::min(threads, count) > 1 ? std::min(threads, count) - 1 : 0;
  try {
    pool.reserve(extra);
    for (size_t t = 0; t < extra; ++t) pool.emplace_back(worker);
  } catch (...) {
  }
  worker();
  for (std::thread &t : pool) t.join();
  return ok;
}

}  // namespace mptc_host
