// Worker threads for the host setup passes (ordering, symbolic structure,
// matrix permutations).  Every caller writes disjoint outputs from inputs no
// thread modifies, so the results do not depend on the thread count.
#pragma once
#include <algorithm>
#include <cstdlib>
#include <exception>
#include <thread>
#include <vector>

namespace rschol {

// Threads a setup pass may use: the hardware's, at most 16.  The environment
// variable RSCHOL_HOST_THREADS overrides it (1: everything on the calling
// thread); it is read at every call.
inline int host_threads() {
  if (const char* e = std::getenv("RSCHOL_HOST_THREADS")) {
    const int v = std::atoi(e);
    if (v >= 1) return std::min(v, 64);
  }
  const int hw = (int)std::thread::hardware_concurrency();
  return std::max(1, std::min(hw, 16));
}

// fn(begin, end) over [0, n) in contiguous chunks, one per thread, on at most
// host_threads() threads and with at least `grain` items per chunk.
// An exception thrown by fn on any thread is rethrown on the calling thread
// once all of them have finished.
template <class F>
void parallel_chunks(long long n, long long grain, F&& fn) {
  if (n <= 0) return;
  const long long want = (n + std::max(1LL, grain) - 1) / std::max(1LL, grain);
  const int T = (int)std::min<long long>(host_threads(), want);
  if (T <= 1) {
    fn(0LL, n);
    return;
  }
  const long long chunk = (n + T - 1) / T;
  std::vector<std::exception_ptr> err(T);
  std::vector<std::thread> pool;
  pool.reserve(T - 1);
  for (int t = 1; t < T; ++t) {
    const long long b = std::min(n, t * chunk), e = std::min(n, b + chunk);
    pool.emplace_back([&fn, &err, t, b, e]() {
      try {
        fn(b, e);
      } catch (...) {
        err[t] = std::current_exception();
      }
    });
  }
  try {
    fn(0LL, std::min(n, chunk));
  } catch (...) {
    err[0] = std::current_exception();
  }
  for (std::thread& th : pool) th.join();
  for (std::exception_ptr& x : err)
    if (x) std::rethrow_exception(x);
}

// fn(worker) for worker = 0 .. T-1 on T threads (the calling thread is
// worker 0); for work queues whose items the workers take themselves.
template <class F>
void run_workers(int T, F&& fn) {
  parallel_chunks(T, 1, [&fn](long long b, long long e) {
    for (long long t = b; t < e; ++t) fn((int)t);
  });
}

}  // namespace rschol
