// Host-side parallel loop for the setup passes (pattern, coarsening): [0, n) split into contiguous
// chunks over the hardware threads.  Each index's work writes only its own outputs, so results do
// not depend on the split.
#pragma once

#include <algorithm>
#include <thread>
#include <vector>

template <class Fn>
void host_parallel_for(long n, long min_chunk, Fn fn) {
  const long hw = std::max(1u, std::thread::hardware_concurrency());
  const long nt = std::max(1L, std::min({hw, 32L, (n + min_chunk - 1) / std::max(1L, min_chunk)}));
  if (nt <= 1) {
    fn(0L, n, 0);
    return;
  }
  std::vector<std::thread> pool;
  const long chunk = (n + nt - 1) / nt;
  for (long t = 0; t < nt; ++t) {
    const long b = t * chunk, e = std::min(n, b + chunk);
    if (b >= e) break;
    pool.emplace_back([=, &fn] { fn(b, e, (int)t); });
  }
  for (auto& th : pool) th.join();
}

inline int host_threads() { return (int)std::min(32u, std::max(1u, std::thread::hardware_concurrency())); }
