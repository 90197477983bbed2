// Host-side parallel loop for the setup passes (pattern, coarsening): [0, n) split into contiguous
// chunks over the hardware threads.  Each index's work writes only its own outputs, so results do
// not depend on the split.
#pragma once

#include <algorithm>
#include <thread>
#include <vector>

// The split host_parallel_for makes of [0, n): chunk t is [t * chunk, min(n, (t + 1) * chunk)).
struct HostSplit {
  long nt, chunk;
};
inline HostSplit host_split(long n, long min_chunk) {
  const long hw = std::max(1u, std::thread::hardware_concurrency());
  const long nt = std::max(1L, std::min({hw, 32L, (n + min_chunk - 1) / std::max(1L, min_chunk)}));
  return HostSplit{nt, std::max(1L, (n + nt - 1) / nt)};
}

template <class Fn>
void host_parallel_for(long n, long min_chunk, Fn fn) {
  const HostSplit sp = host_split(n, min_chunk);
  const long nt = sp.nt, chunk = sp.chunk;
  if (nt <= 1) {
    fn(0L, n, 0);
    return;
  }
  std::vector<std::thread> pool;
  for (long t = 0; t < nt; ++t) {
    const long b = t * chunk, e = std::min(n, b + chunk);
    if (b >= e) break;
    pool.emplace_back([=, &fn] { fn(b, e, (int)t); });
  }
  for (auto& th : pool) th.join();
}

inline int host_threads() { return (int)std::min(32u, std::max(1u, std::thread::hardware_concurrency())); }

// True when some a[q], q in [0, n), lies outside [lo, hi) (checked over the host threads).
inline bool host_any_outside(const int* a, long n, int lo, int hi) {
  std::vector<char> bad(32, 0);
  host_parallel_for(n, 1 << 18, [&](long q0, long q1, int t) {
    for (long q = q0; q < q1; ++q)
      if (a[q] < lo || a[q] >= hi) bad[t] = 1;
  });
  for (char b : bad)
    if (b) return true;
  return false;
}
