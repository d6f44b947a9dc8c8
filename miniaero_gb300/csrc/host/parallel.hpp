// Host-side parallel loop for mesh setup.
#pragma once
#include <algorithm>
#include <cstddef>
#include <thread>
#include <vector>

namespace miniaero {

// body(begin, end) over [0, n) in contiguous chunks on the host's threads
// (at most 64, at least 16384 items each). Every item is computed by the same
// expressions whatever the chunking, so results do not depend on the thread
// count; body must only write what its own items own.
template <class F>
void parallel_for(size_t n, F body) {
  const size_t hw = std::max(1u, std::thread::hardware_concurrency());
  const size_t nt = std::min<size_t>(std::min<size_t>(hw, 64), n / 16384);
  if (nt <= 1) {
    body(size_t(0), n);
    return;
  }
  const size_t chunk = (n + nt - 1) / nt;
  std::vector<std::thread> threads;
  for (size_t t = 0; t < nt; ++t) {
    const size_t b = t * chunk, e = std::min(n, b + chunk);
    if (b < e) threads.emplace_back(body, b, e);
  }
  for (auto& th : threads) th.join();
}

}  // namespace miniaero
