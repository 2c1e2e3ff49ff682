// Host-side data parallelism for the scene upload: fn(begin, end) over contiguous ranges of
// [0, n) on up to one thread per hardware thread (at most 64), each range at least `grain`
// items. The calling thread takes the first range.
#pragma once
#include <stddef.h>

#include <algorithm>
#include <thread>
#include <vector>

namespace nehost {

template <class F>
void parallelFor(size_t n, size_t grain, F fn) {
  if (n == 0) return;
  const size_t hw = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
  const size_t parts = std::max<size_t>(1, std::min(hw, (n + grain - 1) / std::max<size_t>(1, grain)));
  const size_t step = (n + parts - 1) / parts;
  std::vector<std::thread> ts;
  ts.reserve(parts);
  for (size_t p = 1; p < parts; p++) {
    const size_t b = p * step, e = std::min(n, b + step);
    if (b < e) ts.emplace_back([=] { fn(b, e); });
  }
  fn(0, std::min(n, step));
  for (std::thread& t : ts) t.join();
}

}  // namespace nehost
