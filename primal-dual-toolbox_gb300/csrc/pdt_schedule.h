// pdt_schedule.h -- host-side assignment of a batch's problems to worker streams (header-only, so that the
// CPU tests build it as is).
#pragma once

#include <algorithm>
#include <cstddef>
#include <vector>

namespace pdt {

// Worker stream (0 .. P-1) of each problem, given each problem's cost per iteration: problems in order of
// decreasing cost (ties by index), each to the stream with the least cost so far (ties: the lowest stream).
// Longest-processing-time-first list scheduling: the most loaded stream, the critical path of a batched
// round, is at most 4/3 of the best possible. With no more problems than streams every problem has its own.
inline std::vector<size_t> assign_longest_first(const std::vector<size_t>& cost, size_t P) {
  const size_t n = cost.size();
  std::vector<size_t> owner(n, 0);
  if (P == 0 || n == 0) return owner;
  std::vector<size_t> order(n);
  for (size_t i = 0; i < n; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return cost[a] > cost[b]; });
  std::vector<size_t> load(P, 0);
  for (size_t i : order) {
    const size_t w = (size_t)(std::min_element(load.begin(), load.end()) - load.begin());
    owner[i] = w;
    load[w] += cost[i];
  }
  return owner;
}

}  // namespace pdt
