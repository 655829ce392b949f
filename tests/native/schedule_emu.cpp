// Host build of the batch's stream assignment (pdt_schedule.h) for the scheduling tests.
#include <cstring>

#include "../../primal-dual-toolbox_gb300/csrc/pdt_schedule.h"

extern "C" {

// owner[i] = worker stream of problem i (n problems with the given costs, P streams).
void emu_assign(const unsigned long long* cost, int n, int P, unsigned long long* owner) {
  std::vector<size_t> c(cost, cost + n);
  const std::vector<size_t> o = pdt::assign_longest_first(c, (size_t)P);
  for (int i = 0; i < n; ++i) owner[i] = o[i];
}
}
