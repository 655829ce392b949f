// Host build of the tensor-core row passes' DFT-factor tables (pdt_cart_tiles.h) for the layout tests.
#include "../../primal-dual-toolbox_gb300/csrc/pdt_cart_tiles.h"

extern "C" {

// Fills out[0 .. n) with the table for the given geometry; returns its length in floats, or -1 if n is
// too small.
long long emu_adj_table(int W, int ns, const int* col_x, int NB, float* out, long long n) {
  std::vector<float> h;
  pdt::build_tc_adj_table(W, ns, col_x, (W + 1) / 2, W / 2, NB, h);
  if ((long long)h.size() > n) return -1;
  std::memcpy(out, h.data(), h.size() * sizeof(float));
  return (long long)h.size();
}

// The same for the forward rows' table.
long long emu_fwd_table(int W, int ns, const int* col_x, float* out, long long n) {
  std::vector<float> h;
  pdt::build_tc_fwd_table(W, ns, col_x, (W + 1) / 2, W / 2, h);
  if ((long long)h.size() > n) return -1;
  std::memcpy(out, h.data(), h.size() * sizeof(float));
  return (long long)h.size();
}

// The roots the tables are built from: cos (which = 0) or sin (which = 1) of 2 pi m / n.
void emu_roots(int n, int which, double* out) {
  const std::vector<double> r = pdt::host_roots(n, which);
  std::memcpy(out, r.data(), r.size() * sizeof(double));
}
}
