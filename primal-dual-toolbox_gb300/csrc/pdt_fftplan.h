// pdt_fftplan.h -- host-side FFT planning: radix factorisation and twiddle table for the device FFT.
#pragma once

#include <cmath>

namespace pdt {

// Factorise n into radices: 8s first, then one 4 or 2, then 3, 5 and other odd primes. Returns false if
// n < 1 or the plan would exceed kMaxStages.
inline bool make_fft_plan(int n, FftPlan* pl) {
  if (n < 1) return false;
  pl->n = n;
  pl->nst = 0;
  int m = n;
  auto push = [&](int r) {
    if (pl->nst >= kMaxStages) return false;
    pl->radix[pl->nst++] = r;
    m /= r;
    return true;
  };
  while (m % 8 == 0)
    if (!push(8)) return false;
  if (m % 4 == 0 && !push(4)) return false;
  if (m % 2 == 0 && !push(2)) return false;
  for (int f = 3; m > 1; f += 2)
    while (m % f == 0)
      if (!push(f)) return false;
  return true;
}

// tw[t] = exp(-2 pi i t / n), evaluated in double and rounded to float.
inline void fill_twiddles(int n, float2* tw) {
  const double two_pi = 6.283185307179586476925286766559;
  for (int t = 0; t < n; ++t) {
    const double a = -two_pi * (double)t / (double)n;
    tw[t] = make_float2((float)std::cos(a), (float)std::sin(a));
  }
}

}  // namespace pdt
