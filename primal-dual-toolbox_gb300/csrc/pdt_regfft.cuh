// pdt_regfft.cuh -- FFTs of compile-time length held in one thread's registers, and the two-level
// (four-step) decomposition that spreads a longer transform over a group of threads.
//
// reg_fft<N, TS>(x, tw, s): in-place DFT of x[0..N) with sign s (-1 forward, +1 inverse), natural order
// in and out. Twiddles come from a shared-memory table tw[t] = exp(-2 pi i t / L) of some length L; TS
// = L / N is the table stride of w_N, so every table index is a compile-time constant after unrolling.
// N = P * Q is split decimation-in-time:
//   X[k1 + Q k2] = sum_p w_P^(p k2) w_N^(p k1) Y_p[k1],   Y_p = DFT_Q(x[p + P q])
// with P = 4, 2 or the smallest odd prime; primes above 5 use the symmetric direct DFT
//   X[k], X[P-k] = x0 + sum_j (x_j + x_{P-j}) cos(2 pi jk/P)  +-  s i sum_j (x_j - x_{P-j}) sin(2 pi jk/P).
#pragma once

#include "pdt_device.cuh"

namespace pdt {

constexpr int ct_smallest_odd_factor(int n, int f = 3) { return f * f > n ? n : (n % f == 0 ? f : ct_smallest_odd_factor(n, f + 2)); }
constexpr int ct_split(int n) { return n % 4 == 0 && n != 4 && n != 8 ? 4 : (n % 2 == 0 && n != 2 ? 2 : ct_smallest_odd_factor(n)); }
constexpr bool ct_is_base(int n) { return n == 1 || n == 2 || n == 3 || n == 4 || n == 5 || n == 8; }

template <int N, int TS>
__device__ __forceinline__ void reg_fft(float2 (&x)[N], const float2* __restrict__ tw, float s);

// Symmetric direct DFT of odd prime length P (> 5). Roots w_P^m = tw[m * TS].
template <int P, int TS>
__device__ __forceinline__ void dft_prime(float2 (&x)[P], const float2* __restrict__ tw, float s) {
  constexpr int Hh = (P - 1) / 2;
  float cs[Hh], sn[Hh];
#pragma unroll
  for (int m = 1; m <= Hh; ++m) {
    const float2 w = tw[m * TS];  // (cos, -sin) of 2 pi m / P
    cs[m - 1] = w.x;
    sn[m - 1] = -w.y;
  }
  float2 t[Hh], d[Hh];
  float2 x0 = x[0];
  float2 sum = x0;
#pragma unroll
  for (int j = 1; j <= Hh; ++j) {
    t[j - 1] = x[j] + x[P - j];
    d[j - 1] = x[j] - x[P - j];
    sum += t[j - 1];
  }
  x[0] = sum;
#pragma unroll
  for (int k = 1; k <= Hh; ++k) {
    float2 A = x0, B = c2(0.f, 0.f);
#pragma unroll
    for (int j = 1; j <= Hh; ++j) {
      const int m = (j * k) % P;
      const float cv = m <= Hh ? cs[m - 1] : cs[P - m - 1];
      const float sv = m <= Hh ? sn[m - 1] : -sn[P - m - 1];
      A.x = fmaf(cv, t[j - 1].x, A.x);
      A.y = fmaf(cv, t[j - 1].y, A.y);
      B.x = fmaf(sv, d[j - 1].x, B.x);
      B.y = fmaf(sv, d[j - 1].y, B.y);
    }
    const float2 jb = mul_si(B, s);
    x[k] = A + jb;
    x[P - k] = A - jb;
  }
}

template <int N, int TS>
__device__ __forceinline__ void reg_fft(float2 (&x)[N], const float2* __restrict__ tw, float s) {
  if constexpr (N == 1) {
    return;
  } else if constexpr (N == 2) {
    dft2(x[0], x[1]);
  } else if constexpr (N == 3) {
    dft3(x, s);
  } else if constexpr (N == 4) {
    dft4(x[0], x[1], x[2], x[3], s);
  } else if constexpr (N == 5) {
    dft5(x, s);
  } else if constexpr (N == 8) {
    dft8(x, s);
  } else if constexpr (ct_split(N) == N) {
    dft_prime<N, TS>(x, tw, s);
  } else {
    constexpr int P = ct_split(N);
    constexpr int Q = N / P;
    float2 y[P][Q];
#pragma unroll
    for (int p = 0; p < P; ++p)
#pragma unroll
      for (int q = 0; q < Q; ++q) y[p][q] = x[p + P * q];
#pragma unroll
    for (int p = 0; p < P; ++p) reg_fft<Q, TS * P>(y[p], tw, s);
#pragma unroll
    for (int p = 1; p < P; ++p)
#pragma unroll
      for (int k1 = 1; k1 < Q; ++k1) {
        float2 w = tw[((p * k1) % N) * TS];
        w.y *= -s;
        y[p][k1] = cmul(y[p][k1], w);
      }
#pragma unroll
    for (int k1 = 0; k1 < Q; ++k1) {
      float2 z[P];
#pragma unroll
      for (int p = 0; p < P; ++p) z[p] = y[p][k1];
      reg_fft<P, TS * Q>(z, tw, s);
#pragma unroll
      for (int k2 = 0; k2 < P; ++k2) x[k1 + Q * k2] = z[k2];
    }
  }
}

// ------------------------------------------------------------------------------------------------
// Two-level transform of length n = A * B over a thread group (four-step / Bailey):
//   step 1  thread a < A holds x[a + A b] (b < B):  B-point FFT, times w_n^(a kb)  -> smem Y[kb][a]
//   step 2  thread kb < B holds Y[kb][a] (a < A):   A-point FFT -> X[kb + B ka]
// and the inverse runs the same steps backwards from the registers step 2 leaves.
// The shared-memory exchange buffer of one sequence holds B * (A + 1) elements (the +1 spreads banks).
// ------------------------------------------------------------------------------------------------
template <int A, int B>
struct TwoLevel {
  static constexpr int n = A * B;
  static constexpr int ldx = A + 1;  // exchange row stride
  static constexpr int xch = B * ldx;

  // Forward step 1 for thread a: v[b] = x[a + A b] on entry, leaves Y[kb][a] (twiddled) in smem.
  static __device__ __forceinline__ void fwd_step1(float2 (&v)[B], int a, float2* __restrict__ ex,
                                                   const float2* __restrict__ tw) {
    reg_fft<B, A>(v, tw, -1.f);
#pragma unroll
    for (int kb = 0; kb < B; ++kb) {
      const float2 w = tw[(a * kb) % n];
      ex[kb * ldx + a] = kb ? cmul(v[kb], w) : v[kb];
    }
  }
  // Forward step 2 for thread kb: u[ka] = X[kb + B ka] on exit.
  static __device__ __forceinline__ void fwd_step2(float2 (&u)[A], int kb, const float2* __restrict__ ex,
                                                   const float2* __restrict__ tw) {
#pragma unroll
    for (int a = 0; a < A; ++a) u[a] = ex[kb * ldx + a];
    reg_fft<A, B>(u, tw, -1.f);
  }
  // Inverse step 1 for thread kb: u[ka] = Z[kb + B ka] on entry; leaves V[kb][a] (twiddled) in smem.
  static __device__ __forceinline__ void inv_step1(float2 (&u)[A], int kb, float2* __restrict__ ex,
                                                   const float2* __restrict__ tw) {
    reg_fft<A, B>(u, tw, 1.f);
#pragma unroll
    for (int a = 0; a < A; ++a) {
      const float2 w = conjf2(tw[(a * kb) % n]);
      ex[kb * ldx + a] = (a && kb) ? cmul(u[a], w) : u[a];
    }
  }
  // Inverse step 2 for thread a: v[b] = z[a + A b] on exit (unscaled).
  static __device__ __forceinline__ void inv_step2(float2 (&v)[B], int a, const float2* __restrict__ ex,
                                                   const float2* __restrict__ tw) {
#pragma unroll
    for (int kb = 0; kb < B; ++kb) v[kb] = ex[kb * ldx + a];
    reg_fft<B, A>(v, tw, 1.f);
  }
};


// ------------------------------------------------------------------------------------------------
// Lane-distributed transform of length n = M * L over a group of L lanes (L = 8, 16, 32):
// lane t holds x[t + L j] (j < M) in registers. The forward transform is an M-point register FFT per
// lane, a twiddle w_n^(t k1), and an L-point FFT across the lanes (radix-2 decimation in frequency, one
// __shfl_xor_sync butterfly per stage and value):
//   X[k1 + M k2] = sum_t w_L^(t k2) w_n^(t k1) sum_j w_M^(j k1) x[t + L j]
// leaving X[k1 + M brev_L(t)] in register k1 of lane t. The inverse runs the same network backwards
// (decimation in time) with conjugate twiddles, from that order back to natural order. Every lane
// works in every stage and no shared-memory exchange is needed. All 32 lanes of a warp must call it.
// ------------------------------------------------------------------------------------------------
constexpr int ct_log2(int n) { return n <= 1 ? 0 : 1 + ct_log2(n / 2); }

#ifndef PDT_HOST_EMULATION
__device__ __forceinline__ float2 shfl_xor2(float2 v, int m) {
  return c2(__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m));
}

// bit reversal of t over log2(L) bits
template <int L>
__device__ __forceinline__ int lane_brev(int t) {
  return (int)(__brev((unsigned)t) >> (32 - ct_log2(L)));
}
#else
// host build of the layout tests: the exchange between lanes and the 64-thread barrier are supplied by
// the test harness, which runs one host thread per lane
float2 shfl_xor2(float2 v, int m);
void emu_sync64(int bar_id);

template <int L>
inline int lane_brev(int t) {
  int r = 0;
  for (int b = 0; b < ct_log2(L); ++b) r |= ((t >> b) & 1) << (ct_log2(L) - 1 - b);
  return r;
}
#endif

template <int M, int L>
struct LaneFft {
  static_assert(L == 8 || L == 16 || L == 32, "lanes per sequence");
  static constexpr int n = M * L;

  // Forward: v[j] = x[t + L j] on entry; v[k1] = X[k1 + M brev_L(t)] on exit. tw[i] = exp(-2 pi i i / n).
  static __device__ __forceinline__ void fwd(float2 (&v)[M], int t, const float2* __restrict__ tw) {
    reg_fft<M, L>(v, tw, -1.f);
#pragma unroll
    for (int k1 = 1; k1 < M; ++k1) v[k1] = cmul(v[k1], tw[t * k1]);  // t k1 < n
    // stage h: the lower lane of a pair keeps a + b, the upper (p - v) w_2h^(t mod h); the last stage
    // (h = 1) has no twiddle
#pragma unroll
    for (int h = L / 2; h >= 1; h >>= 1) {
      const bool up = (t & h) != 0;
      const float sg = up ? -1.f : 1.f;
      float2 w = c2(1.f, 0.f);
      if (h > 1 && up) w = tw[(t & (h - 1)) * (n / (2 * h))];
#pragma unroll
      for (int k1 = 0; k1 < M; ++k1) {
        const float2 p = shfl_xor2(v[k1], h);
        const float2 y = c2(fmaf(sg, v[k1].x, p.x), fmaf(sg, v[k1].y, p.y));
        v[k1] = (h > 1) ? cmul(y, w) : y;
      }
    }
  }

  // Unnormalised inverse: v[k1] = Z[k1 + M brev_L(t)] on entry; v[j] = n z[t + L j] on exit.
  static __device__ __forceinline__ void inv(float2 (&v)[M], int t, const float2* __restrict__ tw) {
#pragma unroll
    for (int h = 1; h < L; h <<= 1) {
      const bool up = (t & h) != 0;
      const float sg = up ? -1.f : 1.f;
      float2 w = c2(1.f, 0.f);
      if (h > 1 && up) w = conjf2(tw[(t & (h - 1)) * (n / (2 * h))]);
#pragma unroll
      for (int k1 = 0; k1 < M; ++k1) {
        const float2 m = (h > 1) ? cmul(v[k1], w) : v[k1];
        const float2 p = shfl_xor2(m, h);
        v[k1] = c2(fmaf(sg, m.x, p.x), fmaf(sg, m.y, p.y));  // lower m + p, upper p - m
      }
    }
#pragma unroll
    for (int k1 = 1; k1 < M; ++k1) v[k1] = cmul(v[k1], conjf2(tw[t * k1]));
    reg_fft<M, L>(v, tw, 1.f);
  }
};

// The same transform over two warps (n = M * 64): lanes 0-31 of the first warp and 32-63 of the second
// hold the sequence. The stage that pairs lane t with t ^ 32 goes through the shared-memory buffer xbuf
// (M x 64 values) between two syncs of the named barrier bar_id (64 threads); the others are shuffles.
// Both warps must call it.
template <int M>
struct LaneFft64 {
  static constexpr int L = 64;
  static constexpr int n = M * L;

  static __device__ __forceinline__ void sync64(int bar_id) {
#ifndef PDT_HOST_EMULATION
    asm volatile("bar.sync %0, 64;" ::"r"(bar_id) : "memory");
#else
    emu_sync64(bar_id);
#endif
  }

  static __device__ __forceinline__ void fwd(float2 (&v)[M], int t, const float2* __restrict__ tw, float2* xbuf,
                                             int bar_id) {
    reg_fft<M, L>(v, tw, -1.f);
#pragma unroll
    for (int k1 = 1; k1 < M; ++k1) v[k1] = cmul(v[k1], tw[t * k1]);
    {  // h = 32: across the two warps
      const bool up = (t & 32) != 0;
      const float sg = up ? -1.f : 1.f;
      const float2 w = up ? tw[(t & 31) * (n / 64)] : c2(1.f, 0.f);
#pragma unroll
      for (int k1 = 0; k1 < M; ++k1) xbuf[k1 * 64 + t] = v[k1];
      sync64(bar_id);
#pragma unroll
      for (int k1 = 0; k1 < M; ++k1) {
        const float2 p = xbuf[k1 * 64 + (t ^ 32)];
        v[k1] = cmul(c2(fmaf(sg, v[k1].x, p.x), fmaf(sg, v[k1].y, p.y)), w);
      }
      sync64(bar_id);  // xbuf free again
    }
#pragma unroll
    for (int h = 16; h >= 1; h >>= 1) {
      const bool up = (t & h) != 0;
      const float sg = up ? -1.f : 1.f;
      float2 w = c2(1.f, 0.f);
      if (h > 1 && up) w = tw[(t & (h - 1)) * (n / (2 * h))];
#pragma unroll
      for (int k1 = 0; k1 < M; ++k1) {
        const float2 p = shfl_xor2(v[k1], h);
        const float2 y = c2(fmaf(sg, v[k1].x, p.x), fmaf(sg, v[k1].y, p.y));
        v[k1] = (h > 1) ? cmul(y, w) : y;
      }
    }
  }

  static __device__ __forceinline__ void inv(float2 (&v)[M], int t, const float2* __restrict__ tw, float2* xbuf,
                                             int bar_id) {
#pragma unroll
    for (int h = 1; h < 32; h <<= 1) {
      const bool up = (t & h) != 0;
      const float sg = up ? -1.f : 1.f;
      float2 w = c2(1.f, 0.f);
      if (h > 1 && up) w = conjf2(tw[(t & (h - 1)) * (n / (2 * h))]);
#pragma unroll
      for (int k1 = 0; k1 < M; ++k1) {
        const float2 m = (h > 1) ? cmul(v[k1], w) : v[k1];
        const float2 p = shfl_xor2(m, h);
        v[k1] = c2(fmaf(sg, m.x, p.x), fmaf(sg, m.y, p.y));
      }
    }
    {  // h = 32: across the two warps
      const bool up = (t & 32) != 0;
      const float sg = up ? -1.f : 1.f;
      const float2 w = up ? conjf2(tw[(t & 31) * (n / 64)]) : c2(1.f, 0.f);
#pragma unroll
      for (int k1 = 0; k1 < M; ++k1) {
        v[k1] = cmul(v[k1], w);
        xbuf[k1 * 64 + t] = v[k1];
      }
      sync64(bar_id);
#pragma unroll
      for (int k1 = 0; k1 < M; ++k1) {
        const float2 p = xbuf[k1 * 64 + (t ^ 32)];
        v[k1] = c2(fmaf(sg, v[k1].x, p.x), fmaf(sg, v[k1].y, p.y));
      }
      sync64(bar_id);
    }
#pragma unroll
    for (int k1 = 1; k1 < M; ++k1) v[k1] = cmul(v[k1], conjf2(tw[t * k1]));
    reg_fft<M, L>(v, tw, 1.f);
  }
};


}  // namespace pdt
