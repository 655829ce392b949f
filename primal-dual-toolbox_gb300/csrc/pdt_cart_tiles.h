// pdt_cart_tiles.h -- host construction of the tensor-core row passes' DFT-factor operand tiles (plain
// C++, no CUDA: also compiled for the host-side layout tests).
//
// The adjoint rows compute g_c[y][x] = sum_s t2[c][s][y] exp(+2 pi i p_s q(x) / W), with p_s the
// inverse-FFT input slot of sampled column s, p_s = (col_x[s] + mxW) mod W, and q(x) = (x - oxW) mod W
// (mxW = int((W+1)/2), oxW = W/2: the ifftshift / fftshift mids). As a real GEMM D = A B the data operand
// A interleaves re/im along K (k = 2 s + ri) and the factor B expands each complex entry e into the 2 x 2
// block [[Re e, -Im e], [Im e, Re e]] along (N, K): B row n = 2 x + o gives part o (re/im) of output x.
//
// Table layout, the order tc_rows_adj copies it in: [range i][K chunk j][hi rows | lo rows], a range of
// NB rows n (output columns 2 x + o, the last range holding nb = min(NB, round16(2 W - n0)) rows), a K chunk
// 32 elements (16 sampled columns), each row 32 floats = 128 bytes whose 16-byte chunks are swizzled
// (chunk c of row n stored at c ^ (n mod 8)), TF32 hi = tf32(v) and lo = tf32(v - hi). Entries outside
// the matrix (x >= W, s >= ns) are zero.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace pdt {

// v rounded to TF32 (10 explicit mantissa bits, ties away from zero): the host side of split_tf32
inline float tc_host_tf32(float v) {
  uint32_t u;
  std::memcpy(&u, &v, 4);
  u = (u + 0x1000u) & 0xFFFFE000u;
  std::memcpy(&v, &u, 4);
  return v;
}

// cos (which = 0) or sin (which = 1) of 2 pi m / n for m < n, in double precision
inline std::vector<double> host_roots(int n, int which) {
  const double two_pi = 6.283185307179586476925286766559;
  std::vector<double> r(n);
  for (int m = 0; m < n; ++m) r[m] = which ? std::sin(two_pi * m / n) : std::cos(two_pi * m / n);
  return r;
}

inline int tc_adj_chunk_count(int ns) { return (2 * ns + 31) / 32; }

// The table above for output-column ranges of NB rows (NB a multiple of 16); `h` is resized and filled.
inline void build_tc_adj_table(int W, int ns, const int* col_x, int mxW, int oxW, int NB, std::vector<float>& h) {
  const int nch = tc_adj_chunk_count(ns), nranges = (2 * W + NB - 1) / NB;
  h.assign((size_t)nranges * nch * 2 * NB * 32, 0.f);
  std::vector<float> wc(W), ws(W);  // cos, sin of 2 pi m / W, rounded from double
  {
    const std::vector<double> c = host_roots(W, 0), sn = host_roots(W, 1);
    for (int m = 0; m < W; ++m) wc[m] = (float)c[m], ws[m] = (float)sn[m];
  }
  // along a tile row x advances by one, so the root index p_s q(x) mod W advances by p_s
  for (int i = 0; i < nranges; ++i) {
    const int n0 = i * NB, nb = std::min(NB, (2 * W - n0 + 15) & ~15);
    const int x0 = n0 >> 1, x1 = std::min(W, (n0 + nb) >> 1);
    const int q0 = ((x0 - oxW) % W + W) % W;
    for (int j = 0; j < nch; ++j) {
      float* hi = &h[((size_t)i * nch + j) * 2 * NB * 32];
      float* lo = hi + (size_t)nb * 32;
      const int kn = std::min(16, ns - 16 * j);  // sampled columns of this K chunk
      int m[16], p[16];
      for (int kk = 0; kk < kn; ++kk) {
        p[kk] = (col_x[16 * j + kk] + mxW) % W;
        m[kk] = (int)(((long long)p[kk] * q0) % W);
      }
      for (int x = x0; x < x1; ++x) {
        const int n = 2 * (x - x0);
        for (int o = 0; o < 2; ++o) {
          float* hr = hi + (size_t)(n + o) * 32;
          float* lr = lo + (size_t)(n + o) * 32;
          const int sw = (n + o) & 7;
          for (int kk = 0; kk < kn; ++kk) {
            const float er = wc[m[kk]], ei = ws[m[kk]];
            const float v0 = o == 0 ? er : ei, v1 = o == 0 ? -ei : er;
            const int k0 = 2 * kk, k1 = k0 + 1;
            const int a0 = (((k0 >> 2) ^ sw) << 2) + (k0 & 3), a1 = (((k1 >> 2) ^ sw) << 2) + (k1 & 3);
            hr[a0] = tc_host_tf32(v0);
            lr[a0] = tc_host_tf32(v0 - hr[a0]);
            hr[a1] = tc_host_tf32(v1);
            lr[a1] = tc_host_tf32(v1 - hr[a1]);
          }
        }
        for (int kk = 0; kk < kn; ++kk) {
          m[kk] += p[kk];
          if (m[kk] >= W) m[kk] -= W;
        }
      }
    }
  }
}

// The forward rows' factor for tc_rows_fwd: t1[c][s][y] = sum_x (ubar . sens_c)[y][x] w^(q(x) f_s) with
// w = exp(-2 pi i / W), q(x) = (x + mxW) mod W the ifftshift slot of image column x and f_s = (col_x[s] - oxW)
// mod W the forward-FFT output slot of sampled column s. Layout: [s tile z of 128 sampled columns][K chunk
// j of 16 image columns][hi rows | lo rows], chunk stride 2 nbmax 32 floats with nbmax = round16(2 min(128,
// ns)); row n = 2 sl + o (output s = 128 z + sl, re/im part o; a tile's nb = round16(2 nsl) rows), K element
// k = 2 (x - 16 j) + (re/im input), the same 2 x 2 blocks, swizzle and split as the adjoint table.
inline int tc_fwd_rows_max(int ns) { return (2 * std::min(128, ns) + 15) & ~15; }

inline void build_tc_fwd_table(int W, int ns, const int* col_x, int mxW, int oxW, std::vector<float>& h) {
  const int nchT = (2 * W + 31) / 32, stiles = (ns + 127) / 128;
  const int nbmax = tc_fwd_rows_max(ns);
  h.assign((size_t)stiles * nchT * 2 * nbmax * 32, 0.f);
  const std::vector<double> wc = host_roots(W, 0), ws = host_roots(W, 1);  // cos, sin of 2 pi m / W
  for (int z = 0; z < stiles; ++z) {
    const int nsl = std::min(128, ns - 128 * z), nb = (2 * nsl + 15) & ~15;
    for (int j = 0; j < nchT; ++j) {
      float* hi = &h[((size_t)z * nchT + j) * 2 * nbmax * 32];
      float* lo = hi + (size_t)nb * 32;
      for (int n = 0; n < 2 * nsl; ++n) {
        const int s = 128 * z + (n >> 1), o = n & 1;
        const int f = ((col_x[s] - oxW) % W + W) % W;  // forward-FFT output slot of s
        for (int k = 0; k < 32; ++k) {
          const int x = 16 * j + (k >> 1), ri = k & 1;
          if (x >= W) continue;
          const int q = (x + mxW) % W;  // ifftshift slot of image column x
          const int m = (int)(((long long)q * f) % W);
          const float er = (float)wc[m], ei = -(float)ws[m];  // w^(q f) = exp(-2 pi i m / W)
          const float v = o == 0 ? (ri == 0 ? er : -ei) : (ri == 0 ? ei : er);
          const int pos = n * 32 + (((k >> 2) ^ (n & 7)) << 2) + (k & 3);
          hi[pos] = tc_host_tf32(v);
          lo[pos] = tc_host_tf32(v - hi[pos]);
        }
      }
    }
  }
}

}  // namespace pdt
