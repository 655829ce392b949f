// pdt_cart_fast.cuh -- register-FFT kernels of the Cartesian operator for even W and H with a
// compile-time two-level split (W = A * B, A, B <= 32). One warp owns one sequence (an image row or a
// k-space column): lanes < A run the first-level B-point FFTs in registers, lanes < B the second-level
// A-point FFTs, exchanging once through the warp's own shared-memory tile. The column kernel runs
// forward FFT, mask, k-space dual prox and inverse FFT with two exchanges, because the inverse starts
// from the registers the forward leaves (the shifts cancel for even H: slot k of the forward output is
// slot k of the inverse input). Included by pdt_cartesian.cu after CartDev.
#pragma once

#include <cooperative_groups.h>

#include "pdt_regfft.cuh"

namespace cg = cooperative_groups;

namespace pdt {
namespace {

constexpr int kMaxWarps = 8;  // largest warps-per-block instance (one sequence per warp)

// Phase 1 (fast): rows of ubar . sens_c -> FFT along W -> sampled columns t1[c][s][yi].
template <int A, int B, int WPB>
__global__ void __launch_bounds__(32 * WPB) fr_rows_fwd(CartDev d, const float2* __restrict__ ubar,
                                                               float2* __restrict__ t1, int* __restrict__ tick) {
  using TL = TwoLevel<A, B>;
  extern __shared__ float2 sm[];
  float2* tw = sm;
  float2* ex = tw + TL::n;
  float2* stage = ex + WPB * TL::xch;
  int* fs2s = reinterpret_cast<int*>(stage + (size_t)d.ns * WPB);
  if (tick && blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) atomicAdd(tick, 1);
  for (int i = threadIdx.x; i < TL::n; i += blockDim.x) {
    tw[i] = d.twW[i];
    fs2s[i] = d.fslot2s[i];
  }
  __syncthreads();
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int yi0 = blockIdx.x * WPB, yi = yi0 + w, c = blockIdx.y;
  float2* myex = ex + w * TL::xch;
  const bool ok = yi < d.Hi;
  if (ok && lane < A) {
    float2 v[B];
    const float2* urow = ubar + (size_t)yi * TL::n;
    const float2* srow = d.sens ? d.sens + ((size_t)c * d.Hf + yi + d.y0) * TL::n : nullptr;
#pragma unroll
    for (int b = 0; b < B; ++b) {
      int x = lane + A * b - d.mxW;  // FFT slot j holds image column (j - mid) mod W
      if (x < 0) x += TL::n;
      float2 val = urow[x];
      if (srow) val = cmul(val, srow[x]);
      v[b] = val;
    }
    TL::fwd_step1(v, lane, myex, tw);
  }
  __syncwarp();
  if (ok && lane < B) {
    float2 u[A];
    TL::fwd_step2(u, lane, myex, tw);
#pragma unroll
    for (int ka = 0; ka < A; ++ka) {
      const int s = fs2s[lane + B * ka];
      if (s >= 0) stage[s * WPB + w] = u[ka];
    }
  }
  __syncthreads();
  const int nr = min(WPB, d.Hi - yi0);
  for (int i = threadIdx.x; i < d.ns * nr; i += blockDim.x) {
    const int s = i / nr, r = i - s * nr;
    t1[((size_t)c * d.ns + s) * d.Hi + yi0 + r] = stage[s * WPB + r];
  }
}

// Phase 2 (fast): per sampled column, FFT along H -> mask -> (prox) -> mask -> IFFT along H.
template <int A, int B, int WPB>
__global__ void __launch_bounds__(32 * WPB) fr_cols(CartDev d, int mode, const float2* t_in, float2* t_out,
                                                           float2* __restrict__ r, const float2* __restrict__ fc,
                                                           const float2* __restrict__ kin, float2* __restrict__ kout,
                                                           float sigma, float lambda) {
  using TL = TwoLevel<A, B>;
  extern __shared__ float2 sm[];
  float2* tw = sm;
  float2* ex = tw + TL::n;
  for (int i = threadIdx.x; i < TL::n; i += blockDim.x) tw[i] = d.twH[i];
  __syncthreads();
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int s = blockIdx.x * WPB + w, c = blockIdx.y;
  const bool ok = s < d.ns;
  float2* myex = ex + w * TL::xch;
  constexpr int Hf = TL::n;
  const size_t colc = ((size_t)c * d.ns + s);
  float2 u[A];
  if (mode == COL_SOLVE || mode == COL_FWD_DENSE) {
    if (ok && lane < A) {
      float2 v[B];
#pragma unroll
      for (int b = 0; b < B; ++b) {
        int yf = lane + A * b - d.mxH;
        if (yf < 0) yf += Hf;
        const int yi = yf - d.y0;
        v[b] = (yi >= 0 && yi < d.Hi) ? t_in[colc * d.Hi + yi] : c2(0.f, 0.f);
      }
      TL::fwd_step1(v, lane, myex, tw);
    }
    __syncwarp();
    if (ok && lane < B) {
      TL::fwd_step2(u, lane, myex, tw);
      const float* mrow = d.maskc + (size_t)s * Hf;
      // chunks of loads -> math -> stores: r is read and written in place, so the compiler cannot hoist
      // a later load above an earlier store; batching keeps CH loads in flight per lane
      constexpr int CH = A < 8 ? A : 8;
#pragma unroll
      for (int k0 = 0; k0 < A; k0 += CH) {
        int yp[CH];
        float m[CH];
        float2 fv[CH], rv[CH];
#pragma unroll
        for (int q = 0; q < CH; ++q) {
          int ypos = lane + B * (k0 + q) + d.oyH;
          if (ypos >= Hf) ypos -= Hf;
          yp[q] = ypos;
          m[q] = mrow[ypos];
        }
        if (mode == COL_FWD_DENSE) {
#pragma unroll
          for (int q = 0; q < CH; ++q)
            kout[((size_t)c * Hf + yp[q]) * d.W + d.col_x[s]] = u[k0 + q] * (d.scale * m[q]);
        } else {
#pragma unroll
          for (int q = 0; q < CH; ++q) {
            fv[q] = fc[colc * Hf + yp[q]];
            rv[q] = r[colc * Hf + yp[q]];
          }
#pragma unroll
          for (int q = 0; q < CH; ++q) {
            const float2 kv = u[k0 + q] * (d.scale * m[q]);
            rv[q] = (rv[q] + sigma * (kv - fv[q])) / (1.0f + sigma * lambda);
            u[k0 + q] = rv[q] * m[q];
          }
#pragma unroll
          for (int q = 0; q < CH; ++q) r[colc * Hf + yp[q]] = rv[q];
        }
      }
    }
    if (mode == COL_FWD_DENSE) return;
    __syncwarp();
  } else if (ok && lane < B) {
    const float* mrow = d.maskc + (size_t)s * Hf;
#pragma unroll
    for (int ka = 0; ka < A; ++ka) {
      int ypos = lane + B * ka + d.oyH;
      if (ypos >= Hf) ypos -= Hf;
      const float2 v = (mode == COL_ADJ_DENSE) ? kin[((size_t)c * Hf + ypos) * d.W + d.col_x[s]] : fc[colc * Hf + ypos];
      u[ka] = v * mrow[ypos];
    }
  }
  if (ok && lane < B) TL::inv_step1(u, lane, myex, tw);
  __syncwarp();
  if (ok && lane < A) {
    float2 v[B];
    TL::inv_step2(v, lane, myex, tw);
#pragma unroll
    for (int b = 0; b < B; ++b) {
      int yf = lane + A * b + d.oyH;
      if (yf >= Hf) yf -= Hf;
      const int yi = yf - d.y0;
      if (yi >= 0 && yi < d.Hi) t_out[colc * d.Hi + yi] = v[b] * d.scale;
    }
  }
}

// Phase 3 (fast): per image row block, IFFT along W of the sampled columns, conj(sens_c) multiply and
// the coil sum. A cluster of G blocks shares the row block, each block taking one coil group and
// accumulating in its shared memory; the blocks then reduce the G partial rows through distributed
// shared memory in rank order (deterministic) and write one K^H r plane. With G = 1 it is a plain launch.
template <int A, int B, int WPB>
__global__ void __launch_bounds__(32 * WPB) fr_rows_adj(CartDev d, const float2* __restrict__ t2,
                                                        float2* __restrict__ out, int use_cluster, int G,
                                                        long long gstride) {
  using TL = TwoLevel<A, B>;
  constexpr int W = TL::n;
  extern __shared__ float2 sm[];
  float2* tw = sm;
  float2* ex = tw + W;
  float2* stage = ex + WPB * TL::xch;
  float2* red = stage + (size_t)d.ns * WPB;  // WPB rows x W: this block's coil-group sum
  int* as2s = reinterpret_cast<int*>(red + (size_t)WPB * W);
  // with use_cluster, the G coil groups of a row block form a cluster (grid.y = G); otherwise each
  // block writes its group's partial sum to out + g * gstride
  const int g = blockIdx.y;
  for (int i = threadIdx.x; i < W; i += blockDim.x) {
    tw[i] = d.twW[i];
    as2s[i] = d.slot2s[i];
  }
  for (int i = threadIdx.x; i < WPB * W; i += blockDim.x) red[i] = c2(0.f, 0.f);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int yi0 = blockIdx.x * WPB, yi = yi0 + w;
  const int nr = min(WPB, d.Hi - yi0);
  const int c_begin = (int)((long long)g * d.C / G), c_end = (int)((long long)(g + 1) * d.C / G);
  float2* myex = ex + w * TL::xch;
  const bool ok = w < nr;
  // prefetch of the next coil's sampled columns (ns * nr values spread over the block)
  constexpr int PF = 8;
  float2 pf[PF];
  auto fetch = [&](int c) {
#pragma unroll
    for (int q = 0; q < PF; ++q) {
      const int i = threadIdx.x + q * (int)blockDim.x;
      if (i < d.ns * nr) {
        const int s = i / nr, rr = i - s * nr;
        pf[q] = t2[((size_t)c * d.ns + s) * d.Hi + yi0 + rr];
      }
    }
  };
  const bool pf_all = d.ns * nr <= PF * (int)blockDim.x;
  if (c_begin < c_end && pf_all) fetch(c_begin);
  for (int c = c_begin; c < c_end; ++c) {
    __syncthreads();  // stage free (and, first time, tables and red ready)
    if (pf_all) {
#pragma unroll
      for (int q = 0; q < PF; ++q) {
        const int i = threadIdx.x + q * (int)blockDim.x;
        if (i < d.ns * nr) {
          const int s = i / nr, rr = i - s * nr;
          stage[s * WPB + rr] = pf[q];
        }
      }
      if (c + 1 < c_end) fetch(c + 1);
    } else {
      for (int i = threadIdx.x; i < d.ns * nr; i += blockDim.x) {
        const int s = i / nr, rr = i - s * nr;
        stage[s * WPB + rr] = t2[((size_t)c * d.ns + s) * d.Hi + yi0 + rr];
      }
    }
    __syncthreads();
    if (ok && lane < B) {
      float2 u[A];
#pragma unroll
      for (int ka = 0; ka < A; ++ka) {
        const int s = as2s[lane + B * ka];
        u[ka] = s >= 0 ? stage[s * WPB + w] : c2(0.f, 0.f);
      }
      TL::inv_step1(u, lane, myex, tw);
    }
    __syncwarp();
    if (ok && lane < A) {
      float2 v[B];
      TL::inv_step2(v, lane, myex, tw);
      const float2* srow = d.sens ? d.sens + ((size_t)c * d.Hf + yi + d.y0) * W : nullptr;
      float2* rrow = red + (size_t)w * W;
#pragma unroll
      for (int b = 0; b < B; ++b) {
        int x = lane + A * b + d.oxW;
        if (x >= W) x -= W;
        rrow[x] += srow ? cmulc(v[b], srow[x]) : v[b];
      }
    }
    __syncwarp();
  }
  if (use_cluster) {
    cg::cluster_group cluster = cg::this_cluster();
    cluster.sync();  // every block's coil-group rows complete
    const int total = nr * W;
    const int beg = (int)((long long)g * total / G), end = (int)((long long)(g + 1) * total / G);
    for (int i = beg + threadIdx.x; i < end; i += blockDim.x) {
      float2 acc = c2(0.f, 0.f);
      for (int q = 0; q < G; ++q) acc += cluster.map_shared_rank(red, q)[i];  // rank order: deterministic
      out[(size_t)(yi0 + i / W) * W + i % W] = acc;
    }
    cluster.sync();  // keep this block's shared memory alive until the other blocks have read it
  } else {
    __syncthreads();
    float2* og = out + (size_t)g * gstride;
    for (int i = threadIdx.x; i < nr * W; i += blockDim.x) og[(size_t)(yi0 + i / W) * W + i % W] = red[i];
  }
}

typedef void (*FrRowsFwdFn)(CartDev, const float2*, float2*, int*);
typedef void (*FrColsFn)(CartDev, int, const float2*, float2*, float2*, const float2*, const float2*, float2*, float,
                         float);
typedef void (*FrRowsAdjFn)(CartDev, const float2*, float2*, int, int, long long);

constexpr int kWpbChoices[3] = {2, 4, 8};

// Kernels of one compiled length, one instance per warps-per-block choice.
struct FastRowKernels {
  FrRowsFwdFn fwd[3] = {nullptr, nullptr, nullptr};
  FrRowsAdjFn adj[3] = {nullptr, nullptr, nullptr};
  int A = 0, B = 0;
  bool ok() const { return fwd[0] != nullptr; }
};
struct FastColKernels {
  FrColsFn cols[3] = {nullptr, nullptr, nullptr};
  int A = 0, B = 0;
  bool ok() const { return cols[0] != nullptr; }
};

template <int A, int B>
FastRowKernels row_kernels() {
  FastRowKernels k;
  k.fwd[0] = fr_rows_fwd<A, B, 2>;
  k.fwd[1] = fr_rows_fwd<A, B, 4>;
  k.fwd[2] = fr_rows_fwd<A, B, 8>;
  k.adj[0] = fr_rows_adj<A, B, 2>;
  k.adj[1] = fr_rows_adj<A, B, 4>;
  k.adj[2] = fr_rows_adj<A, B, 8>;
  k.A = A;
  k.B = B;
  return k;
}
template <int A, int B>
FastColKernels col_kernels() {
  FastColKernels k;
  k.cols[0] = fr_cols<A, B, 2>;
  k.cols[1] = fr_cols<A, B, 4>;
  k.cols[2] = fr_cols<A, B, 8>;
  k.A = A;
  k.B = B;
  return k;
}

// Lengths with a compiled two-level split.
#define PDT_FAST_SIZES(X) X(32, 4, 8) X(48, 6, 8) X(64, 8, 8) X(96, 8, 12) X(128, 8, 16) X(192, 12, 16) \
  X(256, 16, 16) X(320, 16, 20) X(368, 16, 23) X(384, 16, 24) X(512, 16, 32) X(640, 32, 20) X(768, 32, 24)

FastRowKernels find_row_kernels(int n) {
#define PDT_ROWCASE(N, A, B) \
  if (n == N) return row_kernels<A, B>();
  PDT_FAST_SIZES(PDT_ROWCASE)
#undef PDT_ROWCASE
  return FastRowKernels();
}
FastColKernels find_col_kernels(int n) {
#define PDT_COLCASE(N, A, B) \
  if (n == N) return col_kernels<A, B>();
  PDT_FAST_SIZES(PDT_COLCASE)
#undef PDT_COLCASE
  return FastColKernels();
}

size_t fast_rows_smem(const CartDev& d, int A, int B, int wpb) {
  const size_t n = (size_t)A * B, xch = (size_t)B * (A + 1);
  return sizeof(float2) * (n + wpb * xch + (size_t)d.ns * wpb) + sizeof(int) * n;
}
size_t fast_rows_adj_smem(const CartDev& d, int A, int B, int wpb) {
  return fast_rows_smem(d, A, B, wpb) + sizeof(float2) * (size_t)wpb * A * B;
}
size_t fast_cols_smem(int A, int B, int wpb) {
  const size_t n = (size_t)A * B, xch = (size_t)B * (A + 1);
  return sizeof(float2) * (n + wpb * xch);
}

}  // namespace
}  // namespace pdt
