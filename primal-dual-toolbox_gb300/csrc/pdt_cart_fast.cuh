// pdt_cart_fast.cuh -- lane-distributed FFT kernels of the Cartesian operator for the lengths with a
// compiled split n = M * L (L = 8, 16 or 32 lanes per sequence, M values per lane). Included by
// pdt_cartesian.cu after CartDev.
//
// The transforms are LaneFft<M, L> (pdt_regfft.cuh): lane t of a group of L lanes holds x[t + L j] in
// registers and ends with X[k1 + M brev_L(t)] in register k1.
//
// Kernels (one sequence per lane group; 32 / L sequences per warp):
//   fl_rows_fwd   rows of ubar . sens_c -> FFT along W -> sampled columns t1[c][s][yi]
//   fl_cols       per sampled column: FFT along Hf -> mask -> k-space dual prox -> mask -> IFFT along Hf
//   fl_rows_adj   per row block and coil group: IFFT along W -> conj(sens_c) . -> coil sum
// The k-space arrays of the column phase (dual r, data f, mask) are stored per sampled column in the
// order the transform leaves them: position P = k1 * L + t holds spectrum index k1 + M brev_L(t), so
// that lanes read and write consecutive addresses. CartDev::kperm maps P to the output row.
#pragma once

#include <cooperative_groups.h>

#include "pdt_regfft.cuh"

namespace cg = cooperative_groups;

namespace pdt {
namespace {

// Phase 1: rows of ubar . sens_c -> FFT along W -> sampled columns t1[c][s][yi]. A block takes
// R = WPB * 32 / L consecutive rows of one coil and writes each sampled column's R rows as one run.
template <int M, int L, int WPB>
__global__ void __launch_bounds__(32 * WPB) fl_rows_fwd(CartDev d, const float2* __restrict__ ubar,
                                                        float2* __restrict__ t1, int* __restrict__ tick) {
  using F = LaneFft<M, L>;
  constexpr int W = F::n, R = WPB * (32 / L);
  extern __shared__ float2 sm[];
  float2* tw = sm;
  float2* stage = tw + W;  // [ns][R]
  int* fs2s = reinterpret_cast<int*>(stage + (size_t)d.ns * R);
  for (int i = threadIdx.x; i < W; i += blockDim.x) {
    tw[i] = d.twW[i];
    fs2s[i] = d.fslot2s[i];
  }
  pdl_wait();  // ubar comes from the previous kernel; t1 may still be read by it
  pdl_trigger();
  if (tick && blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) atomicAdd(tick, 1);
  __syncthreads();
  const int lane = threadIdx.x & 31, t = lane & (L - 1);
  const int r = (threadIdx.x >> 5) * (32 / L) + lane / L;
  const int yi0 = blockIdx.x * R, c = blockIdx.y;
  const int nr = min(R, d.Hi - yi0);
  const bool ok = r < nr;
  const int yi = yi0 + (ok ? r : 0);  // a group past the last row transforms row yi0 and discards it
  const float2* urow = ubar + (size_t)yi * W;
  const float2* srow = d.sens ? d.sens + ((size_t)c * d.Hf + yi + d.y0) * W : nullptr;
  float2 v[M];
#pragma unroll
  for (int j = 0; j < M; ++j) {
    int x = t + L * j - d.mxW;  // FFT slot t + L j holds image column (slot - mid) mod W
    if (x < 0) x += W;
    float2 val = urow[x];
    if (srow) val = cmul(val, srow[x]);
    v[j] = val;
  }
  F::fwd(v, t, tw);
  if (ok) {
    const int kb = M * lane_brev<L>(t);
#pragma unroll
    for (int k1 = 0; k1 < M; ++k1) {
      const int s = fs2s[k1 + kb];
      if (s >= 0) stage[s * R + r] = v[k1];
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < d.ns * nr; i += blockDim.x) {
    const int s = i / nr, rr = i - s * nr;
    t1[((size_t)c * d.ns + s) * d.Hi + yi0 + rr] = stage[s * R + rr];
  }
}

// Phase 2: per sampled column, FFT along Hf -> mask -> (k-space dual prox) -> mask -> IFFT along Hf.
// r, fc and the mask are in the transform order (position k1 * L + t of the column).
template <int M, int L, int WPB>
__global__ void __launch_bounds__(32 * WPB) fl_cols(CartDev d, int mode, const float2* t_in, float2* t_out,
                                                    float2* __restrict__ r, const float2* __restrict__ fc,
                                                    const float2* __restrict__ kin, float2* __restrict__ kout,
                                                    float sigma, float lambda) {
  using F = LaneFft<M, L>;
  constexpr int Hf = F::n;
  extern __shared__ float2 sm[];
  float2* tw = sm;
  for (int i = threadIdx.x; i < Hf; i += blockDim.x) tw[i] = d.twH[i];
  pdl_wait();  // t_in, r and fc come from earlier kernels
  pdl_trigger();
  __syncthreads();
  const int lane = threadIdx.x & 31, t = lane & (L - 1);
  const int s0 = (blockIdx.x * WPB + (threadIdx.x >> 5)) * (32 / L) + lane / L;
  const int c = blockIdx.y;
  const bool ok = s0 < d.ns;
  const int s = ok ? s0 : d.ns - 1;  // a group past the last column reads column ns-1 and discards it
  const size_t colc = (size_t)c * d.ns + s;
  const int kb = M * lane_brev<L>(t);
  const float* mrow = d.maskc + (size_t)s * Hf;
  float2 v[M];
  if (mode == COL_SOLVE || mode == COL_FWD_DENSE) {
#pragma unroll
    for (int j = 0; j < M; ++j) {
      int yf = t + L * j - d.mxH;
      if (yf < 0) yf += Hf;
      const int yi = yf - d.y0;
      v[j] = (yi >= 0 && yi < d.Hi) ? t_in[colc * d.Hi + yi] : c2(0.f, 0.f);
    }
    F::fwd(v, t, tw);
    if (mode == COL_FWD_DENSE) {
      if (ok) {
#pragma unroll
        for (int k1 = 0; k1 < M; ++k1) {
          int ypos = k1 + kb + d.oyH;
          if (ypos >= Hf) ypos -= Hf;
          kout[((size_t)c * Hf + ypos) * d.W + d.col_x[s]] = v[k1] * (d.scale * mrow[k1 * L + t]);
        }
      }
      return;
    }
    // chunks of loads -> math -> stores (r is read and written in place)
    constexpr int CH = M < 8 ? M : 8;
    const float2* fcol = fc + colc * Hf;
    float2* rcol = r + colc * Hf;
#pragma unroll
    for (int k0 = 0; k0 < M; k0 += CH) {
      float m[CH];
      float2 fv[CH], rv[CH];
#pragma unroll
      for (int q = 0; q < CH; ++q) {
        if (k0 + q < M) {
          const int P = (k0 + q) * L + t;
          m[q] = mrow[P];
          fv[q] = fcol[P];
          rv[q] = rcol[P];
        }
      }
#pragma unroll
      for (int q = 0; q < CH; ++q) {
        if (k0 + q < M) {
          const float2 kv = v[k0 + q] * (d.scale * m[q]);
          rv[q] = (rv[q] + sigma * (kv - fv[q])) / (1.0f + sigma * lambda);
          v[k0 + q] = rv[q] * m[q];
        }
      }
      if (ok) {
#pragma unroll
        for (int q = 0; q < CH; ++q)
          if (k0 + q < M) rcol[(k0 + q) * L + t] = rv[q];
      }
    }
  } else {
#pragma unroll
    for (int k1 = 0; k1 < M; ++k1) {
      float2 val;
      if (mode == COL_ADJ_DENSE) {
        int ypos = k1 + kb + d.oyH;
        if (ypos >= Hf) ypos -= Hf;
        val = kin[((size_t)c * Hf + ypos) * d.W + d.col_x[s]];
      } else {
        val = fc[colc * Hf + k1 * L + t];
      }
      v[k1] = val * mrow[k1 * L + t];
    }
  }
  F::inv(v, t, tw);
  if (ok) {
#pragma unroll
    for (int j = 0; j < M; ++j) {
      int yf = t + L * j + d.oyH;
      if (yf >= Hf) yf -= Hf;
      const int yi = yf - d.y0;
      if (yi >= 0 && yi < d.Hi) t_out[colc * d.Hi + yi] = v[j] * d.scale;
    }
  }
}

// Phase 2 over two warps per column (n = M * 64): the same steps as fl_cols with LaneFft64, for column
// lengths whose 32-lane split would hold many values per lane; WPB / 2 columns per block. The compact
// order is position k1 * 64 + t for spectrum index k1 + M brev_64(t).
// ZM: register slots j (bit j) that are known at compile time to hold only rows outside the image, for
// every lane: their forward-transform inputs are zero and their inverse-transform outputs are not
// stored, so the register DFTs fold them away (the host selects it when the geometry matches).
template <int M, int WPB, int ZM = 0>
__global__ void __launch_bounds__(32 * WPB) fl_cols64(CartDev d, int mode, const float2* t_in, float2* t_out,
                                                      float2* __restrict__ r, const float2* __restrict__ fc,
                                                      const float2* __restrict__ kin, float2* __restrict__ kout,
                                                      float sigma, float lambda) {
  static_assert(WPB % 2 == 0, "two warps per column");
  using F = LaneFft64<M>;
  constexpr int Hf = F::n, L = 64;
  extern __shared__ float2 sm[];
  float2* tw = sm;
  const int pair = threadIdx.x >> 6;
  float2* xbuf = tw + Hf + (size_t)pair * M * 64;
  const int bar = 1 + pair;  // named barrier of this column's two warps (0 is __syncthreads)
  for (int i = threadIdx.x; i < Hf; i += blockDim.x) tw[i] = d.twH[i];
  pdl_wait();  // t_in, r and fc come from earlier kernels
  pdl_trigger();
  __syncthreads();
  const int t = threadIdx.x & 63;
  const int s0 = blockIdx.x * (WPB / 2) + pair;
  const int c = blockIdx.y;
  const bool ok = s0 < d.ns;
  const int s = ok ? s0 : d.ns - 1;  // a pair past the last column reads column ns-1 and discards it
  const size_t colc = (size_t)c * d.ns + s;
  const int kb = M * (int)(__brev((unsigned)t) >> 26);
  const float* mrow = d.maskc + (size_t)s * Hf;
  float2 v[M];
  if (mode == COL_SOLVE || mode == COL_FWD_DENSE) {
#pragma unroll
    for (int j = 0; j < M; ++j) {
      if ((ZM >> j) & 1) {
        v[j] = c2(0.f, 0.f);
        continue;
      }
      int yf = t + L * j - d.mxH;
      if (yf < 0) yf += Hf;
      const int yi = yf - d.y0;
      v[j] = (yi >= 0 && yi < d.Hi) ? t_in[colc * d.Hi + yi] : c2(0.f, 0.f);
    }
    F::fwd(v, t, tw, xbuf, bar);
    if (mode == COL_FWD_DENSE) {
      if (ok) {
#pragma unroll
        for (int k1 = 0; k1 < M; ++k1) {
          int ypos = k1 + kb + d.oyH;
          if (ypos >= Hf) ypos -= Hf;
          kout[((size_t)c * Hf + ypos) * d.W + d.col_x[s]] = v[k1] * (d.scale * mrow[k1 * L + t]);
        }
      }
      return;
    }
    const float2* fcol = fc + colc * Hf;
    float2* rcol = r + colc * Hf;
    float m[M];
    float2 fv[M], rv[M];
#pragma unroll
    for (int k1 = 0; k1 < M; ++k1) {
      const int P = k1 * L + t;
      m[k1] = mrow[P];
      fv[k1] = fcol[P];
      rv[k1] = rcol[P];
    }
#pragma unroll
    for (int k1 = 0; k1 < M; ++k1) {
      const float2 kv = v[k1] * (d.scale * m[k1]);
      rv[k1] = (rv[k1] + sigma * (kv - fv[k1])) / (1.0f + sigma * lambda);
      v[k1] = rv[k1] * m[k1];
    }
    if (ok) {
#pragma unroll
      for (int k1 = 0; k1 < M; ++k1) rcol[k1 * L + t] = rv[k1];
    }
  } else {
#pragma unroll
    for (int k1 = 0; k1 < M; ++k1) {
      float2 val;
      if (mode == COL_ADJ_DENSE) {
        int ypos = k1 + kb + d.oyH;
        if (ypos >= Hf) ypos -= Hf;
        val = kin[((size_t)c * Hf + ypos) * d.W + d.col_x[s]];
      } else {
        val = fc[colc * Hf + k1 * L + t];
      }
      v[k1] = val * mrow[k1 * L + t];
    }
  }
  F::inv(v, t, tw, xbuf, bar);
  if (ok) {
#pragma unroll
    for (int j = 0; j < M; ++j) {
      if ((ZM >> j) & 1) continue;
      int yf = t + L * j + d.oyH;
      if (yf >= Hf) yf -= Hf;
      const int yi = yf - d.y0;
      if (yi >= 0 && yi < d.Hi) t_out[colc * d.Hi + yi] = v[j] * d.scale;
    }
  }
}

// Phase 3: per block of R image rows and coil group g, IFFT along W of the sampled columns, conj(sens_c)
// multiply and the coil sum, accumulated in shared memory (each lane always owns the same pixels).
// With use_cluster the G coil groups of a row block form a cluster (grid.y = G) and reduce their rows
// through distributed shared memory in rank order (deterministic) into one K^H r plane; otherwise each
// block writes its group's partial sum to out + g * gstride.
// With `staged`, the sampled columns of the next coil and the coil-map rows of the current coil arrive in
// shared memory by asynchronous copies (two column stages, one map buffer) while the current coil's rows
// are transformed, so neither load's latency sits between the transforms; the arithmetic and its order
// are the same as without.
template <int M, int L, int WPB>
__global__ void __launch_bounds__(32 * WPB, 16 / WPB) fl_rows_adj(CartDev d, const float2* __restrict__ t2,
                                                        float2* __restrict__ out, int use_cluster, int G,
                                                        long long gstride, int staged) {
  using F = LaneFft<M, L>;
  constexpr int W = F::n, R = WPB * (32 / L);
  extern __shared__ __align__(16) float2 sm_adj[];
  float2* tw = sm_adj;
  float2* stage = tw + W;                                                 // [1 or 2][ns][R]
  float2* red = stage + (size_t)(staged ? 2 : 1) * d.ns * R;              // [R][W]
  float2* smap = red + (size_t)R * W;                                     // [R][W] (staged, with coil maps)
  const bool map_staged = staged && d.sens != nullptr;
  int* as2s = reinterpret_cast<int*>(smap + (map_staged ? (size_t)R * W : 0));
  const int g = blockIdx.y;
  for (int i = threadIdx.x; i < W; i += blockDim.x) {
    tw[i] = d.twW[i];
    as2s[i] = d.slot2s[i];
  }
  for (int i = threadIdx.x; i < R * W; i += blockDim.x) red[i] = c2(0.f, 0.f);
  pdl_wait();  // t2 comes from the previous kernel; out may still be read by earlier ones
  pdl_trigger();
  const int lane = threadIdx.x & 31, t = lane & (L - 1);
  const int r = (threadIdx.x >> 5) * (32 / L) + lane / L;
  const int yi0 = blockIdx.x * R;
  const int nr = min(R, d.Hi - yi0);
  const bool ok = r < nr;
  const int rc = ok ? r : 0;  // a group past the last row transforms row 0 of the block and discards it
  const int yi = yi0 + rc;
  const int c_begin = (int)((long long)g * d.C / G), c_end = (int)((long long)(g + 1) * d.C / G);
  const int kb = M * lane_brev<L>(t);
  if (staged) {
    // group order per coil c: [maps of c], [columns of c + 1]; the columns of c_begin before the loop
    auto copy_cols = [&](int c, float2* dst) {
      for (int i = threadIdx.x; i < d.ns * nr; i += blockDim.x) {
        const int s = i / nr, rr = i - s * nr;
        cp_async8(dst + s * R + rr, t2 + ((size_t)c * d.ns + s) * d.Hi + yi0 + rr);
      }
    };
    if (c_begin < c_end) copy_cols(c_begin, stage);
    cp_async_commit();
    for (int c = c_begin; c < c_end; ++c) {
      const int k = c - c_begin;
      float2* cur = stage + (size_t)(k & 1) * d.ns * R;
      __syncthreads();  // the map buffer and the other column stage are free (and the tables ready)
      if (map_staged) {  // rows yi0 .. yi0 + nr - 1 of coil c, 16-byte pieces (W even: rows 16-byte aligned)
        const float2* src = d.sens + ((size_t)c * d.Hf + yi0 + d.y0) * W;
        for (int i = threadIdx.x; i < nr * (W / 2); i += blockDim.x) cp_async16(smap + 2 * i, src + 2 * i);
      }
      cp_async_commit();
      if (c + 1 < c_end) copy_cols(c + 1, stage + (size_t)((k + 1) & 1) * d.ns * R);
      cp_async_commit();
      cp_async_wait<2>();  // this thread's copies of coil c's columns landed
      __syncthreads();
      float2 v[M];
#pragma unroll
      for (int k1 = 0; k1 < M; ++k1) {
        const int s = as2s[k1 + kb];
        v[k1] = s >= 0 ? cur[s * R + rc] : c2(0.f, 0.f);
      }
      F::inv(v, t, tw);
      cp_async_wait<1>();  // this thread's copies of coil c's map rows landed
      __syncthreads();
      if (ok) {
        const float2* srow = map_staged ? smap + (size_t)r * W : nullptr;
        float2* rrow = red + (size_t)r * W;
#pragma unroll
        for (int j = 0; j < M; ++j) {
          int x = t + L * j + d.oxW;  // IFFT slot t + L j lands on image column (slot + n/2) mod W
          if (x >= W) x -= W;
          rrow[x] += srow ? cmulc(v[j], srow[x]) : v[j];
        }
      }
    }
    cp_async_wait<0>();
  } else {
  // register prefetch of the next coil's sampled columns (ns * nr values spread over the block)
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
    __syncthreads();  // stage free (and, the first time, tables and red ready)
    if (pf_all) {
#pragma unroll
      for (int q = 0; q < PF; ++q) {
        const int i = threadIdx.x + q * (int)blockDim.x;
        if (i < d.ns * nr) {
          const int s = i / nr, rr = i - s * nr;
          stage[s * R + rr] = pf[q];
        }
      }
      if (c + 1 < c_end) fetch(c + 1);
    } else {
      for (int i = threadIdx.x; i < d.ns * nr; i += blockDim.x) {
        const int s = i / nr, rr = i - s * nr;
        stage[s * R + rr] = t2[((size_t)c * d.ns + s) * d.Hi + yi0 + rr];
      }
    }
    __syncthreads();
    float2 v[M];
#pragma unroll
    for (int k1 = 0; k1 < M; ++k1) {
      const int s = as2s[k1 + kb];
      v[k1] = s >= 0 ? stage[s * R + rc] : c2(0.f, 0.f);
    }
    F::inv(v, t, tw);
    if (ok) {
      const float2* srow = d.sens ? d.sens + ((size_t)c * d.Hf + yi + d.y0) * W : nullptr;
      float2* rrow = red + (size_t)r * W;
#pragma unroll
      for (int j = 0; j < M; ++j) {
        int x = t + L * j + d.oxW;  // IFFT slot t + L j lands on image column (slot + n/2) mod W
        if (x >= W) x -= W;
        rrow[x] += srow ? cmulc(v[j], srow[x]) : v[j];
      }
    }
  }
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
typedef void (*FrRowsAdjFn)(CartDev, const float2*, float2*, int, int, long long, int);

constexpr int kWpbChoices[3] = {2, 4, 8};

// Kernels of one compiled length n = M * L, one instance per warps-per-block choice.
struct FastRowKernels {
  FrRowsFwdFn fwd[3] = {nullptr, nullptr, nullptr};
  FrRowsAdjFn adj[3] = {nullptr, nullptr, nullptr};
  int M = 0, L = 0;
  bool ok() const { return fwd[0] != nullptr; }
  int rows_per_block(int wpb) const { return wpb * (32 / L); }
};
struct FastColKernels {
  FrColsFn cols[3] = {nullptr, nullptr, nullptr};
  FrColsFn cols_z[3] = {nullptr, nullptr, nullptr};  // specialisation for the zero-slot mask zmask
  int M = 0, L = 0, zmask = 0;
  bool ok() const { return cols[0] != nullptr; }
  int cols_per_block(int wpb) const { return L == 64 ? wpb / 2 : wpb * (32 / L); }
};

template <int M, int L>
FastRowKernels row_kernels() {
  FastRowKernels k;
  k.fwd[0] = fl_rows_fwd<M, L, 2>;
  k.fwd[1] = fl_rows_fwd<M, L, 4>;
  k.fwd[2] = fl_rows_fwd<M, L, 8>;
  k.adj[0] = fl_rows_adj<M, L, 2>;
  k.adj[1] = fl_rows_adj<M, L, 4>;
  k.adj[2] = fl_rows_adj<M, L, 8>;
  k.M = M;
  k.L = L;
  return k;
}
template <int M, int L>
FastColKernels col_kernels() {
  FastColKernels k;
  k.cols[0] = fl_cols<M, L, 2>;
  k.cols[1] = fl_cols<M, L, 4>;
  k.cols[2] = fl_cols<M, L, 8>;
  k.M = M;
  k.L = L;
  return k;
}

// Lengths with a compiled split n = M * L.
#define PDT_FAST_SIZES(X) X(32, 4, 8) X(48, 6, 8) X(64, 8, 8) X(96, 6, 16) X(128, 8, 16) X(192, 12, 16) \
  X(256, 16, 16) X(320, 10, 32) X(368, 46, 8) X(384, 12, 32) X(512, 16, 32) X(640, 20, 32) X(768, 24, 32)

FastRowKernels find_row_kernels(int n) {
#define PDT_ROWCASE(N, M, L) \
  if (n == N) return row_kernels<M, L>();
  PDT_FAST_SIZES(PDT_ROWCASE)
#undef PDT_ROWCASE
  return FastRowKernels();
}

// Row splits for launches that share the SMs with other problems' kernels (batched solves): the 46
// values per lane of 368 = 46 x 8 hold about 200 registers, one 256-thread block per SM, which is fastest
// alone but crowds out the concurrent kernels; 23 x 16 needs about 70. Twiddles and slot maps are indexed
// by the natural spectrum index, so both splits read and write the same arrays from the same tables.
#define PDT_CONCURRENT_ROW_SIZES(X) X(368, 23, 16)

FastRowKernels find_concurrent_row_kernels(int n) {
#define PDT_ROWCASE(N, M, L) \
  if (n == N) return row_kernels<M, L>();
  PDT_CONCURRENT_ROW_SIZES(PDT_ROWCASE)
#undef PDT_ROWCASE
  return FastRowKernels();
}
template <int M>
FastColKernels col_kernels64() {
  FastColKernels k;
  k.cols[0] = fl_cols64<M, 2>;
  k.cols[1] = fl_cols64<M, 4>;
  k.cols[2] = fl_cols64<M, 8>;
  if constexpr (M == 10) {  // 640 rows with readout-oversampling removal: slots 3..6 lie outside the image
    k.cols_z[0] = fl_cols64<M, 2, 0x78>;
    k.cols_z[1] = fl_cols64<M, 4, 0x78>;
    k.cols_z[2] = fl_cols64<M, 8, 0x78>;
    k.zmask = 0x78;
  }
  k.M = M;
  k.L = 64;
  return k;
}

// Column lengths from 320 up run over two warps per column (M = n / 64 values per lane).
#define PDT_COL64_SIZES(X) X(320, 5) X(384, 6) X(512, 8) X(640, 10) X(768, 12)

FastColKernels find_col_kernels(int n) {
#define PDT_COL64CASE(N, M) \
  if (n == N) return col_kernels64<M>();
  PDT_COL64_SIZES(PDT_COL64CASE)
#undef PDT_COL64CASE
#define PDT_COLCASE(N, M, L) \
  if (n == N) return col_kernels<M, L>();
  PDT_FAST_SIZES(PDT_COLCASE)
#undef PDT_COLCASE
  return FastColKernels();
}

size_t fast_rows_smem(const CartDev& d, const FastRowKernels& k, int wpb) {
  const size_t n = (size_t)k.M * k.L, R = (size_t)k.rows_per_block(wpb);
  return sizeof(float2) * (n + (size_t)d.ns * R) + sizeof(int) * n;
}
size_t fast_rows_adj_smem(const CartDev& d, const FastRowKernels& k, int wpb, bool staged = false) {
  const size_t n = (size_t)k.M * k.L, R = (size_t)k.rows_per_block(wpb);
  const size_t extra = staged ? (size_t)d.ns * R + (d.sens ? R * n : 0) : 0;  // second column stage, map rows
  return fast_rows_smem(d, k, wpb) + sizeof(float2) * (R * n + extra);
}
size_t fast_cols_smem(const FastColKernels& k, int wpb) {
  const size_t n = (size_t)k.M * k.L;
  return sizeof(float2) * (n + (k.L == 64 ? (size_t)(wpb / 2) * n : 0));  // twiddles (+ exchange buffers)
}

// Host bit reversal over log2(L) bits (the order LaneFft leaves a spectrum in).
inline int host_lane_brev(int t, int L) {
  int r = 0;
  for (int b = 1; b < L; b <<= 1) r = (r << 1) | ((t & b) ? 1 : 0);
  return r;
}

}  // namespace
}  // namespace pdt
