// pdt_rad_fast.cuh -- lane-distributed FFT passes of the radial operators for grid lengths with a
// compiled split G = M * L (LaneFft, pdt_regfft.cuh). Included by pdt_radial.cu after RadDev.
//
// Same index maps as the generic passes: image x sits on grid slot (x - N/2) mod G, so grid slot p holds
// image x = (p + N/2) mod G when that is < N (zero padding elsewhere); spectra are in natural order.
//   rl_rows_fwd   image rows . sens_c / deap -> FFT along x           -> T[c][gx][image row]
//   rl_cols       FFT along y of each grid column (input on N rows)   -> F[c][gx][gy]
//   rl_cols_inv   IFFT along y of each grid column, keep the N rows   -> T[c][gx][image row]
//   rl_rows_inv   IFFT along x, crop, / deap, conj(sens_c) . and the coil-group sum (the next coil's grid
//                 rows and this coil's map rows arrive by asynchronous copies during the transform)
// Row passes stage R = WPB * 32 / L rows per block in shared memory so that T is written / read in runs
// of R rows; column passes stage one grid column per lane group so that F is written / read whole.
#pragma once

#include "pdt_regfft.cuh"

namespace pdt {
namespace {

constexpr int kRadWpb = 4;  // warps per block of the lane-FFT passes

template <int M, int L>
__global__ void __launch_bounds__(32 * kRadWpb) rl_rows_fwd(RadDev d, const float2* __restrict__ u,
                                                            float2* __restrict__ T) {
  using F = LaneFft<M, L>;
  constexpr int G = F::n, R = kRadWpb * (32 / L);
  extern __shared__ float2 sm[];
  float2* tw = sm;
  float2* stage = tw + G;  // [G][R]
  for (int i = threadIdx.x; i < G; i += blockDim.x) tw[i] = d.tw[i];
  __syncthreads();
  const int lane = threadIdx.x & 31, t = lane & (L - 1);
  const int r = (threadIdx.x >> 5) * (32 / L) + lane / L;
  const int y0 = blockIdx.x * R, c = blockIdx.y;
  const int nr = min(R, d.N - y0);
  const bool ok = r < nr;
  const int y = y0 + (ok ? r : 0);  // a group past the last row transforms row y0 and discards it
  const float2* urow = u + (size_t)y * d.N;
  const float2* srow = d.sens ? d.sens + ((size_t)c * d.N + y) * d.N : nullptr;
  const float dy = d.deap[y];
  float2 v[M];
#pragma unroll
  for (int j = 0; j < M; ++j) {
    int x = t + L * j + d.off;
    if (x >= G) x -= G;
    float2 val = c2(0.f, 0.f);
    if (x < d.N) {
      val = urow[x];
      if (srow) val = cmul(val, srow[x]);
      val = val * (d.scale / (d.deap[x] * dy));
    }
    v[j] = val;
  }
  F::fwd(v, t, tw);
  if (ok) {
    const int kb = M * lane_brev<L>(t);
#pragma unroll
    for (int k1 = 0; k1 < M; ++k1) stage[(k1 + kb) * R + r] = v[k1];
  }
  __syncthreads();
  for (int i = threadIdx.x; i < G * nr; i += blockDim.x) {
    const int gx = i / nr, rr = i - gx * nr;
    T[((size_t)c * G + gx) * d.N + y0 + rr] = stage[gx * R + rr];
  }
}

template <int M, int L>
__global__ void __launch_bounds__(32 * kRadWpb) rl_cols(RadDev d, const float2* __restrict__ T,
                                                        float2* __restrict__ Fo) {
  using F = LaneFft<M, L>;
  constexpr int G = F::n, S = kRadWpb * (32 / L);
  extern __shared__ float2 sm[];
  float2* tw = sm;
  float2* stage = tw + G;  // [S][G]
  for (int i = threadIdx.x; i < G; i += blockDim.x) tw[i] = d.tw[i];
  __syncthreads();
  const int lane = threadIdx.x & 31, t = lane & (L - 1);
  const int q = (threadIdx.x >> 5) * (32 / L) + lane / L;
  const int gx0 = blockIdx.x * S, c = blockIdx.y;
  const int ncol = min(S, G - gx0);
  const bool ok = q < ncol;
  const float2* col = T + ((size_t)c * G + gx0 + (ok ? q : 0)) * d.N;
  float2 v[M];
#pragma unroll
  for (int j = 0; j < M; ++j) {
    int y = t + L * j + d.off;
    if (y >= G) y -= G;
    v[j] = y < d.N ? col[y] : c2(0.f, 0.f);
  }
  F::fwd(v, t, tw);
  if (ok) {
    const int kb = M * lane_brev<L>(t);
#pragma unroll
    for (int k1 = 0; k1 < M; ++k1) stage[q * G + k1 + kb] = v[k1];
  }
  __syncthreads();
  for (int i = threadIdx.x; i < ncol * G; i += blockDim.x) Fo[((size_t)c * G + gx0) * G + i] = stage[i];
}

template <int M, int L>
__global__ void __launch_bounds__(32 * kRadWpb) rl_cols_inv(RadDev d, const float2* __restrict__ H,
                                                            float2* __restrict__ T) {
  using F = LaneFft<M, L>;
  constexpr int G = F::n, S = kRadWpb * (32 / L);
  extern __shared__ float2 sm[];
  float2* tw = sm;
  float2* stage = tw + G;  // [S][G]
  const int gx0 = blockIdx.x * S, c = blockIdx.y;
  const int ncol = min(S, G - gx0);
  for (int i = threadIdx.x; i < G; i += blockDim.x) tw[i] = d.tw[i];
  for (int i = threadIdx.x; i < ncol * G; i += blockDim.x) stage[i] = H[((size_t)c * G + gx0) * G + i];
  __syncthreads();
  const int lane = threadIdx.x & 31, t = lane & (L - 1);
  const int q = (threadIdx.x >> 5) * (32 / L) + lane / L;
  const bool ok = q < ncol;
  const int qc = ok ? q : 0;
  const int kb = M * lane_brev<L>(t);
  float2 v[M];
#pragma unroll
  for (int k1 = 0; k1 < M; ++k1) v[k1] = stage[qc * G + k1 + kb];
  F::inv(v, t, tw);
  if (ok) {
    float2* out = T + ((size_t)c * G + gx0 + q) * d.N;
#pragma unroll
    for (int j = 0; j < M; ++j) {
      int y = t + L * j + d.off;
      if (y >= G) y -= G;
      if (y < d.N) out[y] = v[j];
    }
  }
}

// per block of R image rows and coil group g: IFFT along x of each coil, crop, deapodise, conj(sens) and
// accumulate in shared memory (each lane always owns the same pixels); the group's partial image goes to
// out + g * gstride.
template <int M, int L>
__global__ void __launch_bounds__(32 * kRadWpb) rl_rows_inv(RadDev d, const float2* __restrict__ T,
                                                            float2* __restrict__ out, int G_, long long gstride) {
  using F = LaneFft<M, L>;
  constexpr int G = F::n, R = kRadWpb * (32 / L);
  extern __shared__ __align__(16) float2 sm_ri[];
  float2* tw = sm_ri;
  float2* stage = tw + G;                 // [2][G][R]: this coil's grid rows and the next coil's
  float2* acc = stage + 2 * G * R;        // [R][N]
  float2* smap = acc + (size_t)R * d.N;   // [R][N] coil-map rows of this coil
  float* sdeap = reinterpret_cast<float*>(smap + (size_t)R * d.N);  // [N]
  const int y0 = blockIdx.x * R, g = blockIdx.y;
  const int nr = min(R, d.N - y0);
  const int c_begin = (int)((long long)g * d.C / G_), c_end = (int)((long long)(g + 1) * d.C / G_);
  for (int i = threadIdx.x; i < G; i += blockDim.x) tw[i] = d.tw[i];
  for (int i = threadIdx.x; i < R * d.N; i += blockDim.x) acc[i] = c2(0.f, 0.f);
  for (int i = threadIdx.x; i < d.N; i += blockDim.x) sdeap[i] = d.deap[i];
  const int lane = threadIdx.x & 31, t = lane & (L - 1);
  const int r = (threadIdx.x >> 5) * (32 / L) + lane / L;
  const bool ok = r < nr;
  const int rc = ok ? r : 0;
  const int y = y0 + rc;
  const int kb = M * lane_brev<L>(t);
  const float dy = d.deap[y];
  // asynchronous copies, one commit group each per coil c: [map rows of c], [grid rows of c + 1]; the
  // grid rows of c_begin before the loop, so that both loads overlap the transform before them
  auto copy_rows = [&](int c, float2* dst) {
    for (int i = threadIdx.x; i < G * nr; i += blockDim.x) {
      const int gx = i / nr, rr = i - gx * nr;
      cp_async8(dst + gx * R + rr, T + ((size_t)c * G + gx) * d.N + y0 + rr);
    }
  };
  if (c_begin < c_end) copy_rows(c_begin, stage);
  cp_async_commit();
  for (int c = c_begin; c < c_end; ++c) {
    const int k = c - c_begin;
    float2* cur = stage + (size_t)(k & 1) * G * R;
    __syncthreads();  // the map buffer and the other stage are free (and, the first time, the tables ready)
    if (d.sens) {
      const float2* src = d.sens + ((size_t)c * d.N + y0) * d.N;  // rows y0 .. y0 + nr - 1 of coil c
      for (int i = threadIdx.x; i < nr * d.N; i += blockDim.x) cp_async8(smap + i, src + i);
    }
    cp_async_commit();
    if (c + 1 < c_end) copy_rows(c + 1, stage + (size_t)((k + 1) & 1) * G * R);
    cp_async_commit();
    cp_async_wait<2>();  // this thread's copies of coil c's grid rows landed
    __syncthreads();
    float2 v[M];
#pragma unroll
    for (int k1 = 0; k1 < M; ++k1) v[k1] = cur[(k1 + kb) * R + rc];
    F::inv(v, t, tw);
    cp_async_wait<1>();  // this thread's copies of coil c's map rows landed
    __syncthreads();
    if (ok) {
      const float2* srow = d.sens ? smap + (size_t)r * d.N : nullptr;
      float2* arow = acc + (size_t)r * d.N;
#pragma unroll
      for (int j = 0; j < M; ++j) {
        int x = t + L * j + d.off;
        if (x >= G) x -= G;
        if (x < d.N) {
          float2 val = v[j] * (d.scale / (sdeap[x] * dy));
          if (srow) val = cmulc(val, srow[x]);
          arow[x] += val;
        }
      }
    }
  }
  cp_async_wait<0>();
  __syncthreads();
  float2* og = out + (size_t)g * gstride;
  for (int i = threadIdx.x; i < nr * d.N; i += blockDim.x) {
    const int rr = i / d.N, x = i - rr * d.N;
    og[(size_t)(y0 + rr) * d.N + x] = acc[i];
  }
}

typedef void (*RlRowsFwdFn)(RadDev, const float2*, float2*);
typedef void (*RlColsFn)(RadDev, const float2*, float2*);
typedef void (*RlRowsInvFn)(RadDev, const float2*, float2*, int, long long);

struct RadFastKernels {
  RlRowsFwdFn rows_fwd = nullptr;
  RlColsFn cols = nullptr, cols_inv = nullptr;
  RlRowsInvFn rows_inv = nullptr;
  int M = 0, L = 0;
  bool ok() const { return rows_fwd != nullptr; }
  int per_block() const { return kRadWpb * (32 / L); }  // rows (row passes) or columns (column passes)
};

template <int M, int L>
RadFastKernels rad_kernels() {
  RadFastKernels k;
  k.rows_fwd = rl_rows_fwd<M, L>;
  k.cols = rl_cols<M, L>;
  k.cols_inv = rl_cols_inv<M, L>;
  k.rows_inv = rl_rows_inv<M, L>;
  k.M = M;
  k.L = L;
  return k;
}

// Grid lengths with a compiled split G = M * L (as for the Cartesian kernels).
#define PDT_RAD_SIZES(X) X(32, 4, 8) X(48, 6, 8) X(64, 8, 8) X(96, 6, 16) X(128, 8, 16) X(192, 12, 16) \
  X(256, 16, 16) X(320, 10, 32) X(368, 23, 16) X(384, 12, 32) X(512, 16, 32) X(640, 20, 32) X(768, 24, 32)

RadFastKernels find_rad_kernels(int n) {
#define PDT_RADCASE(N_, M_, L_) \
  if (n == N_) return rad_kernels<M_, L_>();
  PDT_RAD_SIZES(PDT_RADCASE)
#undef PDT_RADCASE
  return RadFastKernels();
}

// dynamic shared memory of each pass
size_t rad_fast_rows_smem(const RadFastKernels& k) {
  const size_t G = (size_t)k.M * k.L;
  return sizeof(float2) * (G + G * k.per_block());
}
size_t rad_fast_rows_inv_smem(const RadFastKernels& k, int N) {
  // second grid-row stage, partial sums and coil-map rows (R x N each), deapodisation table
  const size_t G = (size_t)k.M * k.L, R = (size_t)k.per_block();
  return rad_fast_rows_smem(k) + sizeof(float2) * (G * R + 2 * R * N) + sizeof(float) * N;
}
size_t rad_fast_cols_smem(const RadFastKernels& k) {
  const size_t G = (size_t)k.M * k.L;
  return sizeof(float2) * (G + G * k.per_block());
}

}  // namespace
}  // namespace pdt
