// pdt_image.cu -- fused image-side primal-dual steps (TV, TGV^2, TV/TGV with an operator).
//
// The denoising kernels do one whole iteration's image-side work for a 32 x 8 tile: they stage the
// over-relaxed primal (u-bar, v-bar) plus a one-pixel halo in shared memory, recompute the dual update
// on the halo pixels they need, and finish the primal update from shared memory. The reference does
// the same arithmetic in two to four separate launches (tgv_kernels.cuh:225-324, 432-467, 568-605,
// 647-686), each re-reading its neighbours from global memory. The with-operator solvers split the
// image side into a dual and a primal kernel instead (see below).
//
// Fields read at a neighbour (u-bar, v-bar, p, q -- and u, v for the primal-first TGV order) ping-pong
// between an `in` and an `out` buffer so that tiles never read a neighbour's freshly written values.
//
// Arithmetic follows the reference kernels element by element:
//   grad+  (dp,   tgv_kernels.cuh:40-50)   Neumann forward differences, zero at x = W-1 / y = H-1
//   eps(v) (dp_sym, :25-38)                [dx vx, 0.5 (dy vx + dx vy), dy vy]
//   div-   (dm,   :67-80)                  x==0: p(0); x==W-1: -p(W-2); else p(x) - p(x-1)
//   div_h- (dm_sym, :104-134)
//   projections 1 / max(1, |.| / alpha) with |q|^2 = |qxx|^2 + |qyy|^2 + 2 |qxy|^2 (:136-154)
//   over-relaxation theta = 1: bar = 2 new - old.
#include "pdt_device.cuh"
#include "pdt_internal.h"
#include "pdt_primal.cuh"

namespace pdt {
namespace {

constexpr int TX = 32;
constexpr int TY = 8;
constexpr int NT = TX * TY;

// div- of a 2-component field held in shared memory at local coordinates (lx, ly); (gx, gy) are the
// global coordinates used for the boundary rules.
template <class P, int LDX>
__device__ __forceinline__ P div_minus(const P (*sx)[LDX], const P (*sy)[LDX], int lx, int ly, int gx, int gy, int W,
                                       int H) {
  P d = (gx > 0) ? ((gx < W - 1) ? sx[ly][lx] - sx[ly][lx - 1] : -sx[ly][lx - 1]) : sx[ly][lx];
  d += (gy > 0) ? ((gy < H - 1) ? sy[ly][lx] - sy[ly - 1][lx] : -sy[ly - 1][lx]) : sy[ly][lx];
  return d;
}

__device__ __forceinline__ float proj_scale(float n, float alpha) { return 1.0f / fmaxf(1.0f, n / alpha); }

// ------------------------------------------------------------------------------------------------
// TvOptimizer: p <- proj_1(p + sigma grad+ ub); u+ = (u + tau (div- p + lambda f)) / (1 + tau lambda).
// ------------------------------------------------------------------------------------------------
template <class P>
__global__ void __launch_bounds__(NT) tv_step_kernel(int W, int H, ImgPtrs in, ImgPtrs out,
                                                     const P* __restrict__ f, float tau, float sigma, float lambda) {
  __shared__ P s_ub[TY + 2][TX + 2];  // [x0-1, x0+TX] x [y0-1, y0+TY]
  __shared__ P s_px[TY + 1][TX + 1];  // [x0-1, x0+TX) x [y0-1, y0+TY)
  __shared__ P s_py[TY + 1][TX + 1];
  const int tid = threadIdx.x;
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
  const P* ub = static_cast<const P*>(in.ub);
  const P* px = static_cast<const P*>(in.px);
  const P* py = static_cast<const P*>(in.py);

  for (int i = tid; i < (TX + 2) * (TY + 2); i += NT) {
    const int ly = i / (TX + 2), lx = i - ly * (TX + 2);
    const int gx = x0 - 1 + lx, gy = y0 - 1 + ly;
    if (gx >= 0 && gx < W && gy >= 0 && gy < H) s_ub[ly][lx] = ub[(size_t)gy * W + gx];
  }
  __syncthreads();

  for (int i = tid; i < (TX + 1) * (TY + 1); i += NT) {
    const int ly = i / (TX + 1), lx = i - ly * (TX + 1);
    if (lx == 0 && ly == 0) continue;  // the corner is never read by div-
    const int gx = x0 - 1 + lx, gy = y0 - 1 + ly;
    if (gx < 0 || gx >= W || gy < 0 || gy >= H) continue;
    const int xp = lx + (gx < W - 1), yp = ly + (gy < H - 1);
    const P c = s_ub[ly][lx];
    const P gux = s_ub[ly][xp] - c, guy = s_ub[yp][lx] - c;
    const size_t idx = (size_t)gy * W + gx;
    const P a = px[idx] + sigma * gux;
    const P b = py[idx] + sigma * guy;
    const float s = proj_scale(sqrtf(abs2(a) + abs2(b)), 1.0f);
    const P pa = a * s, pb = b * s;
    s_px[ly][lx] = pa;
    s_py[ly][lx] = pb;
    if (lx > 0 && ly > 0) {
      static_cast<P*>(out.px)[idx] = pa;
      static_cast<P*>(out.py)[idx] = pb;
    }
  }
  __syncthreads();

  const int lx = tid % TX + 1, ly = tid / TX + 1;
  const int gx = x0 + lx - 1, gy = y0 + ly - 1;
  if (gx < W && gy < H) {
    const size_t idx = (size_t)gy * W + gx;
    const P uo = static_cast<const P*>(in.u)[idx];
    const P d = div_minus<P, TX + 1>(s_px, s_py, lx, ly, gx, gy, W, H);
    P un = uo + tau * (d + lambda * f[idx]);
    un = un * (1.0f / (1.0f + tau * lambda));
    static_cast<P*>(out.u)[idx] = un;
    static_cast<P*>(out.ub)[idx] = 2.0f * un - uo;
  }
}

// ------------------------------------------------------------------------------------------------
// TvOptimizer, T iterations per launch (temporal blocking): a block loads its 32 x 16 output tile plus
// a T-pixel halo of the state (u, u-bar, p, f) into shared memory and runs T dual + primal steps there
// with the same per-pixel arithmetic as tv_step_kernel. A step reads u-bar one pixel to the right /
// below and p one pixel to the left / above, so the halo loses at most one valid ring per step and the
// output tile is exact after T steps; cells next to the region edge are simply not updated. Reads the
// state from `in`, writes the tile's final state to `out` (every field ping-pongs).
// ------------------------------------------------------------------------------------------------
template <class P, int T>
__global__ void __launch_bounds__(NT) tv_multi_kernel(int W, int H, ImgPtrs in, ImgPtrs out,
                                                      const P* __restrict__ f, float tau, float sigma, float lambda) {
  constexpr int OX = 32, OY = 16, RX = OX + 2 * T, RY = OY + 2 * T;
  __shared__ P s_u[RY][RX], s_ub[RY][RX], s_px[RY][RX], s_py[RY][RX], s_f[RY][RX];
  const int tid = threadIdx.x;
  const int rx0 = blockIdx.x * OX - T, ry0 = blockIdx.y * OY - T;  // region origin in the image
  for (int i = tid; i < RX * RY; i += NT) {
    const int ly = i / RX, lx = i - ly * RX;
    const int gx = rx0 + lx, gy = ry0 + ly;
    if (gx >= 0 && gx < W && gy >= 0 && gy < H) {
      const size_t idx = (size_t)gy * W + gx;
      s_u[ly][lx] = static_cast<const P*>(in.u)[idx];
      s_ub[ly][lx] = static_cast<const P*>(in.ub)[idx];
      s_px[ly][lx] = static_cast<const P*>(in.px)[idx];
      s_py[ly][lx] = static_cast<const P*>(in.py)[idx];
      s_f[ly][lx] = f[idx];
    }
  }
  __syncthreads();
  const float inv = 1.0f / (1.0f + tau * lambda);
#pragma unroll 1
  for (int it = 0; it < T; ++it) {
    // TV_dual_p_kernel (tgv_kernels.cuh:294-324); needs u-bar to the right and below
    for (int i = tid; i < RX * RY; i += NT) {
      const int ly = i / RX, lx = i - ly * RX;
      const int gx = rx0 + lx, gy = ry0 + ly;
      if (gx < 0 || gx >= W || gy < 0 || gy >= H) continue;
      if ((lx == RX - 1 && gx < W - 1) || (ly == RY - 1 && gy < H - 1)) continue;
      const int xp = lx + (gx < W - 1), yp = ly + (gy < H - 1);
      const P c = s_ub[ly][lx];
      const P gux = s_ub[ly][xp] - c, guy = s_ub[yp][lx] - c;
      const P a = s_px[ly][lx] + sigma * gux;
      const P b = s_py[ly][lx] + sigma * guy;
      const float sc = proj_scale(sqrtf(abs2(a) + abs2(b)), 1.0f);
      s_px[ly][lx] = a * sc;
      s_py[ly][lx] = b * sc;
    }
    __syncthreads();
    // TV_primal_u_kernel (tgv_kernels.cuh:568-605); needs p to the left and above
    for (int i = tid; i < RX * RY; i += NT) {
      const int ly = i / RX, lx = i - ly * RX;
      const int gx = rx0 + lx, gy = ry0 + ly;
      if (gx < 0 || gx >= W || gy < 0 || gy >= H) continue;
      if ((lx == 0 && gx > 0) || (ly == 0 && gy > 0)) continue;
      const P uo = s_u[ly][lx];
      const P d = div_minus<P, RX>(s_px, s_py, lx, ly, gx, gy, W, H);
      P un = uo + tau * (d + lambda * s_f[ly][lx]);
      un = un * inv;
      s_u[ly][lx] = un;
      s_ub[ly][lx] = 2.0f * un - uo;
    }
    __syncthreads();
  }
  for (int i = tid; i < OX * OY; i += NT) {
    const int ly = T + i / OX, lx = T + i % OX;
    const int gx = rx0 + lx, gy = ry0 + ly;
    if (gx < W && gy < H) {
      const size_t idx = (size_t)gy * W + gx;
      static_cast<P*>(out.u)[idx] = s_u[ly][lx];
      static_cast<P*>(out.ub)[idx] = s_ub[ly][lx];
      static_cast<P*>(out.px)[idx] = s_px[ly][lx];
      static_cast<P*>(out.py)[idx] = s_py[ly][lx];
    }
  }
}

// ------------------------------------------------------------------------------------------------
// TgvOptimizer (primal first, tgvoptimizer.cu:117-137):
//   u+ = (u + tau (div- p + lambda f)) / (1 + tau lambda), v+ = v + tau (div_h- q + p)
//   p  <- proj_a1(p + sigma (grad+ ub - vb)),             q  <- proj_a0(q + sigma eps(vb))
// ------------------------------------------------------------------------------------------------
template <class P>
__global__ void __launch_bounds__(NT) tgv_denoise_step_kernel(int W, int H, ImgPtrs in, ImgPtrs out,
                                                              const P* __restrict__ f, float tau, float sigma,
                                                              float lambda, float alpha0, float alpha1) {
  // old duals on [x0-1, x0+TX] x [y0-1, y0+TY]
  __shared__ P s_px[TY + 2][TX + 2], s_py[TY + 2][TX + 2];
  __shared__ P s_qxx[TY + 2][TX + 2], s_qyy[TY + 2][TX + 2], s_qxy[TY + 2][TX + 2];
  // new over-relaxed primals on [x0, x0+TX] x [y0, y0+TY]
  __shared__ P s_ub[TY + 1][TX + 1], s_vbx[TY + 1][TX + 1], s_vby[TY + 1][TX + 1];
  const int tid = threadIdx.x;
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;

  for (int i = tid; i < (TX + 2) * (TY + 2); i += NT) {
    const int ly = i / (TX + 2), lx = i - ly * (TX + 2);
    const int gx = x0 - 1 + lx, gy = y0 - 1 + ly;
    if (gx >= 0 && gx < W && gy >= 0 && gy < H) {
      const size_t idx = (size_t)gy * W + gx;
      s_px[ly][lx] = static_cast<const P*>(in.px)[idx];
      s_py[ly][lx] = static_cast<const P*>(in.py)[idx];
      s_qxx[ly][lx] = static_cast<const P*>(in.qxx)[idx];
      s_qyy[ly][lx] = static_cast<const P*>(in.qyy)[idx];
      s_qxy[ly][lx] = static_cast<const P*>(in.qxy)[idx];
    }
  }
  __syncthreads();

  for (int i = tid; i < (TX + 1) * (TY + 1); i += NT) {
    const int ly = i / (TX + 1), lx = i - ly * (TX + 1);
    const int gx = x0 + lx, gy = y0 + ly;
    if (gx >= W || gy >= H) continue;
    const size_t idx = (size_t)gy * W + gx;
    const int sx = lx + 1, sy = ly + 1;  // position in the dual tiles
    // TV_primal_u_kernel (tgv_kernels.cuh:568-605)
    const P uo = static_cast<const P*>(in.u)[idx];
    const P d = div_minus<P, TX + 2>(s_px, s_py, sx, sy, gx, gy, W, H);
    P un = uo + tau * (d + lambda * f[idx]);
    un = un * (1.0f / (1.0f + tau * lambda));
    const P ubn = 2.0f * un - uo;
    // TGV_primal_v_kernel (tgv_kernels.cuh:647-686)
    const P vxo = static_cast<const P*>(in.vx)[idx], vyo = static_cast<const P*>(in.vy)[idx];
    const P dqxx = (gx > 0) ? ((gx < W - 1) ? s_qxx[sy][sx] - s_qxx[sy][sx - 1] : -s_qxx[sy][sx - 1]) : s_qxx[sy][sx];
    const P dqyy = (gy > 0) ? ((gy < H - 1) ? s_qyy[sy][sx] - s_qyy[sy - 1][sx] : -s_qyy[sy - 1][sx]) : s_qyy[sy][sx];
    const P dqxyx = (gx > 0) ? ((gx < W - 1) ? s_qxy[sy][sx] - s_qxy[sy][sx - 1] : -s_qxy[sy][sx - 1]) : s_qxy[sy][sx];
    const P dqxyy = (gy > 0) ? ((gy < H - 1) ? s_qxy[sy][sx] - s_qxy[sy - 1][sx] : -s_qxy[sy - 1][sx]) : s_qxy[sy][sx];
    const P vxn = vxo + tau * ((dqxx + dqxyy) + s_px[sy][sx]);
    const P vyn = vyo + tau * ((dqyy + dqxyx) + s_py[sy][sx]);
    const P vbxn = 2.0f * vxn - vxo, vbyn = 2.0f * vyn - vyo;
    s_ub[ly][lx] = ubn;
    s_vbx[ly][lx] = vbxn;
    s_vby[ly][lx] = vbyn;
    if (lx < TX && ly < TY) {
      static_cast<P*>(out.u)[idx] = un;
      static_cast<P*>(out.ub)[idx] = ubn;
      static_cast<P*>(out.vx)[idx] = vxn;
      static_cast<P*>(out.vy)[idx] = vyn;
      static_cast<P*>(out.vbx)[idx] = vbxn;
      static_cast<P*>(out.vby)[idx] = vbyn;
    }
  }
  __syncthreads();

  const int lx = tid % TX, ly = tid / TX;
  const int gx = x0 + lx, gy = y0 + ly;
  if (gx < W && gy < H) {
    const size_t idx = (size_t)gy * W + gx;
    const int xp = lx + (gx < W - 1), yp = ly + (gy < H - 1);
    // TGV_dual_p_kernel (tgv_kernels.cuh:260-292)
    const P c = s_ub[ly][lx];
    const P a = s_px[ly + 1][lx + 1] + sigma * ((s_ub[ly][xp] - c) - s_vbx[ly][lx]);
    const P b = s_py[ly + 1][lx + 1] + sigma * ((s_ub[yp][lx] - c) - s_vby[ly][lx]);
    const float sp = proj_scale(sqrtf(abs2(a) + abs2(b)), alpha1);
    static_cast<P*>(out.px)[idx] = a * sp;
    static_cast<P*>(out.py)[idx] = b * sp;
    // TGV_dual_q_kernel (tgv_kernels.cuh:225-258)
    const P vx = s_vbx[ly][lx], vy = s_vby[ly][lx];
    const P gxx = s_vbx[ly][xp] - vx;
    const P gxy = 0.5f * (s_vbx[yp][lx] - vx + s_vby[ly][xp] - vy);
    const P gyy = s_vby[yp][lx] - vy;
    const P qa = s_qxx[ly + 1][lx + 1] + sigma * gxx;
    const P qb = s_qyy[ly + 1][lx + 1] + sigma * gyy;
    const P qc = s_qxy[ly + 1][lx + 1] + sigma * gxy;
    const float sq = proj_scale(sqrtf(abs2(qa) + abs2(qb) + 2.0f * abs2(qc)), alpha0);
    static_cast<P*>(out.qxx)[idx] = qa * sq;
    static_cast<P*>(out.qyy)[idx] = qb * sq;
    static_cast<P*>(out.qxy)[idx] = qc * sq;
  }
}

// ------------------------------------------------------------------------------------------------
// TgvMriOptimizer / TgvOptimizerWithOp / TvOptimizerWithOp image side (dual first, K^H r given), as two
// kernels so that the dual update runs concurrently with the operator chain (it needs only u-bar and
// v-bar of the previous iteration):
//   dual    p <- proj_a1(p + sigma (grad+ ub - vb)),  q <- proj_a0(q + sigma eps(vb))   (in -> out)
//   primal  u+ = u + tau (div- p - K^H r),            v+ = v + tau (div_h- q + p)       (p, q from out)
// u and v are read only at their own pixel and update in place; u-bar and v-bar go to `out`.
// iter[0] is the iteration index (incremented by the primal kernel, which runs after the dual kernel
// has read it), iter[1] the length of the alpha table, iter[2] the non-finite flag: the primal kernel
// sets it to 1 when a new u or v is not finite (NaN or infinite data or operator output propagate
// into u within an iteration or two); the host reads and clears it.
// ------------------------------------------------------------------------------------------------
template <bool TGV>
__global__ void __launch_bounds__(NT) mri_dual_kernel(int W, int H, ImgPtrs in, ImgPtrs out, float sigma,
                                                      const float* __restrict__ alpha_tab,
                                                      const int* __restrict__ iter) {
  const int x = blockIdx.x * TX + threadIdx.x % TX, y = blockIdx.y * TY + threadIdx.x / TX;
  if (x >= W || y >= H) return;
  float alpha0, alpha1;
  dual_alphas<TGV>(alpha_tab, iter, alpha0, alpha1);
  mri_dual_pixel<TGV>(W, H, in, out, sigma, alpha0, alpha1, x, y);
}

template <bool TGV>
__global__ void __launch_bounds__(NT) mri_primal_kernel(int W, int H, ImgPtrs out, const float2* __restrict__ khr,
                                                        int G, long long gstride, float tau, int* __restrict__ iter) {
  pdl_wait();  // K^H r comes from the previous kernel
  pdl_trigger();
  if (iter && blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) atomicAdd(iter, 1);
  const int x = blockIdx.x * TX + threadIdx.x % TX, y = blockIdx.y * TY + threadIdx.x / TX;
  if (x >= W || y >= H) return;
  const size_t idx = (size_t)y * W + x;
  float2 kh = khr[idx];
  for (int g = 1; g < G; ++g) kh += khr[idx + (size_t)g * gstride];
  if (!mri_primal_pixel<TGV>(W, H, out, x, y, kh, tau) && iter) iter[2] = 1;
}

__global__ void tick_kernel(int* tick) { atomicAdd(tick, 1); }

inline dim3 tile_grid(int W, int H) { return dim3((W + TX - 1) / TX, (H + TY - 1) / TY); }

}  // namespace

void launch_tv_step(bool complex_, int W, int H, const ImgPtrs& in, const ImgPtrs& out, const void* f, float tau,
                    float sigma, float lambda, cudaStream_t st) {
  if (complex_)
    tv_step_kernel<float2><<<tile_grid(W, H), NT, 0, st>>>(W, H, in, out, static_cast<const float2*>(f), tau, sigma,
                                                            lambda);
  else
    tv_step_kernel<float><<<tile_grid(W, H), NT, 0, st>>>(W, H, in, out, static_cast<const float*>(f), tau, sigma,
                                                           lambda);
  PDT_LAUNCH_CHECK();
  count_launch();
}

void launch_tv_multi_step(bool complex_, int W, int H, const ImgPtrs& in, const ImgPtrs& out, const void* f,
                          float tau, float sigma, float lambda, cudaStream_t st) {
  const dim3 grid((W + 31) / 32, (H + 15) / 16);
  if (complex_)
    tv_multi_kernel<float2, kTvStepsPerLaunch><<<grid, NT, 0, st>>>(W, H, in, out, static_cast<const float2*>(f),
                                                                    tau, sigma, lambda);
  else
    tv_multi_kernel<float, kTvStepsPerLaunch><<<grid, NT, 0, st>>>(W, H, in, out, static_cast<const float*>(f), tau,
                                                                   sigma, lambda);
  PDT_LAUNCH_CHECK();
  count_launch();
}

void launch_tgv_denoise_step(bool complex_, int W, int H, const ImgPtrs& in, const ImgPtrs& out, const void* f,
                             float tau, float sigma, float lambda, float alpha0, float alpha1, cudaStream_t st) {
  if (complex_)
    tgv_denoise_step_kernel<float2><<<tile_grid(W, H), NT, 0, st>>>(W, H, in, out, static_cast<const float2*>(f),
                                                                     tau, sigma, lambda, alpha0, alpha1);
  else
    tgv_denoise_step_kernel<float><<<tile_grid(W, H), NT, 0, st>>>(W, H, in, out, static_cast<const float*>(f), tau,
                                                                    sigma, lambda, alpha0, alpha1);
  PDT_LAUNCH_CHECK();
  count_launch();
}

void launch_mri_dual(bool tgv, int W, int H, const ImgPtrs& in, const ImgPtrs& out, float sigma,
                     const float* alpha_tab, const int* iter, cudaStream_t st) {
  if (tgv)
    mri_dual_kernel<true><<<tile_grid(W, H), NT, 0, st>>>(W, H, in, out, sigma, alpha_tab, iter);
  else
    mri_dual_kernel<false><<<tile_grid(W, H), NT, 0, st>>>(W, H, in, out, sigma, alpha_tab, iter);
  PDT_LAUNCH_CHECK();
  count_launch();
}

void launch_mri_primal(bool tgv, int W, int H, const ImgPtrs& out, const float2* khr, int G, long long gstride,
                       float tau, int* iter, cudaStream_t st) {
  LaunchEx lx(tile_grid(W, H), dim3(NT), 0, st);
  if (tgv)
    PDT_CUDA_CHECK(cudaLaunchKernelEx(&lx.cfg, mri_primal_kernel<true>, W, H, out, khr, G, gstride, tau, iter));
  else
    PDT_CUDA_CHECK(cudaLaunchKernelEx(&lx.cfg, mri_primal_kernel<false>, W, H, out, khr, G, gstride, tau, iter));
  count_launch();
}

void launch_tick(int* tick, cudaStream_t st) {
  tick_kernel<<<1, 1, 0, st>>>(tick);
  PDT_LAUNCH_CHECK();
  count_launch();
}

void launch_fill_zero(void* p, size_t bytes, cudaStream_t st) {
  if (bytes) PDT_CUDA_CHECK(cudaMemsetAsync(p, 0, bytes, st));
}

}  // namespace pdt
