// pdt_primal.cuh -- the per-pixel updates of the with-operator solvers (TgvMriOptimizer,
// TgvOptimizerWithOp, TvOptimizerWithOp), shared by the image kernels (mri_dual_kernel,
// mri_primal_kernel) and the tensor-core adjoint rows, whose otherwise idle blocks can run the dual update.
//   dual    p <- proj_a1(p + sigma (grad+ ub - vb)),  q <- proj_a0(q + sigma eps(vb))   (tgv_kernels.cuh:225-292)
//   primal  u+ = u + tau (div- p - K^H r),  u-bar = 2 u+ - u                     (tgv_kernels.cuh:432-467)
//           v+ = v + tau (div_h- q + p),    v-bar = 2 v+ - v   (TGV only)        (tgv_kernels.cuh:647-686)
// p and q are read at the pixel and its x-1 / y-1 neighbours; u and v update in place.
#pragma once

#include "pdt_device.cuh"
#include "pdt_internal.h"

namespace pdt {

// div- of a component at (x, y) along x (step 1) or y (step W) with the reference's boundary rows:
// f(0) at the first position, -f(n-2) at the last, f(i) - f(i-1) between.
__device__ __forceinline__ float2 bdiff(const float2* __restrict__ f, size_t idx, int pos, int n, size_t step) {
  return (pos > 0) ? ((pos < n - 1) ? f[idx] - f[idx - step] : -f[idx - step]) : f[idx];
}

// Returns false when the new u (or v) is not finite: the solvers' non-finite check, on values already
// in registers.
template <bool TGV>
__device__ __forceinline__ bool mri_primal_pixel(int W, int H, const ImgPtrs& out, int x, int y, float2 kh,
                                                 float tau) {
  const size_t idx = (size_t)y * W + x;
  const float2* px = static_cast<const float2*>(out.px);
  const float2* py = static_cast<const float2*>(out.py);
  float2* u = static_cast<float2*>(out.u);
  const float2 ou = u[idx];
  const float2 d = bdiff(px, idx, x, W, 1) + bdiff(py, idx, y, H, (size_t)W);
  const float2 un = ou + tau * (d - kh);
  u[idx] = un;
  static_cast<float2*>(out.ub)[idx] = 2.0f * un - ou;
  bool finite = isfinite(un.x) && isfinite(un.y);
  if constexpr (TGV) {
    const float2* qxx = static_cast<const float2*>(out.qxx);
    const float2* qyy = static_cast<const float2*>(out.qyy);
    const float2* qxy = static_cast<const float2*>(out.qxy);
    float2* vx = static_cast<float2*>(out.vx);
    float2* vy = static_cast<float2*>(out.vy);
    const float2 ovx = vx[idx], ovy = vy[idx];
    const float2 dqxx = bdiff(qxx, idx, x, W, 1), dqyy = bdiff(qyy, idx, y, H, (size_t)W);
    const float2 dqxyx = bdiff(qxy, idx, x, W, 1), dqxyy = bdiff(qxy, idx, y, H, (size_t)W);
    const float2 vxn = ovx + tau * ((dqxx + dqxyy) + px[idx]);
    const float2 vyn = ovy + tau * ((dqyy + dqxyx) + py[idx]);
    vx[idx] = vxn;
    vy[idx] = vyn;
    static_cast<float2*>(out.vbx)[idx] = 2.0f * vxn - ovx;
    static_cast<float2*>(out.vby)[idx] = 2.0f * vyn - ovy;
    finite = finite && isfinite(vxn.x) && isfinite(vxn.y) && isfinite(vyn.x) && isfinite(vyn.y);
  }
  return finite;
}

__device__ __forceinline__ float dual_proj_scale(float n, float alpha) { return 1.0f / fmaxf(1.0f, n / alpha); }

// The TGV weights (alpha0, alpha1) of the current iteration: the device table at the solver's iteration
// counter iter[0], clamped to the table length iter[1]. TV uses neither (1, 1).
template <bool TGV>
__device__ __forceinline__ void dual_alphas(const float* __restrict__ alpha_tab, const int* __restrict__ iter,
                                            float& alpha0, float& alpha1) {
  alpha0 = alpha1 = 1.f;
  if constexpr (TGV) {
    const int k = min(max(iter[0], 0), iter[1] - 1);
    alpha0 = alpha_tab[2 * k];
    alpha1 = alpha_tab[2 * k + 1];
  }
}

// The dual update at pixel (x, y): u-bar, v-bar, p, q from `in`; p, q to `out`.
template <bool TGV>
__device__ __forceinline__ void mri_dual_pixel(int W, int H, const ImgPtrs& in, const ImgPtrs& out, float sigma,
                                               float alpha0, float alpha1, int x, int y) {
  const size_t idx = (size_t)y * W + x;
  const bool xn = x < W - 1, yn = y < H - 1;
  const float2* ub = static_cast<const float2*>(in.ub);
  const float2 c = ub[idx];
  const float2 ux = xn ? ub[idx + 1] : c, uy = yn ? ub[idx + W] : c;
  const float2 pxo = static_cast<const float2*>(in.px)[idx], pyo = static_cast<const float2*>(in.py)[idx];
  float2 a, b;
  float2 vx, vy, vxx, vxy, vyx, vyy;
  if constexpr (TGV) {
    const float2* vbx = static_cast<const float2*>(in.vbx);
    const float2* vby = static_cast<const float2*>(in.vby);
    vx = vbx[idx];
    vy = vby[idx];
    vxx = xn ? vbx[idx + 1] : vx;
    vxy = yn ? vbx[idx + W] : vx;
    vyx = xn ? vby[idx + 1] : vy;
    vyy = yn ? vby[idx + W] : vy;
    a = pxo + sigma * ((ux - c) - vx);
    b = pyo + sigma * ((uy - c) - vy);
  } else {
    a = pxo + sigma * (ux - c);
    b = pyo + sigma * (uy - c);
  }
  const float sp = dual_proj_scale(sqrtf(abs2(a) + abs2(b)), alpha1);
  static_cast<float2*>(out.px)[idx] = a * sp;
  static_cast<float2*>(out.py)[idx] = b * sp;
  if constexpr (TGV) {
    const float2 gxx = vxx - vx;
    const float2 gxy = 0.5f * (vxy - vx + vyx - vy);
    const float2 gyy = vyy - vy;
    const float2 qa = static_cast<const float2*>(in.qxx)[idx] + sigma * gxx;
    const float2 qb = static_cast<const float2*>(in.qyy)[idx] + sigma * gyy;
    const float2 qc = static_cast<const float2*>(in.qxy)[idx] + sigma * gxy;
    const float sq = dual_proj_scale(sqrtf(abs2(qa) + abs2(qb) + 2.0f * abs2(qc)), alpha0);
    static_cast<float2*>(out.qxx)[idx] = qa * sq;
    static_cast<float2*>(out.qyy)[idx] = qb * sq;
    static_cast<float2*>(out.qxy)[idx] = qc * sq;
  }
}

// The whole dual update spread over `nd` blocks of another kernel's grid (block `db` of them): pixels
// in row-major order, block-strided, so that each warp reads and writes consecutive addresses.
template <bool TGV>
__device__ __forceinline__ void mri_dual_blocks(const DualStep& ds, int db, int nd) {
  float alpha0, alpha1;
  dual_alphas<TGV>(ds.alpha_tab, ds.iter, alpha0, alpha1);
  const int n = ds.W * ds.H, stride = nd * blockDim.x;
  for (int i = db * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int y = i / ds.W, x = i - y * ds.W;
    mri_dual_pixel<TGV>(ds.W, ds.H, ds.in, ds.out, ds.sigma, alpha0, alpha1, x, y);
  }
}

}  // namespace pdt
