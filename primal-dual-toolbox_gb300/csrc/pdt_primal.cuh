// pdt_primal.cuh -- the primal update of the with-operator solvers at one pixel, shared by the image
// kernel (mri_primal_kernel) and the tensor-core adjoint rows that fuse it into their epilogue.
//   u+ = u + tau (div- p - K^H r),  u-bar = 2 u+ - u                     (tgv_kernels.cuh:432-467)
//   v+ = v + tau (div_h- q + p),    v-bar = 2 v+ - v   (TGV only)        (tgv_kernels.cuh:647-686)
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

template <bool TGV>
__device__ __forceinline__ void mri_primal_pixel(int W, int H, const ImgPtrs& out, int x, int y, float2 kh,
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
  }
}

}  // namespace pdt
