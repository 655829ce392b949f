// pdt_metrics.cu -- the engine's FP64 reductions: energies, norms and distances of FP32 fields,
// accumulated in double (the iterations themselves stay FP32).
//
//   TGV^2 energy  E(u, v) = 1/2 ||K u - f||^2 + alpha1 sum |grad+ u - v| + alpha0 sum |eps(v)|_F
//   TV energy     E(u)    = lambda/2 ||u - f||^2 + sum |grad+ u|
// with |.| the pointwise Euclidean norms the reference's projections use (tgv_kernels.cuh:136-165:
// |eps(v)|_F^2 = |xx|^2 + |yy|^2 + 2 |xy|^2) and the same Neumann forward differences.
#include "pdt_device.cuh"
#include "pdt_internal.h"

namespace pdt {
namespace {

constexpr int kRedThreads = 256;
constexpr int kRedBlocks = 592;  // 4 x 148-152 SMs

__device__ __forceinline__ double dabs2(float2 a) { return (double)a.x * a.x + (double)a.y * a.y; }
__device__ __forceinline__ double dabs2(float a) { return (double)a * a; }
// |a - b|^2 with the difference taken in double (exact for FP32 inputs)
__device__ __forceinline__ double ddist2(float2 a, float2 b) {
  const double dx = (double)a.x - (double)b.x, dy = (double)a.y - (double)b.y;
  return dx * dx + dy * dy;
}
__device__ __forceinline__ double ddist2(float a, float b) {
  const double d = (double)a - (double)b;
  return d * d;
}

__device__ double block_sum(double v) {
  __shared__ double sh[kRedThreads / 32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0;
  if (threadIdx.x < 32) {
    t = threadIdx.x < (int)(blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
  }
  return t;
}

// partial[b] = sum over this block's elements of |a - b|^2 (b may be null)
template <class P>
__global__ void __launch_bounds__(kRedThreads) dist2_kernel(const P* __restrict__ a, const P* __restrict__ b,
                                                            size_t n, double* __restrict__ partial) {
  double s = 0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    s += b ? ddist2(a[i], b[i]) : dabs2(a[i]);
  }
  s = block_sum(s);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

// partial[2 b] = sum |grad+ u - v|, partial[2 b + 1] = sum |eps(v)|_F  (v null: TV, |grad+ u|)
template <class P>
__global__ void __launch_bounds__(kRedThreads) regularizer_kernel(const P* __restrict__ u, const P* __restrict__ vx,
                                                                  const P* __restrict__ vy, int W, int H,
                                                                  double* __restrict__ partial) {
  double s1 = 0, s0 = 0;
  const size_t n = (size_t)W * H;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int x = (int)(i % W), y = (int)(i / W);
    const size_t ixp = i + (x < W - 1), iyp = i + (y < H - 1 ? (size_t)W : 0);
    P gx = u[ixp] - u[i], gy = u[iyp] - u[i];
    if (vx) {
      gx = gx - vx[i];
      gy = gy - vy[i];
      const P exx = vx[ixp] - vx[i], eyy = vy[iyp] - vy[i];
      const P exy = 0.5f * (vx[iyp] - vx[i] + vy[ixp] - vy[i]);
      s0 += sqrt(dabs2(exx) + dabs2(eyy) + 2.0 * dabs2(exy));
    }
    s1 += sqrt(dabs2(gx) + dabs2(gy));
  }
  s1 = block_sum(s1);
  __syncthreads();
  s0 = block_sum(s0);
  if (threadIdx.x == 0) {
    partial[2 * blockIdx.x] = s1;
    partial[2 * blockIdx.x + 1] = s0;
  }
}

__global__ void scale_kernel(float2* __restrict__ x, float s, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    x[i] = x[i] * s;
}

}  // namespace

void launch_scale(float2* x, float s, size_t n, cudaStream_t st) {
  scale_kernel<<<kRedBlocks, kRedThreads, 0, st>>>(x, s, n);
  PDT_LAUNCH_CHECK();
  count_launch();
}

// Sum of |a - b|^2 over n elements (b may be null), in double. Synchronises `st`.
double reduce_dist2(bool complex_, const void* a, const void* b, size_t n, cudaStream_t st) {
  DevBuf part;
  part.ensure(kRedBlocks * sizeof(double));
  if (complex_)
    dist2_kernel<float2><<<kRedBlocks, kRedThreads, 0, st>>>(static_cast<const float2*>(a),
                                                             static_cast<const float2*>(b), n, part.as<double>());
  else
    dist2_kernel<float><<<kRedBlocks, kRedThreads, 0, st>>>(static_cast<const float*>(a), static_cast<const float*>(b),
                                                            n, part.as<double>());
  PDT_LAUNCH_CHECK();
  count_launch();
  std::vector<double> h(kRedBlocks);
  PDT_CUDA_CHECK(cudaMemcpyAsync(h.data(), part.p, kRedBlocks * sizeof(double), cudaMemcpyDeviceToHost, st));
  PDT_CUDA_CHECK(cudaStreamSynchronize(st));
  double s = 0;
  for (double v : h) s += v;  // fixed order: deterministic
  return s;
}

// {sum |grad+ u - v|, sum |eps(v)|_F} (TV: {sum |grad+ u|, 0}), in double. Synchronises `st`.
void reduce_regularizer(bool complex_, const void* u, const void* vx, const void* vy, int W, int H, double out[2],
                        cudaStream_t st) {
  DevBuf part;
  part.ensure(2 * kRedBlocks * sizeof(double));
  if (complex_)
    regularizer_kernel<float2><<<kRedBlocks, kRedThreads, 0, st>>>(
        static_cast<const float2*>(u), static_cast<const float2*>(vx), static_cast<const float2*>(vy), W, H,
        part.as<double>());
  else
    regularizer_kernel<float><<<kRedBlocks, kRedThreads, 0, st>>>(static_cast<const float*>(u),
                                                                   static_cast<const float*>(vx),
                                                                   static_cast<const float*>(vy), W, H,
                                                                   part.as<double>());
  PDT_LAUNCH_CHECK();
  count_launch();
  std::vector<double> h(2 * kRedBlocks);
  PDT_CUDA_CHECK(cudaMemcpyAsync(h.data(), part.p, h.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
  PDT_CUDA_CHECK(cudaStreamSynchronize(st));
  out[0] = out[1] = 0;
  for (int b = 0; b < kRedBlocks; ++b) {
    out[0] += h[2 * b];
    out[1] += h[2 * b + 1];
  }
}

}  // namespace pdt
