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

// partial[b] = sum over this block's elements of Re(a . conj(b))
__global__ void __launch_bounds__(kRedThreads) dot_re_kernel(const float2* __restrict__ a, const float2* __restrict__ b,
                                                            size_t n, double* __restrict__ partial) {
  double s = 0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    s += (double)a[i].x * b[i].x + (double)a[i].y * b[i].y;
  s = block_sum(s);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

// Optimality residuals of the with-operator saddle point, as partial sums of squares:
//   partial[2 b]     = sum |div- p - K^H r|^2            (u-stationarity: the primal u step is zero)
//   partial[2 b + 1] = sum |p + div_h- q|^2              (v-stationarity; TGV only)
// with the reference's div- boundary rules (x == 0: p(0); x == W-1: -p(W-2); else p(x) - p(x-1)).
__device__ __forceinline__ float2 dm_at(const float2* __restrict__ f, size_t i, int pos, int n, size_t step) {
  return (pos > 0) ? ((pos < n - 1) ? f[i] - f[i - step] : -f[i - step]) : f[i];
}
__global__ void __launch_bounds__(kRedThreads) kkt_kernel(int W, int H, const float2* __restrict__ khr,
                                                         const float2* __restrict__ px, const float2* __restrict__ py,
                                                         const float2* __restrict__ qxx, const float2* __restrict__ qyy,
                                                         const float2* __restrict__ qxy, double* __restrict__ partial) {
  double su = 0, sv = 0;
  const size_t n = (size_t)W * H;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int x = (int)(i % W), y = (int)(i / W);
    const float2 d = dm_at(px, i, x, W, 1) + dm_at(py, i, y, H, (size_t)W);
    su += ddist2(d, khr[i]);
    if (qxx) {
      const float2 dx = dm_at(qxx, i, x, W, 1) + dm_at(qxy, i, y, H, (size_t)W);
      const float2 dy = dm_at(qyy, i, y, H, (size_t)W) + dm_at(qxy, i, x, W, 1);
      sv += ddist2(c2(-px[i].x, -px[i].y), dx) + ddist2(c2(-py[i].x, -py[i].y), dy);
    }
  }
  su = block_sum(su);
  __syncthreads();
  sv = block_sum(sv);
  if (threadIdx.x == 0) {
    partial[2 * blockIdx.x] = su;
    partial[2 * blockIdx.x + 1] = sv;
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

// Sum of Re(a . conj(b)) over n complex elements, in double. Synchronises `st`.
double reduce_dot_re(const float2* a, const float2* b, size_t n, cudaStream_t st) {
  DevBuf part;
  part.ensure(kRedBlocks * sizeof(double));
  dot_re_kernel<<<kRedBlocks, kRedThreads, 0, st>>>(a, b, n, part.as<double>());
  PDT_LAUNCH_CHECK();
  count_launch();
  std::vector<double> h(kRedBlocks);
  PDT_CUDA_CHECK(cudaMemcpyAsync(h.data(), part.p, kRedBlocks * sizeof(double), cudaMemcpyDeviceToHost, st));
  PDT_CUDA_CHECK(cudaStreamSynchronize(st));
  double s = 0;
  for (double v : h) s += v;
  return s;
}

// {sum |div- p - K^H r|^2, sum |p + div_h- q|^2} (q null: second entry 0), in double. Synchronises `st`.
void reduce_kkt(int W, int H, const float2* khr, const float2* px, const float2* py, const float2* qxx,
                const float2* qyy, const float2* qxy, double out[2], cudaStream_t st) {
  DevBuf part;
  part.ensure(2 * kRedBlocks * sizeof(double));
  kkt_kernel<<<kRedBlocks, kRedThreads, 0, st>>>(W, H, khr, px, py, qxx, qyy, qxy, part.as<double>());
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
