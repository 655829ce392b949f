// pdt_noalloc.cu -- the Cartesian forward operator for callers that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc: code running inside another framework's memory pool or under a
// strict device-memory budget, real-time loops that must not hit the allocator's synchronisation, and
// plugins whose host application owns every device allocation. pdt_cartesian_forward_noalloc serves
// them: the caller passes the inputs and the output, and the only scratch the computation needs (the
// k-space rows between the row and the column FFT passes) lives in one file-scope static device array
// of kNoAllocScratchBytes that every GPU which loads this library holds until the process exits.
// The FFT plans are factorised on the host and passed by value; the twiddle factors are written by a
// small kernel into a second, 64 KiB file-scope device table at the start of every call, so nothing
// else is allocated either.
//
// The arrays are shared by every call: a call overwrites every scratch and twiddle element it later
// reads, so nothing has to start at zero, but calls that overlap on the GPU (different streams, or
// different host threads) race on them. Serialise them.
#include <cmath>
#include <mutex>
#include <string>

#include "pdt_device.cuh"
#include "pdt_fftplan.h"
#include "pdt_internal.h"

namespace pdt {
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;  // 32 MiB
constexpr int kNoAllocMaxLen = 4096;                        // longest FFT the twiddle table holds
constexpr int kMaxDevices = 64;
constexpr int kNaThreads = 256;
constexpr int kNaRB = 4;  // image rows per block in the row pass
constexpr int kNaCB = 4;  // k-space columns per block in the column pass

// The scratch itself. In host code this name is only a stand-in for the symbol: its device address
// comes from cudaGetSymbolAddress (noalloc_device below).
static __device__ __align__(256) float2 g_noalloc_scratch[kNoAllocScratchBytes / sizeof(float2)];
// Twiddle factors of the row FFT (first kNoAllocMaxLen entries) and of the column FFT (the rest). Only
// device code names it.
static __device__ __align__(256) float2 g_noalloc_tw[2 * kNoAllocMaxLen];

// Per-device set-up, done once under g_noalloc_mu: the scratch's device address and the kernels'
// shared-memory limit. A cudaDeviceReset invalidates it; the library does not expect one between calls.
struct NaDevice {
  float2* scratch = nullptr;
  bool ready = false;
};
std::mutex g_noalloc_mu;
NaDevice g_noalloc_dev[kMaxDevices];

// tw[t] = exp(-2 pi i t / n) for the row (n = W) and column (n = H) transforms, in double.
__global__ void na_twiddles_kernel(int W, int H) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= W + H) return;
  const int n = i < W ? W : H;
  const int t = i < W ? i : i - W;
  double sn, cs;
  sincospi(-2.0 * (double)t / (double)n, &sn, &cs);
  g_noalloc_tw[(i < W ? 0 : kNoAllocMaxLen) + t] = c2((float)cs, (float)sn);
}

__device__ void load_twiddles(int n, int off, float2* tw) {
  for (int t = threadIdx.x; t < n; t += blockDim.x) tw[t] = g_noalloc_tw[off + t];
}

struct NaGeom {
  int W, Hf, C, Hi, y0;
  int mxW, mxH, oxW, oyH;
  float scale;
};

// Row pass: ubar rows (x sens_c) -> FFT along W -> scratch[c][kx][yi] for every FFT slot kx.
__global__ void __launch_bounds__(kNaThreads) na_rows_kernel(NaGeom g, FftPlan plan, const float2* __restrict__ sens,
                                                             const float2* __restrict__ img,
                                                             float2* __restrict__ scratch) {
  extern __shared__ float2 sm[];
  const int ld = g.W + 1;
  float2* tw = sm;
  float2* A = tw + g.W;
  float2* B = A + kNaRB * ld;
  load_twiddles(g.W, 0, tw);
  const int yi0 = blockIdx.x * kNaRB;
  const int c = blockIdx.y;
  const int nr = min(kNaRB, g.Hi - yi0);
  for (int i = threadIdx.x; i < nr * g.W; i += blockDim.x) {
    const int r = i / g.W, x = i - r * g.W;
    const int yi = yi0 + r;
    float2 v = img[(size_t)yi * g.W + x];
    if (sens) v = cmul(v, sens[((size_t)c * g.Hf + yi + g.y0) * g.W + x]);
    int slot = x + g.mxW;
    if (slot >= g.W) slot -= g.W;
    A[r * ld + slot] = v;
  }
  __syncthreads();
  const float2* X = smem_fft(A, B, nr, ld, plan, tw, false);
  for (int i = threadIdx.x; i < g.W * nr; i += blockDim.x) {
    const int k = i / nr, r = i - k * nr;
    scratch[((size_t)c * g.W + k) * g.Hi + yi0 + r] = X[r * ld + k];
  }
}

// Column pass: FFT along Hf of every k-space column, orthonormal scale, fftshift, mask -> dense output.
__global__ void __launch_bounds__(kNaThreads) na_cols_kernel(NaGeom g, FftPlan plan, const float* __restrict__ mask,
                                                             const float2* __restrict__ scratch,
                                                             float2* __restrict__ kspace) {
  extern __shared__ float2 sm[];
  const int ld = g.Hf + 1;
  float2* tw = sm;
  float2* A = tw + g.Hf;
  float2* B = A + kNaCB * ld;
  load_twiddles(g.Hf, kNoAllocMaxLen, tw);
  const int k0 = blockIdx.x * kNaCB;
  const int c = blockIdx.y;
  const int ncb = min(kNaCB, g.W - k0);
  for (int i = threadIdx.x; i < ncb * g.Hf; i += blockDim.x) {
    const int cb = i / g.Hf, j = i - cb * g.Hf;
    int yf = j - g.mxH;
    if (yf < 0) yf += g.Hf;
    const int yi = yf - g.y0;
    A[cb * ld + j] = (yi >= 0 && yi < g.Hi) ? scratch[((size_t)c * g.W + k0 + cb) * g.Hi + yi] : c2(0.f, 0.f);
  }
  __syncthreads();
  const float2* X = smem_fft(A, B, ncb, ld, plan, tw, false);
  for (int i = threadIdx.x; i < ncb * g.Hf; i += blockDim.x) {
    const int cb = i / g.Hf, ky = i - cb * g.Hf;
    int ypos = ky + g.oyH;
    if (ypos >= g.Hf) ypos -= g.Hf;
    int xpos = k0 + cb + g.oxW;
    if (xpos >= g.W) xpos -= g.W;
    kspace[((size_t)c * g.Hf + ypos) * g.W + xpos] = X[cb * ld + ky] * g.scale * mask[(size_t)ypos * g.W + xpos];
  }
}

// Device address of the scratch on the current device; the first call on a device resolves it and
// raises the kernels' dynamic shared-memory limit, under one lock.
float2* noalloc_device(int dev, int max_smem) {
  if (dev < 0 || dev >= kMaxDevices) throw Error(PDT_ERR_UNSUPPORTED, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  NaDevice& d = g_noalloc_dev[dev];
  if (!d.ready) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess)
      throw Error(PDT_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch) failed: ") + cudaGetErrorString(e));
    PDT_CUDA_CHECK(cudaFuncSetAttribute(na_rows_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem - 1024));
    PDT_CUDA_CHECK(cudaFuncSetAttribute(na_cols_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem - 1024));
    d.scratch = static_cast<float2*>(p);
    d.ready = true;
  }
  return d.scratch;
}

}  // namespace
}  // namespace pdt

using namespace pdt;

extern "C" pdt_status pdt_cartesian_forward_noalloc(int roos, const void* sens, const void* mask, int W, int H, int C,
                                                    const void* img, void* kspace, void* stream) {
  try {
    if (W < 1 || H < 1 || C < 1) throw Error(PDT_ERR_INVALID_ARGUMENT, "W, H and C must be positive");
    if (!sens || !mask || !img || !kspace) throw Error(PDT_ERR_INVALID_ARGUMENT, "null device pointer");
    if (roos && (H % 2 || H < 4)) throw Error(PDT_ERR_SIZE, "readout-oversampling removal needs an even H >= 4");
    NaGeom g;
    g.W = W;
    g.Hf = H;
    g.C = C;
    if (roos) {
      g.Hi = H / 2;
      g.y0 = (int)(unsigned int)((float)(unsigned int)H * 0.25f + 1.f);  // mricartesianoperator.cu:341
    } else {
      g.Hi = H;
      g.y0 = 0;
    }
    g.mxW = (int)(((float)W + 1.f) / 2.f);
    g.mxH = (int)(((float)H + 1.f) / 2.f);
    g.oxW = W / 2;
    g.oyH = H / 2;
    g.scale = (float)(1.0 / std::sqrt((double)W * (double)H));
    const size_t need = (size_t)C * W * g.Hi * sizeof(float2);
    if (need > kNoAllocScratchBytes)
      throw Error(PDT_ERR_UNSUPPORTED, "pdt_cartesian_forward_noalloc: coils x W x image rows x 8 bytes = " +
                                           std::to_string(need) + " exceeds the " +
                                           std::to_string(kNoAllocScratchBytes) + "-byte static scratch");
    if (W > kNoAllocMaxLen || H > kNoAllocMaxLen)
      throw Error(PDT_ERR_UNSUPPORTED, "pdt_cartesian_forward_noalloc: W and H must be at most " +
                                           std::to_string(kNoAllocMaxLen));
    FftPlan plan_w, plan_h;
    if (!make_fft_plan(W, &plan_w) || !make_fft_plan(H, &plan_h))
      throw Error(PDT_ERR_UNSUPPORTED, "pdt_cartesian_forward_noalloc: no FFT plan for these lengths");
    const size_t smem_rows = sizeof(float2) * ((size_t)W + 2 * (size_t)kNaRB * (W + 1));
    const size_t smem_cols = sizeof(float2) * ((size_t)H + 2 * (size_t)kNaCB * (H + 1));
    int dev = 0, max_smem = 0;
    PDT_CUDA_CHECK(cudaGetDevice(&dev));
    PDT_CUDA_CHECK(cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    if (smem_rows > (size_t)max_smem - 1024 || smem_cols > (size_t)max_smem - 1024)
      throw Error(PDT_ERR_UNSUPPORTED, "pdt_cartesian_forward_noalloc: FFT length too large for shared memory");
    float2* scratch = noalloc_device(dev, max_smem);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    na_twiddles_kernel<<<(W + H + 255) / 256, 256, 0, st>>>(W, H);
    PDT_LAUNCH_CHECK();
    count_launch();
    na_rows_kernel<<<dim3((g.Hi + kNaRB - 1) / kNaRB, C), kNaThreads, smem_rows, st>>>(
        g, plan_w, static_cast<const float2*>(sens), static_cast<const float2*>(img), scratch);
    PDT_LAUNCH_CHECK();
    count_launch();
    na_cols_kernel<<<dim3((W + kNaCB - 1) / kNaCB, C), kNaThreads, smem_cols, st>>>(
        g, plan_h, static_cast<const float*>(mask), scratch, static_cast<float2*>(kspace));
    PDT_LAUNCH_CHECK();
    count_launch();
    return PDT_OK;
  } catch (const Error& e) {
    set_last_error(e.what());
    return e.code;
  } catch (const std::exception& e) {
    set_last_error(e.what());
    return PDT_ERR_INVALID_ARGUMENT;
  }
}
