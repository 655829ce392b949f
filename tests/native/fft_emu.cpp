// Host emulation harness for the engine's device FFT (pdt_device.cuh): compiles the device code with a
// C++ compiler, one "thread" per block and no-op barriers (exact for Stockham passes, which read one
// buffer and write the other). Used by tests/test_fft_emulated.py to check the FFT plan and butterflies
// against numpy on the CPU before any GPU run.
#include <cmath>
#include <cstring>
#include <vector>
struct float2 { float x, y; };
inline float2 make_float2(float a, float b) { return {a, b}; }
struct dim3_ { unsigned x = 0, y = 0, z = 0; };
static dim3_ threadIdx, blockDim;
inline void __syncthreads() {}
#define __host__
#define __device__
#define __forceinline__ inline
#define __noinline__
#define __restrict__
#define cudaStream_t void*
#define PDT_HOST_EMULATION 1
#include "../../primal-dual-toolbox_gb300/csrc/pdt_device.cuh"
#include "../../primal-dual-toolbox_gb300/csrc/pdt_fftplan.h"

extern "C" int emu_fft(float* data, int n, int nseq, int inverse) {
  pdt::FftPlan pl;
  if (!pdt::make_fft_plan(n, &pl)) return 1;
  std::vector<float2> tw(n);
  pdt::fill_twiddles(n, tw.data());
  const int ld = n + 1;
  std::vector<float2> a((size_t)ld * nseq), b((size_t)ld * nseq);
  for (int s = 0; s < nseq; ++s)
    for (int i = 0; i < n; ++i) a[(size_t)s * ld + i] = {data[2 * ((size_t)s * n + i)], data[2 * ((size_t)s * n + i) + 1]};
  threadIdx.x = 0;
  blockDim.x = 1;
  float2* out = pdt::smem_fft(a.data(), b.data(), nseq, ld, pl, tw.data(), inverse != 0);
  for (int s = 0; s < nseq; ++s)
    for (int i = 0; i < n; ++i) {
      data[2 * ((size_t)s * n + i)] = out[(size_t)s * ld + i].x;
      data[2 * ((size_t)s * n + i) + 1] = out[(size_t)s * ld + i].y;
    }
  return 0;
}
