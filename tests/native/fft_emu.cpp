// Host emulation harness for the engine's device FFT (pdt_device.cuh): compiles the device code with a
// C++ compiler, one "thread" per block and no-op barriers (exact for Stockham passes, which read one
// buffer and write the other). Used by tests/test_fft_emulated.py to check the FFT plan and butterflies
// against numpy on the CPU before any GPU run.
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <mutex>
#include <thread>
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

// ---- register FFTs and the two-level transform (pdt_regfft.cuh) ------------------------------------
#include "../../primal-dual-toolbox_gb300/csrc/pdt_regfft.cuh"

template <int A, int B>
static void twolevel(float* data, int inverse) {
  using T = pdt::TwoLevel<A, B>;
  constexpr int n = A * B;
  std::vector<float2> tw(n), ex(T::xch);
  pdt::fill_twiddles(n, tw.data());
  std::vector<float2> x(n);
  for (int i = 0; i < n; ++i) x[i] = {data[2 * i], data[2 * i + 1]};
  if (!inverse) {
    for (int a = 0; a < A; ++a) {
      float2 v[B];
      for (int b = 0; b < B; ++b) v[b] = x[a + A * b];
      T::fwd_step1(v, a, ex.data(), tw.data());
    }
    for (int kb = 0; kb < B; ++kb) {
      float2 u[A];
      T::fwd_step2(u, kb, ex.data(), tw.data());
      for (int ka = 0; ka < A; ++ka) x[kb + B * ka] = u[ka];
    }
  } else {
    std::vector<float2> z(n);
    for (int kb = 0; kb < B; ++kb) {
      float2 u[A];
      for (int ka = 0; ka < A; ++ka) u[ka] = x[kb + B * ka];
      T::inv_step1(u, kb, ex.data(), tw.data());
    }
    for (int a = 0; a < A; ++a) {
      float2 v[B];
      T::inv_step2(v, a, ex.data(), tw.data());
      for (int b = 0; b < B; ++b) z[a + A * b] = v[b];
    }
    x = z;
  }
  for (int i = 0; i < n; ++i) {
    data[2 * i] = x[i].x;
    data[2 * i + 1] = x[i].y;
  }
}

template <int N>
static void regfft(float* data, int inverse) {
  std::vector<float2> tw(N);
  pdt::fill_twiddles(N, tw.data());
  float2 v[N];
  for (int i = 0; i < N; ++i) v[i] = {data[2 * i], data[2 * i + 1]};
  pdt::reg_fft<N, 1>(v, tw.data(), inverse ? 1.f : -1.f);
  for (int i = 0; i < N; ++i) {
    data[2 * i] = v[i].x;
    data[2 * i + 1] = v[i].y;
  }
}

#define EMU_REG(N) if (n == N) { regfft<N>(data, inverse); return 0; }
extern "C" int emu_regfft(float* data, int n, int inverse) {
  EMU_REG(2) EMU_REG(3) EMU_REG(4) EMU_REG(5) EMU_REG(7) EMU_REG(8) EMU_REG(9) EMU_REG(10) EMU_REG(12)
  EMU_REG(16) EMU_REG(20) EMU_REG(23) EMU_REG(24) EMU_REG(32) EMU_REG(11) EMU_REG(13) EMU_REG(6)
  return 1;
}

#define EMU_TL(A, B) if (a == A && b == B) { twolevel<A, B>(data, inverse); return 0; }
extern "C" int emu_twolevel(float* data, int a, int b, int inverse) {
  EMU_TL(16, 23) EMU_TL(32, 20) EMU_TL(16, 20) EMU_TL(16, 16) EMU_TL(12, 16) EMU_TL(16, 24) EMU_TL(8, 8)
  EMU_TL(16, 12) EMU_TL(8, 16) EMU_TL(32, 24) EMU_TL(16, 32) EMU_TL(8, 12) EMU_TL(8, 20)
  return 1;
}

// ---- the lane-distributed transform (LaneFft, pdt_regfft.cuh): one host thread per lane ------------
namespace {
// L threads that meet at a barrier around every exchange, like the L lanes of a lane group
struct LaneGroup {
  int L = 0;
  std::vector<float2> slot;
  std::mutex mu;
  std::condition_variable cv;
  int count = 0;
  long gen = 0;
  void barrier() {
    std::unique_lock<std::mutex> lk(mu);
    const long g = gen;
    if (++count == L) {
      count = 0;
      ++gen;
      cv.notify_all();
    } else {
      cv.wait(lk, [&] { return gen != g; });
    }
  }
};
thread_local LaneGroup* g_group = nullptr;
thread_local int g_lane = 0;
}  // namespace

namespace pdt {
float2 shfl_xor2(float2 v, int m) {
  LaneGroup& G = *g_group;
  G.slot[g_lane] = v;
  G.barrier();
  const float2 r = G.slot[g_lane ^ m];
  G.barrier();
  return r;
}
void emu_sync64(int) { g_group->barrier(); }
}  // namespace pdt

// forward: natural order in, natural order out (each lane's X[k1 + M brev_L(t)] put back in place);
// inverse: the same order in reverse, unnormalised
template <int M, int L>
static void lanefft(float* data, int inverse) {
  using F = pdt::LaneFft<M, L>;
  constexpr int n = M * L;
  std::vector<float2> tw(n), out(n);
  pdt::fill_twiddles(n, tw.data());
  LaneGroup G;
  G.L = L;
  G.slot.resize(L);
  std::vector<std::thread> lanes;
  for (int t = 0; t < L; ++t)
    lanes.emplace_back([&, t] {
      g_group = &G;
      g_lane = t;
      float2 v[M];
      const int kb = M * pdt::lane_brev<L>(t);
      if (!inverse) {
        for (int j = 0; j < M; ++j) v[j] = {data[2 * (t + L * j)], data[2 * (t + L * j) + 1]};
        F::fwd(v, t, tw.data());
        for (int k1 = 0; k1 < M; ++k1) out[k1 + kb] = v[k1];
      } else {
        for (int k1 = 0; k1 < M; ++k1) v[k1] = {data[2 * (k1 + kb)], data[2 * (k1 + kb) + 1]};
        F::inv(v, t, tw.data());
        for (int j = 0; j < M; ++j) out[t + L * j] = v[j];
      }
    });
  for (auto& th : lanes) th.join();
  for (int i = 0; i < n; ++i) {
    data[2 * i] = out[i].x;
    data[2 * i + 1] = out[i].y;
  }
}

#define EMU_LANE(M, L) if (m == M && l == L) { lanefft<M, L>(data, inverse); return 0; }
extern "C" int emu_lanefft(float* data, int m, int l, int inverse) {
  EMU_LANE(4, 8) EMU_LANE(6, 8) EMU_LANE(8, 8) EMU_LANE(6, 16) EMU_LANE(8, 16) EMU_LANE(12, 16)
  EMU_LANE(16, 16) EMU_LANE(10, 32) EMU_LANE(46, 8) EMU_LANE(23, 16) EMU_LANE(12, 32) EMU_LANE(16, 32)
  EMU_LANE(20, 32) EMU_LANE(24, 32)
  return 1;
}

// the two-warp transform (LaneFft64): 64 threads, the cross-warp stage through a shared buffer
template <int M>
static void lanefft64(float* data, int inverse) {
  using F = pdt::LaneFft64<M>;
  constexpr int L = 64, n = M * L;
  std::vector<float2> tw(n), out(n), xbuf((size_t)M * 64);
  pdt::fill_twiddles(n, tw.data());
  LaneGroup G;
  G.L = L;
  G.slot.resize(L);
  std::vector<std::thread> lanes;
  for (int t = 0; t < L; ++t)
    lanes.emplace_back([&, t] {
      g_group = &G;
      g_lane = t;
      float2 v[M];
      const int kb = M * pdt::lane_brev<L>(t);
      if (!inverse) {
        for (int j = 0; j < M; ++j) v[j] = {data[2 * (t + L * j)], data[2 * (t + L * j) + 1]};
        F::fwd(v, t, tw.data(), xbuf.data(), 1);
        for (int k1 = 0; k1 < M; ++k1) out[k1 + kb] = v[k1];
      } else {
        for (int k1 = 0; k1 < M; ++k1) v[k1] = {data[2 * (k1 + kb)], data[2 * (k1 + kb) + 1]};
        F::inv(v, t, tw.data(), xbuf.data(), 1);
        for (int j = 0; j < M; ++j) out[t + L * j] = v[j];
      }
    });
  for (auto& th : lanes) th.join();
  for (int i = 0; i < n; ++i) {
    data[2 * i] = out[i].x;
    data[2 * i + 1] = out[i].y;
  }
}

extern "C" int emu_lanefft64(float* data, int m, int inverse) {
  if (m == 10) { lanefft64<10>(data, inverse); return 0; }
  if (m == 6) { lanefft64<6>(data, inverse); return 0; }
  return 1;
}
