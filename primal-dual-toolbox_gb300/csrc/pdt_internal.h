// pdt_internal.h -- host-side declarations shared by the engine's translation units.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <string>
#include <stdexcept>
#include <vector>

#include "pdt.h"

namespace pdt {

// Error carried to the C ABI as (status, message).
struct Error : std::runtime_error {
  pdt_status code;
  Error(pdt_status c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define PDT_CUDA_CHECK(call)                                                                         \
  do {                                                                                               \
    cudaError_t e_ = (call);                                                                         \
    if (e_ != cudaSuccess)                                                                           \
      throw ::pdt::Error(PDT_ERR_CUDA, std::string(#call) + " failed: " + cudaGetErrorString(e_));   \
  } while (0)

// Checks the launch that was just enqueued.
#define PDT_LAUNCH_CHECK() PDT_CUDA_CHECK(cudaGetLastError())

// Sets the message pdt_last_error() returns on this thread.
void set_last_error(const std::string& msg);

// Kernels launched by this library (graph replays add their kernel-node count).
extern std::atomic<uint64_t> g_launches;
inline void count_launch(uint64_t n = 1) { g_launches.fetch_add(n, std::memory_order_relaxed); }

// Owning device allocation.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  // (Re)allocates when the size changes; contents are undefined afterwards.
  void ensure(size_t n) {
    if (n == bytes && p) return;
    release();
    if (n == 0) return;
    cudaError_t e = cudaMalloc(&p, n);
    if (e != cudaSuccess) {
      p = nullptr;
      throw Error(PDT_ERR_ALLOC, "device allocation of " + std::to_string(n) + " bytes failed: " +
                                     cudaGetErrorString(e));
    }
    bytes = n;
  }
  template <class T> T* as() const { return static_cast<T*>(p); }
};

// ---------------------------------------------------------------------------------------------
// Image-side state: the primal u, v, their over-relaxations u-bar, v-bar and the duals p, q, each a
// planar W x H array (Variable2 / Variable2sym of optimizer_helper.h:30-224 as separate planes).
// ---------------------------------------------------------------------------------------------
struct ImgPtrs {
  void *u, *ub, *vx, *vy, *vbx, *vby, *px, *py, *qxx, *qyy, *qxy;
};

// One dual update of the with-operator solvers (p, q ascent and projections, state `in` -> `out`, the
// TGV weights from alpha_tab at the iteration counter iter[0]) handed to an operator round that runs it
// in otherwise idle blocks of one of its launches (SolverHooks::can_fuse_dual).
struct DualStep {
  ImgPtrs in, out;
  float sigma;
  const float* alpha_tab;
  const int* iter;
  int W, H;
  int tgv;  // 1: TGV (p and q), 0: TV (p only)
};

// Fused TvOptimizer iteration (tgv_kernels.cuh:294-324 then 568-605): reads u, u-bar and p from `in`,
// writes them to `out`.
void launch_tv_step(bool complex_, int W, int H, const ImgPtrs& in, const ImgPtrs& out, const void* f, float tau,
                    float sigma, float lambda, cudaStream_t st);
// kTvStepsPerLaunch TvOptimizer iterations in one launch (temporal blocking in shared memory); same
// arithmetic per pixel as launch_tv_step, state read from `in` and written to `out`.
constexpr int kTvStepsPerLaunch = 4;
void launch_tv_multi_step(bool complex_, int W, int H, const ImgPtrs& in, const ImgPtrs& out, const void* f,
                          float tau, float sigma, float lambda, cudaStream_t st);

// Fused TgvOptimizer iteration, primal first (tgvoptimizer.cu:117-137): every field ping-pongs.
void launch_tgv_denoise_step(bool complex_, int W, int H, const ImgPtrs& in, const ImgPtrs& out, const void* f,
                             float tau, float sigma, float lambda, float alpha0, float alpha1, cudaStream_t st);

// Image side of one TgvMri / TgvWithOp / TvWithOp iteration (tgvmrioptimizer.cu:177-197).
// Dual: p, q from u-bar, v-bar of `in` into `out`; alpha_tab[2k], alpha_tab[2k+1] = alpha0, alpha1 of
// iteration k = iter[0] (clamped to the table length iter[1]). It does not depend on K^H r, so it may
// run concurrently with the operator. tgv = false gives the TvOptimizerWithOp step (no v, q; unit-ball
// projection).
void launch_mri_dual(bool tgv, int W, int H, const ImgPtrs& in, const ImgPtrs& out, float sigma,
                     const float* alpha_tab, const int* iter, cudaStream_t st);
// Primal: u, v in place and u-bar, v-bar into `out` from the new p, q of `out` and K^H r (G partial
// sums spaced gstride elements apart); increments iter[0] when iter is non-null.
void launch_mri_primal(bool tgv, int W, int H, const ImgPtrs& out, const float2* khr, int G, long long gstride,
                       float tau, int* iter, cudaStream_t st);

// Programmatic dependent launch of the solver kernels (default on; PDT_LAUNCH_PDL=0 turns it off).
bool pdl_enabled();

// Launch configuration for cudaLaunchKernelEx: with pdl_enabled(), on an explicit stream, the kernel
// may be launched while its predecessor finishes (programmatic dependent launch; the kernel calls
// pdl_wait() before it reads the predecessor's results); cluster_y > 0 groups cluster_y blocks along y
// into a thread-block cluster.
struct LaunchEx {
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[2];
  LaunchEx(dim3 grid, dim3 block, size_t smem, cudaStream_t st, int cluster_y = 0) {
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = 0;
    if (st && pdl_enabled()) {
      attr[cfg.numAttrs].id = cudaLaunchAttributeProgrammaticStreamSerialization;
      attr[cfg.numAttrs].val.programmaticStreamSerializationAllowed = 1;
      ++cfg.numAttrs;
    }
    if (cluster_y > 0) {
      attr[cfg.numAttrs].id = cudaLaunchAttributeClusterDimension;
      attr[cfg.numAttrs].val.clusterDim.x = 1;
      attr[cfg.numAttrs].val.clusterDim.y = cluster_y;
      attr[cfg.numAttrs].val.clusterDim.z = 1;
      ++cfg.numAttrs;
    }
  }
};

// Records a CUDA event after each phase of an iteration (per-kernel timing); null in normal runs.
struct PhaseMarker {
  virtual ~PhaseMarker() = default;
  virtual void mark(const char* phase, cudaStream_t st) = 0;
};

// Element-wise helpers.
void launch_fill_zero(void* p, size_t bytes, cudaStream_t st);
// FP64 reductions (pdt_metrics.cu); they synchronise the stream.
double reduce_dist2(bool complex_, const void* a, const void* b, size_t n, cudaStream_t st);
void reduce_regularizer(bool complex_, const void* u, const void* vx, const void* vy, int W, int H, double out[2],
                        cudaStream_t st);
void launch_scale(float2* x, float s, size_t n, cudaStream_t st);
double reduce_dot_re(const float2* a, const float2* b, size_t n, cudaStream_t st);
void reduce_kkt(int W, int H, const float2* khr, const float2* px, const float2* py, const float2* qxx,
                const float2* qyy, const float2* qxy, double out[2], cudaStream_t st);
// *tick += 1 (one thread).
void launch_tick(int* tick, cudaStream_t st);

// Test hook of the bounded waits (pdt_debug_drop_arrival): the tensor-core kernels of the Cartesian
// operators and of the warm-start network withhold one arrival while it is on.
void cartesian_set_drop_arrival(int on);
void cnn_set_drop_arrival(int on);

}  // namespace pdt
