// pdt_cartesian.cu -- Cartesian multi-coil MRI operators (plain and readout-oversampling removal) and
// the single-coil sampling operator, as three shared-memory FFT phases.
//
// Reference: MriCartesianOperator / MriCartesianRemoveROOSOperator (mricartesianoperator.cu:27-414)
// and MriSamplingOperator (mrisamplingoperator.cu:58-88):
//   forward  K u = mask . fftshift2( fft2( ifftshift2( pad(u) . sens_c ) ) / sqrt(W H) )
//   adjoint  K^H k = crop( sum_c conj(sens_c) . fftshift2( ifft2( ifftshift2( mask . k_c ) ) / sqrt(W H) ) )
// with ifftshift written as dst[(i + mid) % n] = src[i], mid = int((n+1)/2) (mricartesianoperator.cu:41-49),
// fftshift2 as dst[(i + n/2) % n] = src[i], and the ROOS image occupying frequency-encode rows
// [FE_idx, FE_idx + H/2) with FE_idx = unsigned(H * 0.25f + 1) (mricartesianoperator.cu:341).
//
// GB300 layout. W = phase-encode (contiguous), Hf = frequency-encode, C = coils. Shifts, padding and
// cropping are folded into the FFT load/store index maps, and only phase-encode columns with a
// non-zero mask entry ("sampled columns", ns of W) are ever transformed along Hf:
//   rows_fwd  (row blocks x coils)   ubar . sens -> FFT along W -> t[c][s][yi] for sampled columns
//   cols      (column blocks x coils) pruned FFT along Hf -> mask -> k-space dual prox -> mask -> IFFT
//   rows_adj  (row blocks x coil groups) t -> IFFT along W -> conj(sens) . -> coil sum
// The k-space dual r and the data f live in the compact layout [c][s][Hf] (sampled columns only);
// the entries of unsampled columns never reach u in the reference either (the mask zeroes them).
// Within a column the compact order is the output row for the generic kernels and the order the
// lane-distributed FFT leaves its spectrum in for the fast kernels (kperm maps one to the other).
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <mutex>
#include <sstream>

#include "pdt_cart_tiles.h"
#include "pdt_device.cuh"
#include "pdt_fftplan.h"
#include "pdt_ops.h"

namespace pdt {

namespace {

constexpr int kThreads = 256;

struct CartDev {
  int W, Hf, C, Hi, y0, ns;
  int mxW, mxH;  // ifftshift mids: int((n+1)/2)
  int oxW, oyH;  // fftshift mids: n/2
  float scale;   // 1/sqrt(W*Hf)
  int RB, CB, ldW, ldH;
  const float2* sens;   // (W, Hf, C) or null (sampling operator)
  const float* maskc;   // [ns][Hf] mask values of sampled columns, in compact order
  const int* kperm;     // [Hf] compact position -> output row (null: compact order = output row)
  const int* fwd_slot;  // [ns] forward-FFT output slot of sampled column s
  const int* col_x;     // [ns] k-space column of s
  const int* slot2s;    // [W] inverse-FFT input slot -> s (or -1)
  const int* fslot2s;   // [W] forward-FFT output slot -> s (or -1)
  const float2* twW;
  const float2* twH;
  FftPlan planW, planH;
  int tc_yb;  // tensor-core row passes: image rows per 128-row tile (the tile holds them for every coil)
};

enum ColMode { COL_SOLVE = 0, COL_FWD_DENSE = 1, COL_ADJ_DENSE = 2, COL_ADJ_COMPACT = 3 };

__device__ __forceinline__ int imod(int a, int n) {
  a %= n;
  return a < 0 ? a + n : a;
}

// Phase 1: rows of ubar (x sens_c) -> FFT along W; keep the sampled columns.
__global__ void __launch_bounds__(kThreads) rows_fwd_kernel(CartDev d, const float2* __restrict__ ubar,
                                                            float2* __restrict__ t1, int* __restrict__ tick) {
  if (tick && blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) atomicAdd(tick, 1);
  extern __shared__ float2 sm[];
  float2* tw = sm;
  float2* A = tw + d.W;
  float2* B = A + d.RB * d.ldW;
  const int yi0 = blockIdx.x * d.RB;
  const int c = blockIdx.y;
  const int nr = min(d.RB, d.Hi - yi0);
  for (int i = threadIdx.x; i < d.W; i += blockDim.x) tw[i] = d.twW[i];
  for (int i = threadIdx.x; i < nr * d.W; i += blockDim.x) {
    const int r = i / d.W, x = i - r * d.W;
    const int yi = yi0 + r;
    float2 v = ubar[(size_t)yi * d.W + x];
    if (d.sens) v = cmul(v, d.sens[((size_t)c * d.Hf + yi + d.y0) * d.W + x]);  // prefft_kernel
    int slot = x + d.mxW;
    if (slot >= d.W) slot -= d.W;
    A[r * d.ldW + slot] = v;
  }
  __syncthreads();
  const float2* X = smem_fft(A, B, nr, d.ldW, d.planW, tw, false);
  for (int i = threadIdx.x; i < d.ns * nr; i += blockDim.x) {
    const int s = i / nr, r = i - s * nr;
    t1[((size_t)c * d.ns + s) * d.Hi + yi0 + r] = X[r * d.ldW + d.fwd_slot[s]];
  }
}

// Phase 2: per sampled column, FFT along Hf (input non-zero on the Hi image rows), mask, and -- in
// solve mode -- the k-space dual prox r = (r + sigma (K u - f)) / (1 + sigma lambda) followed by the
// adjoint's mask . r -> IFFT along Hf restricted to the image rows.
__global__ void __launch_bounds__(kThreads) cols_kernel(CartDev d, int mode, const float2* t_in, float2* t_out,
                                                        float2* __restrict__ r, const float2* __restrict__ fc,
                                                        const float2* __restrict__ kin, float2* __restrict__ kout,
                                                        float sigma, float lambda) {
  extern __shared__ float2 sm[];
  float2* tw = sm;
  float2* A = tw + d.Hf;
  float2* B = A + d.CB * d.ldH;
  const int s0 = blockIdx.x * d.CB;
  const int c = blockIdx.y;
  const int ncb = min(d.CB, d.ns - s0);
  const int Hf = d.Hf;
  for (int i = threadIdx.x; i < Hf; i += blockDim.x) tw[i] = d.twH[i];

  float2* Y;  // inverse-FFT input buffer
  float2* Yo;
  if (mode == COL_SOLVE || mode == COL_FWD_DENSE) {
    for (int i = threadIdx.x; i < ncb * Hf; i += blockDim.x) {
      const int cb = i / Hf, j = i - cb * Hf;
      const int yf = imod(j - d.mxH, Hf);  // image row that lands in FFT slot j after ifftshift
      const int yi = yf - d.y0;
      float2 v = c2(0.f, 0.f);
      if (yi >= 0 && yi < d.Hi) v = t_in[((size_t)c * d.ns + s0 + cb) * d.Hi + yi];
      A[cb * d.ldH + j] = v;
    }
    __syncthreads();
    float2* X = smem_fft(A, B, ncb, d.ldH, d.planH, tw, false);
    Y = (X == A) ? B : A;
    for (int i = threadIdx.x; i < ncb * Hf; i += blockDim.x) {
      const int cb = i / Hf, ky = i - cb * Hf;
      const int s = s0 + cb;
      int ypos = ky + d.oyH;
      if (ypos >= Hf) ypos -= Hf;
      const float m = d.maskc[(size_t)s * Hf + ypos];
      const float2 k = X[cb * d.ldH + ky] * d.scale * m;  // fft2(..)/sqrt(N), fftshift2, applyMask
      if (mode == COL_FWD_DENSE) {
        kout[((size_t)c * Hf + ypos) * d.W + d.col_x[s]] = k;
      } else {
        const size_t o = ((size_t)c * d.ns + s) * Hf + ypos;
        // addWeighted(tmp, 1, f, -1) then TGV_prox_r_kernel (tgvmrioptimizer.cu:167-174)
        const float2 rn = (r[o] + sigma * (k - fc[o])) / (1.0f + sigma * lambda);
        r[o] = rn;
        Y[cb * d.ldH + imod(ypos + d.mxH, Hf)] = rn * m;  // preifft_kernel
      }
    }
    if (mode == COL_FWD_DENSE) return;
    Yo = X;
  } else {
    Y = A;
    Yo = B;
    for (int i = threadIdx.x; i < ncb * Hf; i += blockDim.x) {
      const int cb = i / Hf, ypos = i - cb * Hf;
      const int s = s0 + cb;
      const float m = d.maskc[(size_t)s * Hf + ypos];
      const float2 v = (mode == COL_ADJ_DENSE) ? kin[((size_t)c * Hf + ypos) * d.W + d.col_x[s]]
                                               : fc[((size_t)c * d.ns + s) * Hf + ypos];
      Y[cb * d.ldH + imod(ypos + d.mxH, Hf)] = v * m;
    }
  }
  __syncthreads();
  const float2* Z = smem_fft(Y, Yo, ncb, d.ldH, d.planH, tw, true);
  for (int i = threadIdx.x; i < ncb * Hf; i += blockDim.x) {
    const int cb = i / Hf, j = i - cb * Hf;
    int yf = j + d.oyH;
    if (yf >= Hf) yf -= Hf;
    const int yi = yf - d.y0;  // cropFOV
    if (yi >= 0 && yi < d.Hi) t_out[((size_t)c * d.ns + s0 + cb) * d.Hi + yi] = Z[cb * d.ldH + j] * d.scale;
  }
}

// Phase 3: per image row block and coil group, IFFT along W of the sampled columns, multiply by
// conj(sens_c) and sum the group's coils in coil order (combineImg_kernel, mricartesianoperator.cu:99-126).
__global__ void __launch_bounds__(kThreads) rows_adj_kernel(CartDev d, const float2* __restrict__ t2,
                                                            float2* __restrict__ out, int G, long long gstride) {
  extern __shared__ float2 sm[];
  float2* tw = sm;
  float2* A = tw + d.W;
  float2* B = A + d.RB * d.ldW;
  float2* acc = B + d.RB * d.ldW;
  const int yi0 = blockIdx.x * d.RB;
  const int g = blockIdx.y;
  const int nr = min(d.RB, d.Hi - yi0);
  const int c_begin = (int)((long long)g * d.C / G), c_end = (int)((long long)(g + 1) * d.C / G);
  for (int i = threadIdx.x; i < d.W; i += blockDim.x) tw[i] = d.twW[i];
  for (int i = threadIdx.x; i < nr * d.W; i += blockDim.x) acc[i] = c2(0.f, 0.f);
  for (int c = c_begin; c < c_end; ++c) {
    for (int i = threadIdx.x; i < nr * d.W; i += blockDim.x) {
      const int j = i / nr, r = i - j * nr;
      const int s = d.slot2s[j];
      A[r * d.ldW + j] = (s >= 0) ? t2[((size_t)c * d.ns + s) * d.Hi + yi0 + r] : c2(0.f, 0.f);
    }
    __syncthreads();
    const float2* Z = smem_fft(A, B, nr, d.ldW, d.planW, tw, true);
    for (int i = threadIdx.x; i < nr * d.W; i += blockDim.x) {
      const int r = i / d.W, j = i - r * d.W;
      int x = j + d.oxW;
      if (x >= d.W) x -= d.W;
      float2 v = Z[r * d.ldW + j];
      if (d.sens) v = cmulc(v, d.sens[((size_t)c * d.Hf + yi0 + r + d.y0) * d.W + x]);
      acc[r * d.W + x] += v;
    }
    __syncthreads();
  }
  for (int i = threadIdx.x; i < nr * d.W; i += blockDim.x) {
    const int r = i / d.W, x = i - r * d.W;
    out[(size_t)g * gstride + (size_t)(yi0 + r) * d.W + x] = acc[i];
  }
}

// dense user k-space (W, Hf, C) -> compact [c][s][Hf]
__global__ void gather_kernel(CartDev d, const float2* __restrict__ dense, float2* __restrict__ compact) {
  const size_t n = (size_t)d.C * d.ns * d.Hf;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int P = (int)(i % d.Hf);
    const int ypos = d.kperm ? d.kperm[P] : P;
    const size_t cs = i / d.Hf;
    const int s = (int)(cs % d.ns), c = (int)(cs / d.ns);
    compact[i] = dense[((size_t)c * d.Hf + ypos) * d.W + d.col_x[s]];
  }
}

// compact [c][s][Hf] -> dense user k-space (W, Hf, C); the caller zeroes the unsampled columns first
__global__ void scatter_kernel(CartDev d, const float2* __restrict__ compact, float2* __restrict__ dense) {
  const size_t n = (size_t)d.C * d.ns * d.Hf;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int P = (int)(i % d.Hf);
    const int ypos = d.kperm ? d.kperm[P] : P;
    const size_t cs = i / d.Hf;
    const int s = (int)(cs % d.ns), c = (int)(cs / d.ns);
    dense[((size_t)c * d.Hf + ypos) * d.W + d.col_x[s]] = compact[i];
  }
}

size_t rows_smem(const CartDev& d, bool with_acc) {
  return sizeof(float2) * ((size_t)d.W + 2 * (size_t)d.RB * d.ldW + (with_acc ? (size_t)d.RB * d.W : 0));
}
size_t cols_smem(const CartDev& d) { return sizeof(float2) * ((size_t)d.Hf + 2 * (size_t)d.CB * d.ldH); }

int g_num_sms = 0;
int g_max_smem = 0;
void query_device() {
  if (g_num_sms) return;
  int dev = 0;
  PDT_CUDA_CHECK(cudaGetDevice(&dev));
  PDT_CUDA_CHECK(cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev));
  PDT_CUDA_CHECK(cudaDeviceGetAttribute(&g_max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  PDT_CUDA_CHECK(cudaFuncSetAttribute(rows_fwd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, g_max_smem));
  PDT_CUDA_CHECK(cudaFuncSetAttribute(rows_adj_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, g_max_smem));
  PDT_CUDA_CHECK(cudaFuncSetAttribute(cols_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, g_max_smem));
}

}  // namespace
}  // namespace pdt

#include "pdt_cart_fast.cuh"
#include "pdt_cart_tc.cuh"

namespace pdt {

// ------------------------------------------------------------------------------------------------
// Operator object
// ------------------------------------------------------------------------------------------------
class CartesianOp : public OpImpl, public SolverHooks {
 public:
  CartesianOp(pdt_op_kind kind)
      : OpImpl(kind,
               kind == PDT_OP_CARTESIAN        ? "MriCartesianOperator"
               : kind == PDT_OP_CARTESIAN_ROOS ? "MriCartesianRemoveROOSOperator"
                                               : "MriSamplingOperator",
               kind == PDT_OP_SAMPLING ? 1u : 2u, {}) {}

  // getInputSize / getOutputSize (mricartesianoperator.cu:183-194, 291-303; mrisamplingoperator.cu:40-51)
  Dims input_size(const Dims& out) override {
    if (out.size() < 2) throw Error(PDT_ERR_SIZE, name_ + ": output must have at least 2 dimensions");
    if (kind_ == PDT_OP_CARTESIAN_ROOS) return {out[0], out[1] / 2};
    if (kind_ == PDT_OP_SAMPLING) return out;
    return {out[0], out[1]};
  }
  Dims output_size(const Dims& in) override {
    (void)in;
    if (kind_ == PDT_OP_SAMPLING) return in;
    return constant(0, PDT_C64, 3).size;
  }
  SolverHooks* hooks() override { return this; }
  void check_device_errors() override {
    if (const int e = take_tc_error()) {
      char code[16];
      std::snprintf(code, sizeof code, "0x%x", e);
      throw Error(PDT_ERR_TIMEOUT, name_ + ": a tensor-core row kernel gave up a bounded wait (code " + code +
                                       "); results since the last check are not valid");
    }
  }
  std::string tuning() override {
    prepare();
    check_device_errors();
    std::ostringstream os;
    os << "W=" << dev_.W << " H=" << dev_.Hf << " C=" << dev_.C << " sampled_columns=" << dev_.ns;
    if (tune_.tcf)
      os << " rows_fwd=tensor_dft(tf32x3,k_split=" << tune_.ks << ",stages=" << tc_fwd_stages() << ")";
    else if (frow_.ok())
      os << " rows_fwd=lane_fft(" << frow_.M << "x" << frow_.L << ",warps=" << kWpbChoices[tune_.wf]
         << (frow_cc_.ok() ? ",batched:" + std::to_string(frow_cc_.M) + "x" + std::to_string(frow_cc_.L) +
                                 ",warps=" + std::to_string(kWpbChoices[tune_.wfc])
                           : std::string())
         << ")";
    else
      os << " rows_fwd=stockham";
    if (tune_.tca)
      os << " rows_adj=tensor_dft(tf32x3,n_ranges=" << (2 * dev_.W + tc_adj_nb(tune_.nr) - 1) / tc_adj_nb(tune_.nr)
         << ",row_tiles=" << tc_adj_tiles() << "x" << tc_adj_yb() << "rows,stages=" << tc_adj_stages(tc_adj_nb(tune_.nr))
         << ",coil_sum_on_chip)";
    else if (frow_.ok())
      os << " rows_adj=lane_fft(warps=" << kWpbChoices[tune_.wa] << ",coil_groups=" << G_
         << (tune_.cluster ? ",cluster" : ",partials")
         << (rows_adj_staged(frow_, kWpbChoices[tune_.wa]) ? ",staged" : "") << ")";
    else
      os << " rows_adj=stockham(coil_groups=" << G_ << ")";
    if (fcol_.ok())
      os << " cols=lane_fft(" << fcol_.M << "x" << fcol_.L << ",warps=" << kWpbChoices[tune_.wc]
         << (colz_ ? ",image_rows_only" : "") << ")";
    else
      os << " cols=stockham";
    if (tune_.tca && dev_.ns > 0 && fuse_dual_ && dual_rows() > 0)
      os << " solver_dual=adjoint_launch(" << dual_rows() * ((2 * dev_.W + tc_adj_nb(tune_.nr) - 1) / tc_adj_nb(tune_.nr))
         << "_blocks)";
    if (frow_.ok())  // what a batched solve runs (tca(), tcf(), groups_run())
      os << " in_batch=lane_fft_rows(batch_adj_groups=" << std::min(G_, batch_groups())
         << (tune_.cluster ? ",cluster" : ",partials") << ")";
    return os.str();
  }
  Dims natural_input_size() override {
    if (kind_ == PDT_OP_SAMPLING) return constant(0, PDT_F32, 2).size;
    const Dims& m = constant(1, PDT_F32, 2).size;
    return kind_ == PDT_OP_CARTESIAN_ROOS ? Dims{m[0], m[1] / 2} : m;
  }

  // SolverHooks
  size_t compact_elems() override {
    prepare();
    return (size_t)dev_.C * dev_.ns * dev_.Hf;
  }
  void gather(const float2* dense, float2* compact, cudaStream_t st) override {
    prepare();
    if (dev_.ns == 0) return;
    const size_t n = (size_t)dev_.C * dev_.ns * dev_.Hf;
    const int blocks = (int)std::min<size_t>((n + 255) / 256, 4096);
    gather_kernel<<<blocks, 256, 0, st>>>(dev_, dense, compact);
    PDT_LAUNCH_CHECK();
    count_launch();
  }
  void scatter(const float2* compact, float2* dense, cudaStream_t st) override {
    prepare();
    launch_fill_zero(dense, sizeof(float2) * (size_t)dev_.C * dev_.Hf * dev_.W, st);
    if (dev_.ns == 0) return;
    const size_t n = (size_t)dev_.C * dev_.ns * dev_.Hf;
    const int blocks = (int)std::min<size_t>((n + 255) / 256, 4096);
    scatter_kernel<<<blocks, 256, 0, st>>>(dev_, compact, dense);
    PDT_LAUNCH_CHECK();
    count_launch();
  }
  int groups() override {
    prepare();
    if (tca()) return 1;                         // the tensor-core adjoint rows sum the coils on chip
    return (frow_.ok() && tune_.cluster) ? 1 : groups_run();  // a cluster reduces its coil groups on chip
  }
  long long group_stride() override { return (long long)dev_.Hi * dev_.W; }
  // The dual update rides in the tensor-core adjoint launch when its row tiles leave at least
  // kMinDualBlocks SMs free (one CTA per SM), one row of dual blocks per N range, and no more rows than
  // give each thread a pixel.
  static constexpr int kMinDualBlocks = 8;
  int dual_rows() {
    const int gx = (2 * dev_.W + tc_adj_nb(tune_.nr) - 1) / tc_adj_nb(tune_.nr);
    const int idle = g_num_sms - gx * tc_adj_tiles();
    const long long need = ((long long)dev_.W * dev_.Hi + kTcAdjThreads - 1) / kTcAdjThreads;  // blocks
    return idle >= kMinDualBlocks ? (int)std::min<long long>(idle / gx, (need + gx - 1) / gx) : 0;
  }
  void set_concurrent(bool on) override { concurrent_ = on; }
  bool can_fuse_dual(int W, int H) override {
    prepare();
    return tca() && dev_.ns > 0 && fuse_dual_ && W == dev_.W && H == dev_.Hi && dual_rows() > 0;
  }
  void round(const float2* ubar, float2* r, const float2* fc, float sigma, float lambda, float2* khr, int* tick,
             cudaStream_t st, PhaseMarker* mk, const DualStep* dual) override {
    prepare();
    if (dual && !can_fuse_dual(dual->W, dual->H))
      throw Error(PDT_ERR_STATE, name_ + ": round() given a dual update it cannot run");
    if (dev_.ns == 0) {
      launch_fill_zero(khr, sizeof(float2) * (size_t)groups_run() * dev_.Hi * dev_.W, st);
      if (tick) launch_tick(tick, st);
      return;
    }
    float2* t = scratch_.as<float2>();
    launch_rows_fwd(ubar, t, tick, st);
    if (mk) mk->mark("cart_rows_fwd", st);
    launch_cols(COL_SOLVE, t, t, r, fc, nullptr, nullptr, sigma, lambda, st);
    if (mk) mk->mark("cart_cols_prox", st);
    if (tca())
      launch_tc_rows_adj(t, khr, st, dual);  // the coil sum on chip: one K^H r plane
    else
      launch_rows_adj(t, khr, groups_run(), st);
    if (mk) mk->mark("cart_rows_adj", st);
  }
  void adjoint_compact(const float2* fc, float2* img, cudaStream_t st) override {
    prepare();
    if (dev_.ns == 0) {
      launch_fill_zero(img, sizeof(float2) * (size_t)dev_.Hi * dev_.W, st);
      return;
    }
    float2* t = scratch_.as<float2>();
    launch_cols(COL_ADJ_COMPACT, nullptr, t, nullptr, fc, nullptr, nullptr, 0.f, 0.f, st);
    if (tca())
      launch_tc_rows_adj(t, img, st);
    else
      launch_rows_adj(t, img, 1, st);
  }

 protected:
  // sizeCheck (mricartesianoperator.cu:174-181, 305-314; mrisamplingoperator.cu:32-38)
  void size_check(const Dims& src, const Dims& dst) override {
    if (kind_ == PDT_OP_SAMPLING) {
      const Dims& m = constant(0, PDT_F32, 2).size;
      size_check_eq(dst, m);
      size_check_eq(src, m);
      return;
    }
    const Dims& s = constant(0, PDT_C64, 3).size;
    const Dims& m = constant(1, PDT_F32, 2).size;
    size_check_eq(dst, s);
    if (kind_ == PDT_OP_CARTESIAN_ROOS) {
      if (src.size() != 2) throw Error(PDT_ERR_SIZE, name_ + ": image must be 2-D, got " + dims_str(src));
      size_check_eq(Dims{src[0], src[1] * 2}, m);
    } else {
      size_check_eq(src, m);
      size_check_eq(src, Dims{dst[0], dst[1]});
    }
  }
  void execute_forward(const float2* src, float2* dst, cudaStream_t st) override {
    prepare();
    launch_fill_zero(dst, sizeof(float2) * (size_t)dev_.C * dev_.Hf * dev_.W, st);
    if (dev_.ns == 0) return;
    float2* t = scratch_.as<float2>();
    launch_rows_fwd(src, t, nullptr, st);
    launch_cols(COL_FWD_DENSE, t, nullptr, nullptr, nullptr, nullptr, dst, 0.f, 0.f, st);
  }
  void execute_adjoint(const float2* src, float2* dst, cudaStream_t st) override {
    prepare();
    if (dev_.ns == 0) {
      launch_fill_zero(dst, sizeof(float2) * (size_t)dev_.Hi * dev_.W, st);
      return;
    }
    float2* t = scratch_.as<float2>();
    launch_cols(COL_ADJ_DENSE, nullptr, t, nullptr, nullptr, src, nullptr, 0.f, 0.f, st);
    if (tca())
      launch_tc_rows_adj(t, dst, st);
    else
      launch_rows_adj(t, dst, 1, st);
  }
  void invalidate() override { prepared_ = false; }

 private:
  // Launch configuration of the lane-FFT kernels, chosen by the autotuner in prepare().
  struct Tune {
    int wf = 2, wc = 2, wa = 2;  // warps-per-block index (kWpbChoices) of rows_fwd, cols, rows_adj
    bool cluster = false;        // coil groups of a row block reduced in a cluster (else partial images)
    int tcf = 0, tca = 0;        // 1: tensor-core DFT rows (forward / adjoint) instead of the FFT kernels
    int ks = 4, nr = 4;          // tensor-core forward K split (cluster size), adjoint N ranges
    int wfc = 1;  // warps-per-block index of the concurrent forward-row split (4 warps; 2 and 4 measured alike)
    int sst = 1;  // 1: the FFT adjoint rows stage columns and coil maps by asynchronous copies (where they fit)
  };

  int tc_adj_nb(int nr) const { return std::min(kTcAdjMaxNB, ((2 * dev_.W + nr - 1) / nr + 15) & ~15); }
  int tc_fwd_nb() const { return tc_fwd_rows_max(dev_.ns); }
  int tc_fwd_stages() const {
    return std::min(kTcMaxStages,
                    (int)(((size_t)g_max_smem - tc_fwd_smem(tc_fwd_nb(), 0)) / tc_stage_bytes(tc_fwd_nb())));
  }
  // The forward rows' DFT factor as TF32 hi/lo operand tiles in the layout tc_rows_fwd copies:
  // [s tile][K chunk][hi rows | lo rows] (chunk stride 2 nbmax 128 bytes), row n = 2 sl + o (output s =
  // 128 z + sl, re/im o), K element k = 2 (x - 16 j) + (re/im input), 128-byte swizzle; E'[x][s] =
  // w^(q(x) f_s), values in double precision, then split.
  void build_tc_fwd_tiles() {
    if (tcf_built_) return;
    std::vector<float> h;
    build_tc_fwd_table(dev_.W, dev_.ns, col_x_h_.data(), dev_.mxW, dev_.oxW, h);
    tcf_tiles_.ensure(h.size() * sizeof(float));
    PDT_CUDA_CHECK(cudaMemcpy(tcf_tiles_.p, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice));
    tcf_built_ = true;
  }
  void launch_tc_rows_fwd(const float2* ubar, float2* t1, int* tick, cudaStream_t st) {
    const int ks = tune_.ks, stiles = (dev_.ns + 127) / 128, nst = tc_fwd_stages();
    if (!tcf_built_) throw Error(PDT_ERR_STATE, name_ + ": tensor-core forward tiles not built");
    CartDev dd = dev_;
    dd.tc_yb = tc_adj_yb();
    LaunchEx lx(dim3(tc_adj_tiles(), ks, stiles), dim3(kTcFwdThreads), tc_fwd_smem(tc_fwd_nb(), nst), st,
                ks > 1 ? ks : 0);
    auto fn = dev_.sens ? tc_rows_fwd<true> : tc_rows_fwd<false>;
    PDT_CUDA_CHECK(cudaLaunchKernelEx(&lx.cfg, fn, dd, ubar, (const unsigned char*)tcf_tiles_.p, t1, tick, nst,
                                      tc_err()));
    count_launch();
  }
  int tc_adj_chunks() const { return tc_adj_chunk_count(dev_.ns); }
  // image rows per adjoint row tile: the tile's 128 rows hold them for every coil
  int tc_adj_yb() const { return kTcRows / dev_.C; }
  int tc_adj_tiles() const { return (dev_.Hi + tc_adj_yb() - 1) / tc_adj_yb(); }
  int tc_adj_stages(int NB) const {
    return std::min(kTcMaxStages, (int)(((size_t)g_max_smem - tc_adj_smem(NB, 0)) / tc_stage_bytes(NB)));
  }
  // The adjoint rows' DFT factor for output-column ranges of NB, as TF32 hi/lo operand tiles in the layout
  // tc_rows_adj copies: [range][K chunk][hi rows | lo rows], row n = 2 x + o of the range (o = re/im
  // output), K element k = 2 s + (re/im input), 128-byte swizzle. Values in double precision, then split.
  void build_tc_adj_tiles(int NB) {
    if (tcb_nb_ == NB) return;
    std::vector<float> h;
    build_tc_adj_table(dev_.W, dev_.ns, col_x_h_.data(), dev_.mxW, dev_.oxW, NB, h);
    tcb_.ensure(h.size() * sizeof(float));
    PDT_CUDA_CHECK(cudaMemcpy(tcb_.p, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice));
    tcb_nb_ = NB;
  }
  void launch_tc_rows_adj(const float2* t2, float2* out, cudaStream_t st, const DualStep* dual = nullptr) {
    const int NB = tc_adj_nb(tune_.nr);
    if (tcb_nb_ != NB) throw Error(PDT_ERR_STATE, name_ + ": tensor-core adjoint tiles not built for this range size");
    const int nst = tc_adj_stages(NB);
    CartDev dd = dev_;
    dd.tc_yb = tc_adj_yb();
    const int ntiles = tc_adj_tiles();
    const DualStep ds = dual ? *dual : DualStep{};
    LaunchEx lx(dim3((2 * dev_.W + NB - 1) / NB, ntiles + (dual ? dual_rows() : 0)), dim3(kTcAdjThreads),
                tc_adj_smem(NB, nst), st);
    auto fn = dev_.sens ? tc_rows_adj<true> : tc_rows_adj<false>;
    PDT_CUDA_CHECK(cudaLaunchKernelEx(&lx.cfg, fn, dd, t2, (const unsigned char*)tcb_.p, out, NB, nst, tc_err(),
                                      ntiles, ds));
    count_launch();
  }
  int* tc_err() { return reinterpret_cast<int*>(tc_err_.p); }
  // Reads (and clears) the tensor-core kernels' error word: non-zero when an MMA completion wait ran
  // out of time, in which case that launch's output is not valid.
  int take_tc_error() {
    if (!tc_err_.p) return 0;
    int e = 0;
    PDT_CUDA_CHECK(cudaMemcpy(&e, tc_err_.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (e) PDT_CUDA_CHECK(cudaMemset(tc_err_.p, 0, sizeof(int)));
    return e;
  }

  // The tensor-core row passes take one 198 KB CTA per SM and are chosen by timing the operator alone;
  // among the concurrent problems of a batch the lane-FFT rows, which share SMs, run instead.
  bool tca() const { return tune_.tca && !(concurrent_ && frow_.ok()); }
  // Coil groups of the FFT adjoint rows: the tuned count alone; in a batch at most batch_groups() (2;
  // PDT_BATCH_GROUPS overrides), since each group adds a K^H r partial image that the adjoint writes and
  // the primal step reads, and the other problems supply the parallelism that more groups would (64 mixed
  // problems: 26.9k problem-iterations/s uncapped, 29.1k at 4, 30.6-31.2k at 2, 30.8k at 1)
  static int batch_groups() {
    static const int cap = [] {
      const char* e = std::getenv("PDT_BATCH_GROUPS");
      return (e && *e) ? std::max(1, std::atoi(e)) : 2;
    }();
    return cap;
  }
  int groups_run() const { return concurrent_ ? std::min(G_, batch_groups()) : G_; }
  bool tcf() const { return tune_.tcf && !(concurrent_ && frow_.ok()); }

  void launch_rows_fwd(const float2* ubar, float2* t1, int* tick, cudaStream_t st) {
    if (tcf()) {
      launch_tc_rows_fwd(ubar, t1, tick, st);
      return;
    }
    if (frow_.ok()) {
      const bool cc = concurrent_ && frow_cc_.ok();
      const FastRowKernels& k = cc ? frow_cc_ : frow_;
      const int wf = cc ? tune_.wfc : tune_.wf;
      const int wpb = kWpbChoices[wf];
      const int R = k.rows_per_block(wpb);
      LaunchEx lx(dim3((dev_.Hi + R - 1) / R, dev_.C), dim3(32 * wpb), fast_rows_smem(dev_, k, wpb), st);
      PDT_CUDA_CHECK(cudaLaunchKernelEx(&lx.cfg, k.fwd[wf], dev_, ubar, t1, tick));
      count_launch();
      return;
    }
    dim3 grid((dev_.Hi + dev_.RB - 1) / dev_.RB, dev_.C);
    rows_fwd_kernel<<<grid, kThreads, rows_smem(dev_, false), st>>>(dev_, ubar, t1, tick);
    PDT_LAUNCH_CHECK();
    count_launch();
  }
  void launch_cols(int mode, const float2* tin, float2* tout, float2* r, const float2* fc, const float2* kin,
                   float2* kout, float sigma, float lambda, cudaStream_t st) {
    if (fcol_.ok()) {
      const int wpb = kWpbChoices[tune_.wc];
      const int S = fcol_.cols_per_block(wpb);
      LaunchEx lx(dim3((dev_.ns + S - 1) / S, dev_.C), dim3(32 * wpb), fast_cols_smem(fcol_, wpb), st);
      const FrColsFn fn = colz_ ? fcol_.cols_z[tune_.wc] : fcol_.cols[tune_.wc];
      PDT_CUDA_CHECK(cudaLaunchKernelEx(&lx.cfg, fn, dev_, mode, tin, tout, r, fc, kin, kout, sigma, lambda));
      count_launch();
      return;
    }
    dim3 grid((dev_.ns + dev_.CB - 1) / dev_.CB, dev_.C);
    cols_kernel<<<grid, kThreads, cols_smem(dev_), st>>>(dev_, mode, tin, tout, r, fc, kin, kout, sigma, lambda);
    PDT_LAUNCH_CHECK();
    count_launch();
  }
  // The staged FFT adjoint rows where chosen and where their larger shared-memory footprint fits
  // (PDT_ROWS_ADJ_STAGED=0 / 1 overrides the choice).
  bool rows_adj_staged(const FastRowKernels& k, int wpb) const {
    static const char* env = std::getenv("PDT_ROWS_ADJ_STAGED");
    const bool want = (env && *env) ? std::atoi(env) != 0 : tune_.sst != 0;
    return want && fast_rows_adj_smem(dev_, k, wpb, true) <= (size_t)g_max_smem;
  }
  // K^H: G coil-group partial images (or, with a cluster, one reduced image) into out.
  void launch_rows_adj(const float2* t2, float2* out, int G, cudaStream_t st) {
    if (frow_.ok()) {
      const FastRowKernels& k = (concurrent_ && frow_cc_.ok()) ? frow_cc_ : frow_;
      const int wpb = kWpbChoices[tune_.wa];
      const bool cl = tune_.cluster && G > 1;
      const int R = k.rows_per_block(wpb);
      const bool stg = rows_adj_staged(k, wpb);
      LaunchEx lx(dim3((dev_.Hi + R - 1) / R, G), dim3(32 * wpb), fast_rows_adj_smem(dev_, k, wpb, stg), st,
                  cl ? G : 0);
      PDT_CUDA_CHECK(cudaLaunchKernelEx(&lx.cfg, k.adj[tune_.wa], dev_, t2, out, cl ? 1 : 0, G,
                                        (long long)dev_.Hi * dev_.W, stg ? 1 : 0));
      count_launch();
      return;
    }
    dim3 grid((dev_.Hi + dev_.RB - 1) / dev_.RB, G);
    rows_adj_kernel<<<grid, kThreads, rows_smem(dev_, true), st>>>(dev_, t2, out, G, (long long)dev_.Hi * dev_.W);
    PDT_LAUNCH_CHECK();
    count_launch();
  }

  // Builds the sampled-column tables, twiddles and FFT plans from the current constants.
  void prepare() {
    if (prepared_) return;
    query_device();
    const bool samp = kind_ == PDT_OP_SAMPLING;
    Constant& mk = samp ? constant(0, PDT_F32, 2) : constant(1, PDT_F32, 2);
    const int W = (int)mk.size[0], Hf = (int)mk.size[1];
    int C = 1;
    const float2* sens = nullptr;
    if (!samp) {
      Constant& sc = constant(0, PDT_C64, 3);
      if (sc.size[0] != W || sc.size[1] != Hf)
        throw Error(PDT_ERR_SIZE, name_ + ": coil sensitivities " + dims_str(sc.size) + " do not match mask " +
                                      dims_str(mk.size));
      C = (int)sc.size[2];
      sens = sc.dev.as<float2>();
    }
    CartDev d{};
    d.W = W;
    d.Hf = Hf;
    d.C = C;
    if (kind_ == PDT_OP_CARTESIAN_ROOS) {
      d.Hi = Hf / 2;
      d.y0 = (int)(unsigned int)((float)(unsigned int)(2 * d.Hi) * 0.25f + 1.f);
      if (d.y0 + d.Hi > Hf)
        throw Error(PDT_ERR_SIZE, name_ + ": frequency-encode size " + std::to_string(Hf) + " too small");
    } else {
      d.Hi = Hf;
      d.y0 = 0;
    }
    d.mxW = (int)(((float)W + 1.f) / 2.f);
    d.mxH = (int)(((float)Hf + 1.f) / 2.f);
    d.oxW = W / 2;
    d.oyH = Hf / 2;
    d.scale = (float)(1.0 / std::sqrt((double)W * (double)Hf));
    d.sens = sens;
    if (!make_fft_plan(W, &d.planW) || !make_fft_plan(Hf, &d.planH))
      throw Error(PDT_ERR_UNSUPPORTED, name_ + ": cannot plan FFT sizes " + std::to_string(W) + " x " +
                                           std::to_string(Hf));
    // sampled columns
    const float* mask = reinterpret_cast<const float*>(mk.host.data());
    std::vector<int> col_x;
    {
      std::vector<char> sampled(W, 0);  // row by row: the mask is stored W-fastest
      for (int y = 0; y < Hf; ++y) {
        const float* row = mask + (size_t)y * W;
        for (int x = 0; x < W; ++x) sampled[x] |= row[x] != 0.0f;
      }
      for (int x = 0; x < W; ++x)
        if (sampled[x]) col_x.push_back(x);
    }
    d.ns = (int)col_x.size();
    // lane-FFT kernels where the length has a compiled split (they fix the compact k-space order)
    frow_ = find_row_kernels(W);
    frow_cc_ = frow_.ok() ? find_concurrent_row_kernels(W) : FastRowKernels();  // forward and adjoint rows
    fcol_ = find_col_kernels(Hf);
    if (frow_.ok() && fast_rows_adj_smem(d, frow_, 8) > (size_t)g_max_smem) frow_ = frow_cc_ = FastRowKernels();
    // tensor-core DFT rows: even W (16-byte row vectors), at most 128 coils (a row tile holds one image row
    // of every coil)
    const bool tc_any = W % 2 == 0 && d.ns > 0 && std::getenv("PDT_NO_TENSOR_ROWS") == nullptr;
    tcf_ok_ = tc_any && C <= kTcRows && tc_fwd_smem(256, 2) <= (size_t)g_max_smem;
    tca_ok_ = tc_any && C <= kTcRows && tc_adj_smem(kTcAdjMaxNB, 2) <= (size_t)g_max_smem;
    fuse_dual_ = std::getenv("PDT_NO_FUSED_DUAL") == nullptr;
    if (fcol_.ok() && fast_cols_smem(fcol_, 8) > (size_t)g_max_smem) fcol_ = FastColKernels();
    // register slots of the 64-lane column kernel that hold only rows outside the image for every lane
    // (forward input zero, inverse output unused): the specialised kernel folds them away
    colz_ = false;
    if (fcol_.ok() && fcol_.zmask && fcol_.L == 64) {
      int zm = 0;
      for (int j = 0; j < fcol_.M; ++j) {
        bool outside = true;
        for (int t = 0; t < 64 && outside; ++t) {
          const int yin = ((t + 64 * j - d.mxH) % Hf + Hf) % Hf - d.y0, yout = (t + 64 * j + d.oyH) % Hf - d.y0;
          outside = (yin < 0 || yin >= d.Hi) && (yout < 0 || yout >= d.Hi);
        }
        if (outside) zm |= 1 << j;
      }
      colz_ = (zm & fcol_.zmask) == fcol_.zmask;  // every slot the specialisation skips is outside
    }
    // compact position P -> output row: P = k1 L + t holds spectrum index k1 + M brev_L(t), which the
    // fftshift puts on row (k + Hf/2) mod Hf
    std::vector<int> kperm(Hf);
    for (int P = 0; P < Hf; ++P) {
      if (fcol_.ok()) {
        const int k = P / fcol_.L + fcol_.M * host_lane_brev(P % fcol_.L, fcol_.L);
        kperm[P] = (k + d.oyH) % Hf;
      } else {
        kperm[P] = P;
      }
    }
    std::vector<int> fwd_slot(d.ns), slot2s(W, -1), fslot2s(W, -1);
    std::vector<float> maskc((size_t)d.ns * Hf);
    for (int s = 0; s < d.ns; ++s) {
      const int x = col_x[s];
      fwd_slot[s] = ((x - d.oxW) % W + W) % W;
      fslot2s[fwd_slot[s]] = s;
      slot2s[(x + d.mxW) % W] = s;
      for (int P = 0; P < Hf; ++P) maskc[(size_t)s * Hf + P] = mask[(size_t)kperm[P] * W + x];
    }
    // launch shapes
    d.ldW = W + 1;
    d.ldH = Hf + 1;
    d.RB = 4;
    d.CB = 4;
    while (d.RB > 1 && rows_smem(d, true) > (size_t)g_max_smem) d.RB /= 2;
    while (d.CB > 1 && cols_smem(d) > (size_t)g_max_smem) d.CB /= 2;
    if (rows_smem(d, true) > (size_t)g_max_smem || cols_smem(d) > (size_t)g_max_smem)
      throw Error(PDT_ERR_UNSUPPORTED, name_ + ": FFT size too large for shared memory");
    // device tables (one allocation, 16-byte aligned sub-arrays)
    std::vector<float2> twW(W), twH(Hf);
    fill_twiddles(W, twW.data());
    fill_twiddles(Hf, twH.data());
    const size_t need = 16 * 9 + sizeof(int) * (2 * (size_t)d.ns + 2 * (size_t)W + Hf) +
                        sizeof(float) * maskc.size() + sizeof(float2) * ((size_t)W + Hf);
    tables_.ensure(need);
    char* base = tables_.as<char>();
    std::vector<char> staged(need);  // assembled on the host, uploaded in one copy below
    size_t off = 0;
    auto put = [&](const void* src, size_t bytes) {
      off = (off + 15) & ~(size_t)15;
      if (off + bytes > need) throw Error(PDT_ERR_STATE, name_ + ": operator tables overflow their allocation");
      if (bytes) std::memcpy(staged.data() + off, src, bytes);
      char* dst = base + off;
      off += bytes;
      return dst;
    };
    d.twW = reinterpret_cast<const float2*>(put(twW.data(), sizeof(float2) * W));
    d.twH = reinterpret_cast<const float2*>(put(twH.data(), sizeof(float2) * Hf));
    d.fwd_slot = reinterpret_cast<const int*>(put(fwd_slot.data(), sizeof(int) * d.ns));
    d.col_x = reinterpret_cast<const int*>(put(col_x.data(), sizeof(int) * d.ns));
    d.slot2s = reinterpret_cast<const int*>(put(slot2s.data(), sizeof(int) * W));
    d.fslot2s = reinterpret_cast<const int*>(put(fslot2s.data(), sizeof(int) * W));
    d.maskc = reinterpret_cast<const float*>(put(maskc.data(), sizeof(float) * maskc.size()));
    d.kperm = fcol_.ok() ? reinterpret_cast<const int*>(put(kperm.data(), sizeof(int) * Hf)) : nullptr;
    PDT_CUDA_CHECK(cudaMemcpy(base, staged.data(), off, cudaMemcpyHostToDevice));
    scratch_.ensure(std::max<size_t>(1, (size_t)C * d.ns * d.Hi) * sizeof(float2));
    for (int w = 0; w < 3; ++w) {
      if (frow_.ok()) {
        PDT_CUDA_CHECK(cudaFuncSetAttribute(frow_.fwd[w], cudaFuncAttributeMaxDynamicSharedMemorySize, g_max_smem));
        PDT_CUDA_CHECK(cudaFuncSetAttribute(frow_.adj[w], cudaFuncAttributeMaxDynamicSharedMemorySize, g_max_smem));
      }
      if (frow_cc_.ok()) {
        PDT_CUDA_CHECK(cudaFuncSetAttribute(frow_cc_.fwd[w], cudaFuncAttributeMaxDynamicSharedMemorySize, g_max_smem));
        PDT_CUDA_CHECK(cudaFuncSetAttribute(frow_cc_.adj[w], cudaFuncAttributeMaxDynamicSharedMemorySize, g_max_smem));
      }
      if (fcol_.ok())
        PDT_CUDA_CHECK(cudaFuncSetAttribute(fcol_.cols[w], cudaFuncAttributeMaxDynamicSharedMemorySize, g_max_smem));
      if (fcol_.ok() && fcol_.cols_z[w])
        PDT_CUDA_CHECK(cudaFuncSetAttribute(fcol_.cols_z[w], cudaFuncAttributeMaxDynamicSharedMemorySize, g_max_smem));
    }
    col_x_h_ = col_x;
    tcb_nb_ = 0;
    tcf_built_ = false;
    if (tcf_ok_ || tca_ok_) {
      for (auto fn : {tc_rows_fwd<true>, tc_rows_fwd<false>})
        PDT_CUDA_CHECK(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, g_max_smem));
      for (auto fn : {tc_rows_adj<true>, tc_rows_adj<false>})
        PDT_CUDA_CHECK(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, g_max_smem));
      tc_err_.ensure(sizeof(int));
      PDT_CUDA_CHECK(cudaMemset(tc_err_.p, 0, sizeof(int)));
    }
    tune_ = Tune();
    const int row_blocks = (d.Hi + d.RB - 1) / d.RB;
    G_ = std::max(1, std::min(C, (2 * g_num_sms + row_blocks - 1) / row_blocks));
    dev_ = d;
    autotune();
    dev_ = d;
    prepared_ = true;
  }

  // Times the candidate launch shapes of the lane-FFT kernels on scratch buffers (CUDA events, a
  // few launches each) and keeps the fastest: warps per block of each kernel, and for the adjoint rows
  // the number of coil groups and cluster reduction versus partial images. Results are cached per
  // (W, H, coils, sampled columns).
  void autotune() {
    if (!frow_.ok() && !fcol_.ok() && !tcf_ok_ && !tca_ok_) return;
    if (pinned_tune()) return;
    // candidates are timed with the kernels of a problem alone (an operator first prepared inside a
    // batched solve would otherwise time the concurrent row split for every forward and adjoint choice)
    struct Alone {
      bool& flag;
      const bool saved;
      explicit Alone(bool& f) : flag(f), saved(f) { flag = false; }
      ~Alone() { flag = saved; }
    } alone(concurrent_);
    static std::mutex g_tune_mu;
    static std::map<std::array<int, 6>, std::pair<Tune, int>> g_tune_cache;
    const std::array<int, 6> key = {dev_.W, dev_.Hf, dev_.Hi, dev_.C, dev_.ns, dev_.sens ? 1 : 0};
    {
      std::lock_guard<std::mutex> lock(g_tune_mu);
      auto it = g_tune_cache.find(key);
      if (it != g_tune_cache.end()) {
        tune_ = it->second.first;
        G_ = it->second.second;
        if (tune_.tca) build_tc_adj_tiles(tc_adj_nb(tune_.nr));
        if (tune_.tcf) build_tc_fwd_tiles();
        return;
      }
    }
    if (dev_.ns == 0) return;
    const size_t nimg = (size_t)dev_.Hi * dev_.W, nk = (size_t)dev_.C * dev_.ns * dev_.Hf;
    DevBuf ub, rr, ff, kh;
    ub.ensure(nimg * sizeof(float2));
    rr.ensure(nk * sizeof(float2));
    ff.ensure(nk * sizeof(float2));
    kh.ensure((size_t)dev_.C * nimg * sizeof(float2));
    PDT_CUDA_CHECK(cudaMemset(ub.p, 0, ub.bytes));
    PDT_CUDA_CHECK(cudaMemset(rr.p, 0, rr.bytes));
    PDT_CUDA_CHECK(cudaMemset(ff.p, 0, ff.bytes));
    float2* t = scratch_.as<float2>();
    cudaStream_t st = 0;
    cudaEvent_t e0, e1;
    PDT_CUDA_CHECK(cudaEventCreate(&e0));
    PDT_CUDA_CHECK(cudaEventCreate(&e1));
    // a candidate whose launch is rejected (e.g. a cluster shape the device cannot schedule) is skipped
    // the best of three batches of ten launches (after one warm-up launch)
    auto time = [&](const std::function<void()>& fn) {
      try {
        fn();
        float best = 1e30f;
        for (int rep = 0; rep < 3; ++rep) {
          PDT_CUDA_CHECK(cudaEventRecord(e0, st));
          for (int i = 0; i < 10; ++i) fn();
          PDT_CUDA_CHECK(cudaEventRecord(e1, st));
          PDT_CUDA_CHECK(cudaEventSynchronize(e1));
          float ms = 0;
          PDT_CUDA_CHECK(cudaEventElapsedTime(&ms, e0, e1));
          best = std::min(best, ms);
        }
        return best;
      } catch (const Error&) {
        cudaGetLastError();
        PDT_CUDA_CHECK(cudaDeviceSynchronize());  // a sticky error surfaces here and fails the operator
        return 1e30f;
      }
    };
    const uint64_t launches0 = g_launches.load();
    Tune best = tune_;
    float bt = 1e30f, ba = 1e30f;  // best forward / adjoint row times so far
    if (frow_.ok()) {
      for (int w = 0; w < 3; ++w) {
        tune_.wf = w;
        const float ms = time([&] { launch_rows_fwd(ub.as<float2>(), t, nullptr, st); });
        if (ms < bt) bt = ms, best.wf = w;
      }
      tune_.wf = best.wf;
      int bestG = G_;
      const int gmax = std::min(dev_.C, 16);
      for (int w = 0; w < 3; ++w)
        for (int cl = 0; cl < 2; ++cl)
          for (int g : {1, 2, 3, 4, 5, 6, 8, 10, 12, 16}) {
            if (g > gmax || (cl && (g < 2 || g > 8))) continue;
            tune_.wa = w;
            tune_.cluster = cl != 0;
            const float ms = time([&] { launch_rows_adj(t, kh.as<float2>(), g, st); });
            if (ms < ba) ba = ms, best.wa = w, best.cluster = cl != 0, bestG = g;
          }
      G_ = bestG;
      // the chosen shape with register-prefetched columns and global coil-map loads instead of staging
      tune_.wa = best.wa;
      tune_.cluster = best.cluster;
      tune_.sst = 0;
      if (const float ms = time([&] { launch_rows_adj(t, kh.as<float2>(), G_, st); }); ms < ba) ba = ms, best.sst = 0;
      tune_.sst = best.sst;
    } else if (tcf_ok_) {
      bt = time([&] { launch_rows_fwd(ub.as<float2>(), t, nullptr, st); });
    }
    if (tcf_ok_) {  // tensor-core forward rows: K splits (cluster sizes)
      build_tc_fwd_tiles();
      const int nchT = (2 * dev_.W + 31) / 32;
      for (int ks : {2, 3, 4}) {
        if (ks > nchT) continue;
        tune_.tcf = 1;
        tune_.ks = ks;
        const float ms = time([&] { launch_rows_fwd(ub.as<float2>(), t, nullptr, st); });
        if (ms < bt) bt = ms, best.tcf = 1, best.ks = ks;
      }
      tune_.tcf = 0;
    }
    if (fcol_.ok()) {
      float bc = 1e30f;
      for (int w = 0; w < 3; ++w) {
        tune_.wc = w;
        const float ms = time([&] {
          launch_cols(COL_SOLVE, t, t, rr.as<float2>(), ff.as<float2>(), nullptr, nullptr, 0.125f, 1.f, st);
        });
        if (ms < bc) bc = ms, best.wc = w;
      }
      tune_.wc = best.wc;
    }
    if (tca_ok_) {
      // the adjoint rows: FFT rows (tuned above, with their coil-group partial images) against the
      // tensor-core rows (coil sum on chip), for a few output-column range counts
      tune_.wa = best.wa;
      tune_.cluster = best.cluster;
      float pair = time([&] { launch_rows_adj(t, kh.as<float2>(), G_, st); });
      for (int nr : {2, 3, 4, 5, 6, 8}) {
        tune_.nr = nr;
        build_tc_adj_tiles(tc_adj_nb(nr));
        const float ms = time([&] { launch_tc_rows_adj(t, kh.as<float2>(), st); });
        if (ms < pair) pair = ms, best.tca = 1, best.nr = nr;
      }
    }
    if (const int e = take_tc_error()) {
      std::fprintf(stderr, "pdt: tensor-core row kernels reported error %d while tuning; using the FFT rows\n", e);
      best.tcf = best.tca = 0;
    }
    g_launches.fetch_sub(g_launches.load() - launches0);  // tuning launches are not solver work
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    tune_ = best;
    if (tune_.tca) build_tc_adj_tiles(tc_adj_nb(tune_.nr));
    if (tune_.tcf) build_tc_fwd_tiles();
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune_cache[key] = {tune_, G_};
  }

  // PDT_CARTESIAN_TUNE="wf,wc,wa,groups,cluster[,tcf,tca[,ks,nr]]" (warps per block of rows_fwd, cols,
  // rows_adj; coil groups; 1 = cluster reduction; 1 = tensor-core DFT forward / adjoint rows; their K
  // split and output-column ranges) replaces the autotuner, e.g. to profile one fixed configuration.
  bool pinned_tune() {
    const char* env = std::getenv("PDT_CARTESIAN_TUNE");
    if (!env || !*env) return false;
    int v[9];
    const int n = std::sscanf(env, "%d,%d,%d,%d,%d,%d,%d,%d,%d", &v[0], &v[1], &v[2], &v[3], &v[4], &v[5], &v[6],
                              &v[7], &v[8]);
    if (n != 5 && n != 7 && n != 9)
      throw Error(PDT_ERR_INVALID_ARGUMENT, "PDT_CARTESIAN_TUNE: expected wf,wc,wa,groups,cluster[,tcf,tca[,ks,nr]]");
    auto idx = [&](int w) {
      for (int i = 0; i < 3; ++i)
        if (kWpbChoices[i] == w) return i;
      throw Error(PDT_ERR_INVALID_ARGUMENT, "PDT_CARTESIAN_TUNE: warps per block must be 2, 4 or 8");
    };
    tune_.wf = idx(v[0]);
    tune_.wc = idx(v[1]);
    tune_.wa = idx(v[2]);
    tune_.cluster = v[4] != 0;
    if (v[3] < 1 || v[3] > std::min(dev_.C, 16) || (tune_.cluster && (v[3] < 2 || v[3] > 8)))
      throw Error(PDT_ERR_INVALID_ARGUMENT, "PDT_CARTESIAN_TUNE: coil groups out of range for this operator");
    G_ = v[3];
    if (n >= 7) {  // where the tensor-core rows are not available (odd W, ...) the FFT rows run
      tune_.tcf = v[5] != 0 && tcf_ok_;
      tune_.tca = v[6] != 0 && tca_ok_;
    }
    if (n == 9) {
      if (v[7] < 1 || v[7] > 8 || v[8] < 1 || v[8] > 64)
        throw Error(PDT_ERR_INVALID_ARGUMENT, "PDT_CARTESIAN_TUNE: K split must be 1..8 and ranges 1..64");
      tune_.ks = std::min(v[7], (2 * dev_.W + 31) / 32);
      tune_.nr = v[8];
    }
    if (tune_.tca) build_tc_adj_tiles(tc_adj_nb(tune_.nr));
    if (tune_.tcf) build_tc_fwd_tiles();
    return true;
  }

  bool prepared_ = false;
  Tune tune_;
  CartDev dev_{};
  FastRowKernels frow_;
  FastColKernels fcol_;
  bool tcf_ok_ = false, tca_ok_ = false;
  FastRowKernels frow_cc_;  // forward-row split for concurrent rounds (set_concurrent)
  bool concurrent_ = false;
  bool fuse_dual_ = true;  // PDT_NO_FUSED_DUAL: the solvers' dual update always in its own kernel
  bool colz_ = false;  // the column kernel's zero-slot specialisation applies
  std::vector<int> col_x_h_;
  int tcb_nb_ = 0;         // range size the adjoint DFT tiles in tcb_ were built for
  bool tcf_built_ = false;  // forward DFT tiles in tcf_tiles_
  int G_ = 1;
  DevBuf tables_, scratch_, tc_err_, tcb_, tcf_tiles_;
};

std::shared_ptr<OpImpl> make_cartesian_operator(pdt_op_kind kind) { return std::make_shared<CartesianOp>(kind); }

void cartesian_set_drop_arrival(int on) { PDT_CUDA_CHECK(tc::set_drop_arrival(on)); }

}  // namespace pdt
