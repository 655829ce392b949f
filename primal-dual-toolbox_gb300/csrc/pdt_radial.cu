// pdt_radial.cu -- radial (non-Cartesian) MRI operators: MriRadialOperator and
// MriRadialSinglecoilOperator (mriradialoperator.cu:27-321).
//
// The reference hands these to gpuNUFFT (absent here). This engine implements the same method --
// Kaiser-Bessel gridding on an osf-oversampled grid with deapodisation and density-compensation weights
// -- with its own kernels:
//   A u [c, j] = w_j / N * sum_{x,y} sens_c(x,y) u(x,y) exp(-2 pi i (k0_j (x - N/2) + k1_j (y - N/2)))
// approximated on the G x G grid (G = ceil(osf N), even), kernel width W = kernel_width grid cells,
// beta = pi sqrt((W/osf)^2 (osf - 1/2)^2 - 0.8) (Beatty et al. 2005), deapodisation = the kernel's
// continuous Fourier transform. Trajectory {Ns, 2} is planar (k0 for all samples, then k1; k0 pairs with
// image x); dcf {Ns, 1}; coil maps {N, N, C}.
//
// Kernels (all FFTs are the batched shared-memory FFT of pdt_device.cuh over the G-point axes):
//   rad_rows_fwd   image rows . sens_c / deap  -> zero-padded FFT along x   -> T[c][gx][image row]
//   rad_cols       FFT along y of each grid column (input on the N image rows) -> F[c][gx][gy]
//   rad_degrid     per sample: 9 (W^2) taps of F, dcf weight; solver mode adds the k-space dual prox
//   rad_grid       gridding as a gather: one thread per grid cell walks the samples whose footprint covers
//                  the cell, in sample order, with their tap weights (lists built at set-up) --
//                  deterministic, no atomics
//   rad_cols_inv   IFFT along y of each grid column, keep the N image rows
//   rad_rows_inv   IFFT along x, crop, / deap, conj(sens_c) . and the coil sum
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <sstream>

#include "pdt_device.cuh"
#include "pdt_fftplan.h"
#include "pdt_ops.h"

namespace pdt {
namespace {

constexpr int kRT = 256;   // threads per block
constexpr int kMaxKw = 8;  // largest supported kernel width
constexpr int kRR = 4;     // rows per block in the row passes
constexpr int kRC = 4;     // columns per block in the column passes
constexpr int kHeavy = 12; // gridding: cells with longer sample lists get a warp each

struct RadDev {
  int N, G, C, Ns, kw;
  int off;          // N/2: image x maps to grid (x - N/2) mod G
  float scale;      // 1/N
  int ldG;          // G + 1
  const float2* sens;   // (N, N, C) or null
  const float* deap;    // [N] deapodisation (already 1/(deap) * ... no: raw values)
  const float* w;       // [Ns] density compensation
  const int* g0;        // [2*Ns] gx0, gy0 (may be negative; wrap mod G)
  const float* wt;      // [Ns][2][kw] tap weights (x then y)
  const int* cell_ptr;  // [G*G+1] per grid cell gx * G + gy: range of its entries
  const int* cell_idx;  // samples whose footprint covers the cell, ascending
  const float* cell_w;  // their tap weights wx * wy
  const int* heavy;     // cells with more than kHeavy entries (gridded one warp per cell)
  int n_heavy;
  const float2* tw;     // [G]
  FftPlan plan;
};

__device__ __forceinline__ int wrapG(int g, int G) {
  g %= G;
  return g < 0 ? g + G : g;
}

// image rows -> FFT along x on the zero-padded grid row; writes every grid column for these rows.
__global__ void __launch_bounds__(kRT) rad_rows_fwd(RadDev d, const float2* __restrict__ u, float2* __restrict__ T) {
  extern __shared__ float2 sm[];
  float2* tw = sm;
  float2* A = tw + d.G;
  float2* B = A + kRR * d.ldG;
  const int y0 = blockIdx.x * kRR, c = blockIdx.y;
  const int nr = min(kRR, d.N - y0);
  for (int i = threadIdx.x; i < d.G; i += blockDim.x) tw[i] = d.tw[i];
  for (int i = threadIdx.x; i < nr * d.G; i += blockDim.x) A[(i / d.G) * d.ldG + i % d.G] = c2(0.f, 0.f);
  __syncthreads();
  for (int i = threadIdx.x; i < nr * d.N; i += blockDim.x) {
    const int r = i / d.N, x = i - r * d.N, y = y0 + r;
    float2 v = u[(size_t)y * d.N + x];
    if (d.sens) v = cmul(v, d.sens[((size_t)c * d.N + y) * d.N + x]);
    v = v * (d.scale / (d.deap[x] * d.deap[y]));
    A[r * d.ldG + wrapG(x - d.off, d.G)] = v;
  }
  __syncthreads();
  const float2* X = smem_fft(A, B, nr, d.ldG, d.plan, tw, false);
  for (int i = threadIdx.x; i < d.G * nr; i += blockDim.x) {
    const int gx = i / nr, r = i - gx * nr;
    T[((size_t)c * d.G + gx) * d.N + y0 + r] = X[r * d.ldG + gx];
  }
}

// FFT along y of each grid column; input lives on the N image rows (grid rows (y - N/2) mod G).
__global__ void __launch_bounds__(kRT) rad_cols(RadDev d, const float2* __restrict__ T, float2* __restrict__ F) {
  extern __shared__ float2 sm[];
  float2* tw = sm;
  float2* A = tw + d.G;
  float2* B = A + kRC * d.ldG;
  const int gx0 = blockIdx.x * kRC, c = blockIdx.y;
  const int ncb = min(kRC, d.G - gx0);
  for (int i = threadIdx.x; i < d.G; i += blockDim.x) tw[i] = d.tw[i];
  for (int i = threadIdx.x; i < ncb * d.G; i += blockDim.x) A[(i / d.G) * d.ldG + i % d.G] = c2(0.f, 0.f);
  __syncthreads();
  for (int i = threadIdx.x; i < ncb * d.N; i += blockDim.x) {
    const int cb = i / d.N, y = i - cb * d.N;
    A[cb * d.ldG + wrapG(y - d.off, d.G)] = T[((size_t)c * d.G + gx0 + cb) * d.N + y];
  }
  __syncthreads();
  const float2* X = smem_fft(A, B, ncb, d.ldG, d.plan, tw, false);
  for (int i = threadIdx.x; i < ncb * d.G; i += blockDim.x) {
    const int cb = i / d.G, gy = i - cb * d.G;
    F[((size_t)c * d.G + gx0 + cb) * d.G + gy] = X[cb * d.ldG + gy];
  }
}

// Degridding. mode 0: kout[c][j] = A u. mode 1 (solver): r <- (r + sigma (A u - f)) / (1 + sigma lambda),
// s[j][c] = w_j r (the weighted values the adjoint grids, sample-major). blockIdx.y selects a chunk of MAXC
// coils, fully unrolled, so that a sample's tap loads of the chunk are all in flight at once; KW > 0 fixes
// the kernel width at compile time so that the taps unroll too (KW = 0: d.kw at run time).
template <int MAXC, int KW>
__global__ void __launch_bounds__(kRT) rad_degrid(RadDev d, int mode, const float2* __restrict__ F,
                                                  float2* __restrict__ kout, float2* __restrict__ r,
                                                  const float2* __restrict__ f, float2* __restrict__ s,
                                                  float sigma, float lambda) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= d.Ns) return;
  static_assert(KW >= 0 && KW <= kMaxKw, "kernel width");
  const int kw = KW > 0 ? KW : d.kw;
  float wx[kMaxKw], wy[kMaxKw];
  int gxs[kMaxKw], gys[kMaxKw];
#pragma unroll
  for (int t = 0; t < kw; ++t) {
    wx[t] = d.wt[((size_t)j * 2 + 0) * kw + t];
    wy[t] = d.wt[((size_t)j * 2 + 1) * kw + t];
    gxs[t] = wrapG(d.g0[2 * j] + t, d.G);
    gys[t] = wrapG(d.g0[2 * j + 1] + t, d.G);
  }
  const float wj = d.w[j];
  const size_t plane = (size_t)d.G * d.G;
  {
    const int cbase = blockIdx.y * MAXC;
    const int nc = min(MAXC, d.C - cbase);
    float2 a[MAXC];
#pragma unroll
    for (int c = 0; c < MAXC; ++c) a[c] = c2(0.f, 0.f);
#pragma unroll
    for (int tx = 0; tx < kw; ++tx) {
      float2 col[MAXC];
#pragma unroll
      for (int c = 0; c < MAXC; ++c) col[c] = c2(0.f, 0.f);
#pragma unroll
      for (int ty = 0; ty < kw; ++ty) {
        const float2* Fp = F + (size_t)cbase * plane + (size_t)gxs[tx] * d.G + gys[ty];
#pragma unroll
        for (int c = 0; c < MAXC; ++c)
          if (c < nc) col[c] += Fp[(size_t)c * plane] * wy[ty];
      }
#pragma unroll
      for (int c = 0; c < MAXC; ++c) a[c] += col[c] * wx[tx];
    }
#pragma unroll
    for (int c = 0; c < MAXC; ++c) {
      if (c >= nc) break;
      const float2 av = a[c] * wj;
      const size_t o = (size_t)(cbase + c) * d.Ns + j;
      if (mode == 0) {
        kout[o] = av;
      } else {
        const float2 rn = (r[o] + sigma * (av - f[o])) / (1.0f + sigma * lambda);
        r[o] = rn;
        s[(size_t)j * d.C + cbase + c] = rn * wj;  // sample-major for the gridding gather
      }
    }
  }
}

// s[j][c] = w_j k[c][j] (adjoint input weighting for a dense k-space, sample-major).
__global__ void rad_weight(RadDev d, const float2* __restrict__ k, float2* __restrict__ s) {
  const size_t n = (size_t)d.C * d.Ns;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const size_t c = i / d.Ns, j = i - c * d.Ns;
    s[j * d.C + c] = k[i] * d.w[j];
  }
}

// Gridding as a gather: H[c][gx][gy] = sum_j s[j][c] wx[gx - gx0_j] wy[gy - gy0_j] over the samples j whose
// footprint covers the cell (lists built at set-up, entries in sample order). One launch, two kinds of
// block: the first heavy_blocks blocks give each of the cells near k = 0 (more than kHeavy entries) a
// warp, lane l taking entries l, l + 32, ... and an xor-butterfly sum (every lane ends with the same,
// run-to-run identical value); the others give every remaining cell a thread that walks its list in
// order, four entries at a time so that many loads are in flight. A sample's coil values are contiguous.
template <int MAXC>
__global__ void __launch_bounds__(kRT) rad_grid(RadDev d, const float2* __restrict__ s, float2* __restrict__ H,
                                                int heavy_blocks) {
  const size_t ncell = (size_t)d.G * d.G;
  if ((int)blockIdx.x < heavy_blocks) {
    const int wi = blockIdx.x * (kRT / 32) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (wi >= d.n_heavy) return;  // uniform per warp
    const int cell = d.heavy[wi];
    const int beg = d.cell_ptr[cell], end = d.cell_ptr[cell + 1];
    for (int cbase = 0; cbase < d.C; cbase += MAXC) {
      const int nc = min(MAXC, d.C - cbase);
      float2 acc[MAXC];
#pragma unroll
      for (int c = 0; c < MAXC; ++c) acc[c] = c2(0.f, 0.f);
      for (int e = beg + lane; e < end; e += 32) {
        const float2* sj = s + (size_t)d.cell_idx[e] * d.C + cbase;
        const float wgt = d.cell_w[e];
#pragma unroll
        for (int c = 0; c < MAXC; ++c)
          if (c < nc) acc[c] += sj[c] * wgt;
      }
#pragma unroll
      for (int c = 0; c < MAXC; ++c) {
        if (c < nc) {
          for (int o = 16; o > 0; o >>= 1) {
            acc[c].x += __shfl_xor_sync(0xffffffffu, acc[c].x, o);
            acc[c].y += __shfl_xor_sync(0xffffffffu, acc[c].y, o);
          }
          if (lane == 0) H[(size_t)(cbase + c) * ncell + cell] = acc[c];
        }
      }
    }
    return;
  }
  const size_t cell = (blockIdx.x - heavy_blocks) * (size_t)blockDim.x + threadIdx.x;
  if (cell >= ncell) return;
  const int beg = d.cell_ptr[cell], end = d.cell_ptr[cell + 1];
  if (end - beg > kHeavy) return;  // a heavy block's warp grids it
  for (int cbase = 0; cbase < d.C; cbase += MAXC) {
    const int nc = min(MAXC, d.C - cbase);
    float2 acc[MAXC];
#pragma unroll
    for (int c = 0; c < MAXC; ++c) acc[c] = c2(0.f, 0.f);
    // four entries at a time, the last group predicated (most cells have fewer than four), so that a
    // group's index and weight loads, then its sample loads, are each in flight together
    for (int e = beg; e < end; e += 4) {
      const int m = end - e;  // entries e .. e + min(m, 4) - 1 are this cell's
      const float2* sp[4];
      float w[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        sp[k] = s + (size_t)(k < m ? d.cell_idx[e + k] : 0) * d.C + cbase;
        w[k] = k < m ? d.cell_w[e + k] : 0.f;
      }
#pragma unroll
      for (int c = 0; c < MAXC; ++c)
        if (c < nc) {  // loads only for this cell's entries, added in entry order as one at a time
          const float2 z = c2(0.f, 0.f);
          const float2 a0 = sp[0][c], a1 = m > 1 ? sp[1][c] : z, a2 = m > 2 ? sp[2][c] : z,
                       a3 = m > 3 ? sp[3][c] : z;
          acc[c] += a0 * w[0];
          if (m > 1) acc[c] += a1 * w[1];
          if (m > 2) acc[c] += a2 * w[2];
          if (m > 3) acc[c] += a3 * w[3];
        }
    }
#pragma unroll
    for (int c = 0; c < MAXC; ++c)
      if (c < nc) H[(size_t)(cbase + c) * ncell + cell] = acc[c];
  }
}

// IFFT along y of each grid column; keep the N image rows -> T[c][gx][y].
__global__ void __launch_bounds__(kRT) rad_cols_inv(RadDev d, const float2* __restrict__ H, float2* __restrict__ T) {
  extern __shared__ float2 sm[];
  float2* tw = sm;
  float2* A = tw + d.G;
  float2* B = A + kRC * d.ldG;
  const int gx0 = blockIdx.x * kRC, c = blockIdx.y;
  const int ncb = min(kRC, d.G - gx0);
  for (int i = threadIdx.x; i < d.G; i += blockDim.x) tw[i] = d.tw[i];
  for (int i = threadIdx.x; i < ncb * d.G; i += blockDim.x) {
    const int cb = i / d.G, gy = i - cb * d.G;
    A[cb * d.ldG + gy] = H[((size_t)c * d.G + gx0 + cb) * d.G + gy];
  }
  __syncthreads();
  const float2* X = smem_fft(A, B, ncb, d.ldG, d.plan, tw, true);
  for (int i = threadIdx.x; i < ncb * d.N; i += blockDim.x) {
    const int cb = i / d.N, y = i - cb * d.N;
    T[((size_t)c * d.G + gx0 + cb) * d.N + y] = X[cb * d.ldG + wrapG(y - d.off, d.G)];
  }
}

// IFFT along x, crop to the image, deapodise, conj(sens_c) and sum the coils of group g.
__global__ void __launch_bounds__(kRT) rad_rows_inv(RadDev d, const float2* __restrict__ T, float2* __restrict__ out,
                                                    int G, long long gstride) {
  extern __shared__ float2 sm[];
  float2* tw = sm;
  float2* A = tw + d.G;
  float2* B = A + kRR * d.ldG;
  float2* acc = B + kRR * d.ldG;
  const int y0 = blockIdx.x * kRR, g = blockIdx.y;
  const int nr = min(kRR, d.N - y0);
  const int c_begin = (int)((long long)g * d.C / G), c_end = (int)((long long)(g + 1) * d.C / G);
  for (int i = threadIdx.x; i < d.G; i += blockDim.x) tw[i] = d.tw[i];
  for (int i = threadIdx.x; i < nr * d.N; i += blockDim.x) acc[i] = c2(0.f, 0.f);
  for (int c = c_begin; c < c_end; ++c) {
    __syncthreads();
    for (int i = threadIdx.x; i < nr * d.G; i += blockDim.x) {
      const int gx = i / nr, r = i - gx * nr;
      A[r * d.ldG + gx] = T[((size_t)c * d.G + gx) * d.N + y0 + r];
    }
    __syncthreads();
    const float2* Z = smem_fft(A, B, nr, d.ldG, d.plan, tw, true);
    for (int i = threadIdx.x; i < nr * d.N; i += blockDim.x) {
      const int r = i / d.N, x = i - r * d.N, y = y0 + r;
      float2 v = Z[r * d.ldG + wrapG(x - d.off, d.G)] * (d.scale / (d.deap[x] * d.deap[y]));
      if (d.sens) v = cmulc(v, d.sens[((size_t)c * d.N + y) * d.N + x]);
      acc[i] += v;
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nr * d.N; i += blockDim.x) {
    const int r = i / d.N, x = i - r * d.N;
    out[(size_t)g * gstride + (size_t)(y0 + r) * d.N + x] = acc[i];
  }
}

int g_rad_sms = 0, g_rad_smem = 0;

}  // namespace
}  // namespace pdt

#include "pdt_rad_fast.cuh"

namespace pdt {
namespace {

// Kaiser-Bessel kernel and its continuous Fourier transform (host, double precision).
double kb(double dd, int kw, double beta) {
  const double t = 2.0 * dd / kw;
  if (std::fabs(t) > 1.0) return 0.0;
  return std::cyl_bessel_i(0.0, beta * std::sqrt(1.0 - t * t));
}
double kb_ft(int m, int G, int kw, double beta) {
  const int P = 4000;  // composite Simpson over the support
  const double a = -0.5 * kw, h = (double)kw / P;
  double s = 0;
  for (int i = 0; i <= P; ++i) {
    const double t = a + i * h;
    s += kb(t, kw, beta) * std::cos(2.0 * M_PI * t * m / G) * ((i == 0 || i == P) ? 1.0 : (i & 1) ? 4.0 : 2.0);
  }
  return s * h / 3.0;
}

}  // namespace

class RadialOp : public OpImpl, public SolverHooks {
 public:
  RadialOp(pdt_op_kind kind, const std::map<std::string, std::string>& cfg)
      : OpImpl(kind, "MriRadialOperator", kind == PDT_OP_RADIAL ? 3u : 2u, cfg) {
    // OperatorBase(..., config, 4, 4) then getConfigDouble / getConfigInt (mriradialoperator.cu:28-35)
    if (cfg_.size() != 4) {
      std::ostringstream os;
      os << "Operator '" << name_ << "': Invalid amount of configuration parameters (min: 4 max: 4) required, got ("
         << cfg_.size() << ").";
      throw Error(PDT_ERR_CONFIG, os.str());
    }
    osf_ = get<double>("osf");
    sector_width_ = get<int>("sector_width");
    kernel_width_ = get<int>("kernel_width");
    img_dim_ = get<int>("img_dim");
    if (img_dim_ < 1 || osf_ < 1.0 || kernel_width_ < 1 || kernel_width_ > kMaxKw)
      throw Error(PDT_ERR_CONFIG, "Operator '" + name_ + "': unsupported configuration (img_dim >= 1, osf >= 1, "
                                  "1 <= kernel_width <= " + std::to_string(kMaxKw) + ")");
  }

  Dims input_size(const Dims&) override { return {img_dim_, img_dim_}; }
  Dims natural_input_size() override { return {img_dim_, img_dim_}; }
  Dims output_size(const Dims&) override {
    const Dims& t = constant(0, PDT_F32, 2).size;
    return {t[0], multi() ? constant(2, PDT_C64, 3).size[2] : (int64_t)1};
  }
  SolverHooks* hooks() override { return this; }

  // SolverHooks: the k-space layout is the user layout (C, Ns).
  size_t compact_elems() override {
    prepare();
    return (size_t)dev_.C * dev_.Ns;
  }
  void gather(const float2* dense, float2* compact, cudaStream_t st) override {
    prepare();
    PDT_CUDA_CHECK(cudaMemcpyAsync(compact, dense, sizeof(float2) * dev_.C * dev_.Ns, cudaMemcpyDeviceToDevice, st));
  }
  void scatter(const float2* compact, float2* dense, cudaStream_t st) override {
    prepare();
    PDT_CUDA_CHECK(cudaMemcpyAsync(dense, compact, sizeof(float2) * dev_.C * dev_.Ns, cudaMemcpyDeviceToDevice, st));
  }
  int groups() override {
    prepare();
    return G_;
  }
  long long group_stride() override { return (long long)dev_.N * dev_.N; }
  void round(const float2* ubar, float2* r, const float2* fc, float sigma, float lambda, float2* khr, int* tick,
             cudaStream_t st, PhaseMarker* mk, const DualStep*) override {
    prepare();
    if (tick) launch_tick(tick, st);
    forward_grid(ubar, st, mk);
    launch_degrid(1, nullptr, r, fc, sigma, lambda, st);
    if (mk) mk->mark("rad_degrid_prox", st);
    adjoint_from_weighted(svals_.as<float2>(), khr, G_, st, mk);
  }
  void adjoint_compact(const float2* fc, float2* img, cudaStream_t st) override {
    prepare();
    launch_weight(fc, st);
    adjoint_from_weighted(svals_.as<float2>(), img, 1, st, nullptr);
  }

 protected:
  // sizeCheck (mriradialoperator.cu:44-55 multi-coil, 196-205 single-coil)
  void size_check(const Dims& src, const Dims& dst) override {
    size_check_eq(src, Dims{img_dim_, img_dim_});
    if (dst.size() != 2) throw Error(PDT_ERR_SIZE, name_ + ": k-space must be 2-D, got " + dims_str(dst));
    const int64_t nCh = dst[1], kdim = dst[0];
    size_check_eq(constant(0, PDT_F32, 2).size, Dims{kdim, 2});
    size_check_eq(constant(1, PDT_F32, 2).size, Dims{kdim, 1});
    if (multi()) size_check_eq(constant(2, PDT_C64, 3).size, Dims{img_dim_, img_dim_, nCh});
  }
  void execute_forward(const float2* src, float2* dst, cudaStream_t st) override {
    prepare();
    forward_grid(src, st, nullptr);
    launch_degrid(0, dst, nullptr, nullptr, 0.f, 0.f, st);
  }
  void execute_adjoint(const float2* src, float2* dst, cudaStream_t st) override {
    prepare();
    launch_weight(src, st);
    adjoint_from_weighted(svals_.as<float2>(), dst, 1, st, nullptr);
  }
  void invalidate() override { prepared_ = false; }

 private:
  bool multi() const { return kind_ == PDT_OP_RADIAL; }

  template <class T>
  T get(const std::string& key) const {
    auto it = cfg_.find(key);
    std::string why;
    T v{};
    if (it == cfg_.end()) {
      why = "key net found!";
    } else {
      std::istringstream ss(it->second);
      ss >> v;
      if (ss.fail()) why = "could not parse!";
    }
    if (!why.empty())
      throw Error(PDT_ERR_CONFIG, why + "\nOperator '" + name_ + "': could not parse configuration parameter '" +
                                      key + "'!\n");
    return v;
  }

  // mode 0: kout = A u; mode 1: k-space dual prox into r and the weighted samples svals_
  void launch_degrid(int mode, float2* kout, float2* r, const float2* fc, float sigma, float lambda,
                     cudaStream_t st) {
    constexpr int kDegridCoils = 4;  // coils per thread; the chunks are spread over grid.y
    const dim3 nb((dev_.Ns + kRT - 1) / kRT, (dev_.C + kDegridCoils - 1) / kDegridCoils);
    if (dev_.kw == 3)
      rad_degrid<kDegridCoils, 3><<<nb, kRT, 0, st>>>(dev_, mode, grid_.as<float2>(), kout, r, fc, svals_.as<float2>(),
                                                      sigma, lambda);
    else
      rad_degrid<kDegridCoils, 0><<<nb, kRT, 0, st>>>(dev_, mode, grid_.as<float2>(), kout, r, fc, svals_.as<float2>(),
                                                      sigma, lambda);
    PDT_LAUNCH_CHECK();
    count_launch();
  }

  void launch_weight(const float2* k, cudaStream_t st) {
    const size_t n = (size_t)dev_.C * dev_.Ns;
    rad_weight<<<(int)std::min<size_t>((n + 255) / 256, 4096), 256, 0, st>>>(dev_, k, svals_.as<float2>());
    PDT_LAUNCH_CHECK();
    count_launch();
  }

  // grid_ <- FFT2 of the deapodised, zero-padded coil images.
  void forward_grid(const float2* u, cudaStream_t st, PhaseMarker* mk) {
    if (fast_.ok()) {
      const int R = fast_.per_block();
      fast_.rows_fwd<<<dim3((dev_.N + R - 1) / R, dev_.C), 32 * kRadWpb, rad_fast_rows_smem(fast_), st>>>(
          dev_, u, tbuf_.as<float2>());
      PDT_LAUNCH_CHECK();
      count_launch();
      if (mk) mk->mark("rad_rows_fwd", st);
      fast_.cols<<<dim3((dev_.G + R - 1) / R, dev_.C), 32 * kRadWpb, rad_fast_cols_smem(fast_), st>>>(
          dev_, tbuf_.as<float2>(), grid_.as<float2>());
      PDT_LAUNCH_CHECK();
      count_launch();
      if (mk) mk->mark("rad_cols_fwd", st);
      return;
    }
    const size_t smr = sizeof(float2) * ((size_t)dev_.G + 2 * (size_t)kRR * dev_.ldG);
    const size_t smc = sizeof(float2) * ((size_t)dev_.G + 2 * (size_t)kRC * dev_.ldG);
    rad_rows_fwd<<<dim3((dev_.N + kRR - 1) / kRR, dev_.C), kRT, smr, st>>>(dev_, u, tbuf_.as<float2>());
    PDT_LAUNCH_CHECK();
    count_launch();
    if (mk) mk->mark("rad_rows_fwd", st);
    rad_cols<<<dim3((dev_.G + kRC - 1) / kRC, dev_.C), kRT, smc, st>>>(dev_, tbuf_.as<float2>(), grid_.as<float2>());
    PDT_LAUNCH_CHECK();
    count_launch();
    if (mk) mk->mark("rad_cols_fwd", st);
  }

  // out (G partial images) <- K^H applied to the already weighted samples s.
  void adjoint_from_weighted(const float2* s, float2* out, int G, cudaStream_t st, PhaseMarker* mk) {
    const int hblk = (dev_.n_heavy + kRT / 32 - 1) / (kRT / 32);
    const int nblk = hblk + (int)(((size_t)dev_.G * dev_.G + kRT - 1) / kRT);
    if (dev_.C <= 4)
      rad_grid<4><<<nblk, kRT, 0, st>>>(dev_, s, grid_.as<float2>(), hblk);
    else if (dev_.C <= 8)
      rad_grid<8><<<nblk, kRT, 0, st>>>(dev_, s, grid_.as<float2>(), hblk);
    else
      rad_grid<16><<<nblk, kRT, 0, st>>>(dev_, s, grid_.as<float2>(), hblk);
    PDT_LAUNCH_CHECK();
    count_launch();
    if (mk) mk->mark("rad_grid", st);
    if (fast_.ok()) {
      const int R = fast_.per_block();
      fast_.cols_inv<<<dim3((dev_.G + R - 1) / R, dev_.C), 32 * kRadWpb, rad_fast_cols_smem(fast_), st>>>(
          dev_, grid_.as<float2>(), tbuf_.as<float2>());
      PDT_LAUNCH_CHECK();
      count_launch();
      if (mk) mk->mark("rad_cols_inv", st);
      fast_.rows_inv<<<dim3((dev_.N + R - 1) / R, G), 32 * kRadWpb, rad_fast_rows_inv_smem(fast_, dev_.N), st>>>(
          dev_, tbuf_.as<float2>(), out, G, (long long)dev_.N * dev_.N);
      PDT_LAUNCH_CHECK();
      count_launch();
      if (mk) mk->mark("rad_rows_inv", st);
      return;
    }
    const size_t smc = sizeof(float2) * ((size_t)dev_.G + 2 * (size_t)kRC * dev_.ldG);
    rad_cols_inv<<<dim3((dev_.G + kRC - 1) / kRC, dev_.C), kRT, smc, st>>>(dev_, grid_.as<float2>(),
                                                                           tbuf_.as<float2>());
    PDT_LAUNCH_CHECK();
    count_launch();
    if (mk) mk->mark("rad_cols_inv", st);
    const size_t smr = sizeof(float2) * ((size_t)dev_.G + 2 * (size_t)kRR * dev_.ldG + (size_t)kRR * dev_.N);
    rad_rows_inv<<<dim3((dev_.N + kRR - 1) / kRR, G), kRT, smr, st>>>(dev_, tbuf_.as<float2>(), out, G,
                                                                      (long long)dev_.N * dev_.N);
    PDT_LAUNCH_CHECK();
    count_launch();
    if (mk) mk->mark("rad_rows_inv", st);
  }

  void prepare() {
    if (prepared_) return;
    if (!g_rad_sms) {
      int dev = 0;
      PDT_CUDA_CHECK(cudaGetDevice(&dev));
      PDT_CUDA_CHECK(cudaDeviceGetAttribute(&g_rad_sms, cudaDevAttrMultiProcessorCount, dev));
      PDT_CUDA_CHECK(cudaDeviceGetAttribute(&g_rad_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
      for (const void* fn : {(const void*)rad_rows_fwd, (const void*)rad_cols, (const void*)rad_cols_inv,
                             (const void*)rad_rows_inv})
        PDT_CUDA_CHECK(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, g_rad_smem));
    }
    Constant& tc = constant(0, PDT_F32, 2);
    Constant& dc = constant(1, PDT_F32, 2);
    const int Ns = (int)tc.size[0];
    if (tc.size[1] != 2) throw Error(PDT_ERR_SIZE, name_ + ": trajectory must be {Ns, 2}, got " + dims_str(tc.size));
    size_check_eq(dc.size, Dims{Ns, 1});
    const float2* sens = nullptr;
    int C = 1;
    if (multi()) {
      Constant& sc = constant(2, PDT_C64, 3);
      size_check_eq(Dims{sc.size[0], sc.size[1]}, Dims{img_dim_, img_dim_});
      C = (int)sc.size[2];
      sens = sc.dev.as<float2>();
    }
    const int N = (int)img_dim_;
    int G = (int)std::ceil(osf_ * N - 1e-9);
    G += G & 1;
    const int kw = kernel_width_;
    const double a = (double)kw / osf_ * (osf_ - 0.5);
    const double beta = M_PI * std::sqrt(std::max(a * a - 0.8, 1e-12));
    RadDev d{};
    d.N = N;
    d.G = G;
    d.C = C;
    d.Ns = Ns;
    d.kw = kw;
    d.off = N / 2;
    d.scale = 1.0f / (float)N;
    d.ldG = G + 1;
    d.sens = sens;
    if (!make_fft_plan(G, &d.plan)) throw Error(PDT_ERR_UNSUPPORTED, name_ + ": cannot plan FFT of " + std::to_string(G));
    const size_t smr = sizeof(float2) * ((size_t)G + 2 * (size_t)kRR * d.ldG + (size_t)kRR * N);
    if (smr > (size_t)g_rad_smem) throw Error(PDT_ERR_UNSUPPORTED, name_ + ": grid too large for shared memory");
    // per-sample taps, deapodisation, tile lists
    const float* traj = reinterpret_cast<const float*>(tc.host.data());
    const float* dcf = reinterpret_cast<const float*>(dc.host.data());
    std::vector<int> g0(2 * (size_t)Ns);
    std::vector<float> wt((size_t)Ns * 2 * kw), deap(N);
    for (int j = 0; j < Ns; ++j) {
      const double ax = (double)traj[j] * G, ay = (double)traj[Ns + j] * G;
      g0[2 * j] = (int)std::ceil(ax - 0.5 * kw);
      g0[2 * j + 1] = (int)std::ceil(ay - 0.5 * kw);
      for (int t = 0; t < kw; ++t) {
        wt[((size_t)j * 2 + 0) * kw + t] = (float)kb(g0[2 * j] + t - ax, kw, beta);
        wt[((size_t)j * 2 + 1) * kw + t] = (float)kb(g0[2 * j + 1] + t - ay, kw, beta);
      }
    }
    for (int x = 0; x < N; ++x) deap[x] = (float)kb_ft(x - N / 2, G, kw, beta);
    // per-cell gather lists: every (sample, tap) pair lands in the list of the grid cell it covers;
    // samples are visited in ascending order, so each list is ascending
    auto wrap = [G](int g) { g %= G; return g < 0 ? g + G : g; };
    const size_t ncell = (size_t)G * G;
    std::vector<int> ptr(ncell + 1, 0);
    for (int j = 0; j < Ns; ++j)
      for (int ty = 0; ty < kw; ++ty)
        for (int txx = 0; txx < kw; ++txx)
          ++ptr[(size_t)wrap(g0[2 * j] + txx) * G + wrap(g0[2 * j + 1] + ty) + 1];
    for (size_t c = 0; c < ncell; ++c) ptr[c + 1] += ptr[c];
    std::vector<int> idx((size_t)ptr[ncell]), fill(ptr.begin(), ptr.end() - 1);
    std::vector<float> cw(idx.size());
    std::vector<int> heavy;
    for (size_t c = 0; c < ncell; ++c)
      if (ptr[c + 1] - ptr[c] > kHeavy) heavy.push_back((int)c);
    for (int j = 0; j < Ns; ++j)
      for (int txx = 0; txx < kw; ++txx)
        for (int ty = 0; ty < kw; ++ty) {
          const size_t cell = (size_t)wrap(g0[2 * j] + txx) * G + wrap(g0[2 * j + 1] + ty);
          const int e = fill[cell]++;
          idx[e] = j;
          cw[e] = wt[((size_t)j * 2 + 0) * kw + txx] * wt[((size_t)j * 2 + 1) * kw + ty];
        }
    std::vector<float2> tw(G);
    fill_twiddles(G, tw.data());
    std::vector<float> w(dcf, dcf + Ns);
    const size_t need = 64 * 10 + sizeof(float2) * G + sizeof(float) * (N + (size_t)Ns + wt.size() + cw.size()) +
                        sizeof(int) * (g0.size() + ptr.size() + idx.size() + heavy.size());
    tables_.ensure(need);
    char* base = tables_.as<char>();
    size_t off = 0;
    auto put = [&](const void* src, size_t bytes) {
      off = (off + 15) & ~(size_t)15;
      char* dst = base + off;
      if (bytes) PDT_CUDA_CHECK(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice));
      off += bytes;
      return dst;
    };
    d.tw = reinterpret_cast<const float2*>(put(tw.data(), sizeof(float2) * G));
    d.deap = reinterpret_cast<const float*>(put(deap.data(), sizeof(float) * N));
    d.w = reinterpret_cast<const float*>(put(w.data(), sizeof(float) * Ns));
    d.wt = reinterpret_cast<const float*>(put(wt.data(), sizeof(float) * wt.size()));
    d.g0 = reinterpret_cast<const int*>(put(g0.data(), sizeof(int) * g0.size()));
    d.cell_ptr = reinterpret_cast<const int*>(put(ptr.data(), sizeof(int) * ptr.size()));
    d.cell_idx = reinterpret_cast<const int*>(put(idx.data(), sizeof(int) * idx.size()));
    d.cell_w = reinterpret_cast<const float*>(put(cw.data(), sizeof(float) * cw.size()));
    d.heavy = reinterpret_cast<const int*>(put(heavy.data(), sizeof(int) * heavy.size()));
    d.n_heavy = (int)heavy.size();
    tbuf_.ensure(sizeof(float2) * (size_t)C * G * N);
    grid_.ensure(sizeof(float2) * (size_t)C * G * G);
    svals_.ensure(sizeof(float2) * std::max<size_t>((size_t)C * Ns, 1));
    // lane-FFT passes where the grid length has a compiled split
    fast_ = find_rad_kernels(G);
    if (fast_.ok() && (rad_fast_rows_inv_smem(fast_, N) > (size_t)g_rad_smem ||
                       rad_fast_cols_smem(fast_) > (size_t)g_rad_smem))
      fast_ = RadFastKernels();
    if (fast_.ok()) {
      for (const void* fn : {(const void*)fast_.rows_fwd, (const void*)fast_.cols, (const void*)fast_.cols_inv,
                             (const void*)fast_.rows_inv})
        PDT_CUDA_CHECK(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, g_rad_smem));
    }
    const int rows_per_block = fast_.ok() ? fast_.per_block() : kRR;
    const int row_blocks = (N + rows_per_block - 1) / rows_per_block;
    G_ = std::max(1, std::min(C, (2 * g_rad_sms + row_blocks - 1) / row_blocks));
    if (const char* env = std::getenv("PDT_RADIAL_GROUPS")) {  // coil groups of the adjoint row pass, pinned
      const int g = std::atoi(env);
      if (g < 1 || g > C) throw Error(PDT_ERR_INVALID_ARGUMENT, "PDT_RADIAL_GROUPS must be 1 .. coils");
      G_ = g;
    }
    dev_ = d;
    prepared_ = true;
  }

  double osf_ = 1;
  int64_t sector_width_ = 0, kernel_width_ = 0, img_dim_ = 0;
  bool prepared_ = false;
  RadDev dev_{};
  RadFastKernels fast_;
  int G_ = 1;
  DevBuf tables_, tbuf_, grid_, svals_;
};

std::shared_ptr<OpImpl> make_radial_operator(pdt_op_kind kind, const std::map<std::string, std::string>& cfg) {
  return std::make_shared<RadialOp>(kind, cfg);
}

}  // namespace pdt
