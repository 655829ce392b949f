// pdt_oracle.cpp -- TEST INFRASTRUCTURE ONLY (the checker, never the product).
//
// CPU restatement of the primal-dual toolbox's hot path: the TV / TGV^2 primal-dual iterations and
// the Cartesian / sampling MRI operators. It is used by tests/ (parity), __graft_entry__.smoke()
// (one small check) and bench.py's cpu_baseline leg (timed CPU baseline). The product library never
// links, loads or calls this file.
//
// Two precisions:
//   * f64  -- every operation in double: the accuracy oracle.
//   * f32  -- "FP32 mirror": the pointwise / stencil arithmetic runs in float in the same operation
//             order as the reference's CUDA kernels (including the reference's double-precision
//             promotions of literals such as `2.0 * sqr(...)` and `1.0 / max(...)`); the FFTs are
//             computed in double and rounded to float (the reference calls cuFFT through
//             ImageUtilities, whose exact rounding cannot be mirrored).
//
// Every function cites the reference file:line it restates (paths inside the reference project).
// Parity pins: the reference ships no optimizer output golden vectors and cannot be built here
// (ImageUtilities and gpuNUFFT submodules are absent). This oracle is pinned by (1) the reference's own
// adjointness test (tests/main_adjointness_test.cu:28-120, shapes 10x10x5 double2), (2) numpy.fft for
// the orthonormal FFT that ImageUtilities provides, and (3) the reference's mask/trajectory fixtures.
//
// Layout: ImageUtilities order, x (phase-encoding, W) fastest, then y (frequency-encoding, H), then coil.
// Complex data is interleaved (re, im) -- identical to numpy complex64/complex128 arrays of shape
// (C, H, W) in C order.

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>
#include <algorithm>
#include <cmath>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ------------------------------------------------------------------------------------------------
// Scalar / complex pixel arithmetic (iu::type_trait and iuhelpermath equivalents).
// ------------------------------------------------------------------------------------------------
template <class R> struct cx { R x, y; };
template <class R> inline cx<R> operator+(cx<R> a, cx<R> b) { return {a.x + b.x, a.y + b.y}; }
template <class R> inline cx<R> operator-(cx<R> a, cx<R> b) { return {a.x - b.x, a.y - b.y}; }
template <class R> inline cx<R> operator-(cx<R> a) { return {-a.x, -a.y}; }
template <class R> inline cx<R> operator*(R s, cx<R> a) { return {s * a.x, s * a.y}; }
template <class R> inline cx<R> operator*(cx<R> a, R s) { return {a.x * s, a.y * s}; }
template <class R> inline cx<R> operator/(cx<R> a, R s) { return {a.x / s, a.y / s}; }
template <class R> inline cx<R>& operator+=(cx<R>& a, cx<R> b) { a.x += b.x; a.y += b.y; return a; }
template <class R> inline cx<R>& operator/=(cx<R>& a, R s) { a.x /= s; a.y /= s; return a; }
// complex_multiply(a, b) and complex_multiply_conjugate(a, b) = a * conj(b)
template <class R> inline cx<R> cmul(cx<R> a, cx<R> b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
template <class R> inline cx<R> cmulc(cx<R> a, cx<R> b) { return {a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y}; }

template <class R> inline R pabs(R a) { return std::fabs(a); }
template <class R> inline R pabs(cx<R> a) { return std::sqrt(a.x * a.x + a.y * a.y); }
template <class R> inline R zero_of(R*) { return R(0); }
template <class R> inline cx<R> zero_of(cx<R>*) { return {R(0), R(0)}; }
template <class P> inline P pzero() { return zero_of((P*)nullptr); }

template <class P> struct real_of;
template <> struct real_of<float> { typedef float type; };
template <> struct real_of<double> { typedef double type; };
template <> struct real_of<cx<float>> { typedef float type; };
template <> struct real_of<cx<double>> { typedef double type; };

template <class R> inline R sqr(R a) { return a * a; }

// ------------------------------------------------------------------------------------------------
// Stencils: tgv_kernels.cuh:25-165 (dp, dp_sym, dm, dm_sym, norm, norm_sym).
// Forward differences with Neumann boundary (xp = x + (x < W-1)), divergence as the exact negative
// adjoint with the reference's boundary rows.
// ------------------------------------------------------------------------------------------------
template <class P>
inline void dp(const P* u, int W, int H, int x, int y, P& gx, P& gy) {  // tgv_kernels.cuh:40-50
  const int xp = x + (x < W - 1), yp = y + (y < H - 1);
  const P c = u[x + (size_t)W * y];
  gx = u[xp + (size_t)W * y] - c;
  gy = u[x + (size_t)W * yp] - c;
}

template <class P>
inline void dp_sym(const P* vx, const P* vy, int W, int H, int x, int y, P& gxx, P& gyy, P& gxy) {
  // tgv_kernels.cuh:25-38; the literal 0.5 is double in the reference.
  typedef typename real_of<P>::type R;
  const int xp = x + (x < W - 1), yp = y + (y < H - 1);
  const size_t i = x + (size_t)W * y;
  gxx = vx[xp + (size_t)W * y] - vx[i];
  gxy = (R)0.5 * (vx[x + (size_t)W * yp] - vx[i] + vy[xp + (size_t)W * y] - vy[i]);
  gyy = vy[x + (size_t)W * yp] - vy[i];
}

template <class P>
inline P dm(const P* px, const P* py, int W, int H, int x, int y) {  // tgv_kernels.cuh:67-80
  const size_t i = x + (size_t)W * y;
  P d = (x > 0) ? ((x < W - 1) ? px[i] - px[i - 1] : -px[i - 1]) : px[i];
  d += (y > 0) ? ((y < H - 1) ? py[i] - py[i - W] : -py[i - W]) : py[i];
  return d;
}

template <class P>
inline void dm_sym(const P* qxx, const P* qyy, const P* qxy, int W, int H, int x, int y, P& dx, P& dy) {
  // tgv_kernels.cuh:104-134
  const size_t i = x + (size_t)W * y;
  P a = (x > 0) ? ((x < W - 1) ? qxx[i] - qxx[i - 1] : -qxx[i - 1]) : qxx[i];
  P b = (y > 0) ? ((y < H - 1) ? qyy[i] - qyy[i - W] : -qyy[i - W]) : qyy[i];
  P c = (x > 0) ? ((x < W - 1) ? qxy[i] - qxy[i - 1] : -qxy[i - 1]) : qxy[i];
  P d = (y > 0) ? ((y < H - 1) ? qxy[i] - qxy[i - W] : -qxy[i - W]) : qxy[i];
  dx = a + d;
  dy = b + c;
}

// norm(p_x, p_y) = sqrt(|p_x|^2 + |p_y|^2)  (tgv_kernels.cuh:147-154)
template <class P>
inline typename real_of<P>::type norm2(P a, P b) {
  return std::sqrt(sqr(pabs(a)) + sqr(pabs(b)));
}
// norm_sym = sqrt(|qxx|^2 + |qyy|^2 + 2.0*|qxy|^2): the reference's `2.0` promotes the sum to double
// (tgv_kernels.cuh:136-145).
template <class P>
inline typename real_of<P>::type norm_sym(P a, P b, P c) {
  typedef typename real_of<P>::type R;
  return (R)std::sqrt((double)(sqr(pabs(a)) + sqr(pabs(b))) + 2.0 * (double)sqr(pabs(c)));
}
// scale = 1.0 / max(1.0, n / alpha): double division of a real_type maximum, rounded to real_type.
template <class R>
inline R proj_scale(R n, R alpha) {
  R m = n / alpha;
  m = (R(1) > m) ? R(1) : m;
  return (R)(1.0 / (double)m);
}

// ------------------------------------------------------------------------------------------------
// Kernels, one pass each, following the reference kernels element by element.
// ------------------------------------------------------------------------------------------------
template <class P, class R>
void tv_dual_p(P* px, P* py, const P* ubar, int W, int H, R sigma, R alpha) {
  // tgv_kernels.cuh:294-324 (alpha=1 there; the with-alpha form is TGV_dual_p without v).
#pragma omp parallel for schedule(static)
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      P gx, gy;
      dp(ubar, W, H, x, y, gx, gy);
      const size_t i = x + (size_t)W * y;
      P a = px[i] + sigma * gx, b = py[i] + sigma * gy;
      R s = proj_scale(norm2(a, b), alpha);
      px[i] = a * s;
      py[i] = b * s;
    }
}

template <class P, class R>
void tgv_dual_p(P* px, P* py, const P* ubar, const P* vbx, const P* vby, int W, int H, R sigma, R alpha1) {
  // tgv_kernels.cuh:260-292
#pragma omp parallel for schedule(static)
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      P gx, gy;
      dp(ubar, W, H, x, y, gx, gy);
      const size_t i = x + (size_t)W * y;
      P a = px[i] + sigma * (gx - vbx[i]);
      P b = py[i] + sigma * (gy - vby[i]);
      R s = proj_scale(norm2(a, b), alpha1);
      px[i] = a * s;
      py[i] = b * s;
    }
}

template <class P, class R>
void tgv_dual_q(P* qxx, P* qyy, P* qxy, const P* vbx, const P* vby, int W, int H, R sigma, R alpha0) {
  // tgv_kernels.cuh:225-258
#pragma omp parallel for schedule(static)
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      P gxx, gyy, gxy;
      dp_sym(vbx, vby, W, H, x, y, gxx, gyy, gxy);
      const size_t i = x + (size_t)W * y;
      P a = qxx[i] + sigma * gxx, b = qyy[i] + sigma * gyy, c = qxy[i] + sigma * gxy;
      R s = proj_scale(norm_sym(a, b, c), alpha0);
      qxx[i] = a * s;
      qyy[i] = b * s;
      qxy[i] = c * s;
    }
}

template <class P, class R>
void tv_primal_u(P* u, P* ubar, const P* f, const P* px, const P* py, int W, int H, R tau, R lambda) {
  // tgv_kernels.cuh:568-605 (theta = 1)
  const R theta = 1;
#pragma omp parallel for schedule(static)
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      const size_t i = x + (size_t)W * y;
      P uo = u[i];
      P d = dm(px, py, W, H, x, y);
      P un = uo + tau * (d + lambda * f[i]);
      un /= (R(1) + tau * lambda);
      u[i] = un;
      ubar[i] = (R(1) + theta) * un - theta * uo;
    }
}

template <class P, class R>
void tgv_primal_u_noprox(P* u, P* ubar_khr, const P* px, const P* py, int W, int H, R tau) {
  // tgv_kernels.cuh:432-467: K^H r is read from the u-bar buffer, then u-bar is overwritten.
  const R theta = 1;
#pragma omp parallel for schedule(static)
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      const size_t i = x + (size_t)W * y;
      P uo = u[i];
      P f = ubar_khr[i];
      P d = dm(px, py, W, H, x, y);
      P un = uo + tau * (d - f);
      u[i] = un;
      ubar_khr[i] = (R(1) + theta) * un - theta * uo;
    }
}

template <class P, class R>
void tgv_primal_v(P* vx, P* vy, P* vbx, P* vby, const P* px, const P* py, const P* qxx, const P* qyy,
                  const P* qxy, int W, int H, R tau) {
  // tgv_kernels.cuh:647-686
  const R theta = 1;
#pragma omp parallel for schedule(static)
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      const size_t i = x + (size_t)W * y;
      P ox = vx[i], oy = vy[i];
      P dx, dy;
      dm_sym(qxx, qyy, qxy, W, H, x, y, dx, dy);
      P nx = ox + tau * (dx + px[i]);
      P ny = oy + tau * (dy + py[i]);
      vx[i] = nx;
      vy[i] = ny;
      vbx[i] = (R(1) + theta) * nx - theta * ox;
      vby[i] = (R(1) + theta) * ny - theta * oy;
    }
}

template <class P, class R>
void prox_r(P* r, const P* t, size_t n, R sigma, R lambda) {
  // tgv_kernels.cuh:212-223
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < (long long)n; ++i) r[i] = (r[i] + sigma * t[i]) / (R(1) + sigma * lambda);
}

// ------------------------------------------------------------------------------------------------
// FFT (double): mixed-radix recursive decimation in time, direct DFT for prime factors. This is the
// orthonormal 2-D FFT that ImageUtilities' iu::math::fft::fft2/ifft2(..., true) provides
// (mricartesianoperator.cu:218-219, 252-253); checked against numpy.fft in tests.
// ------------------------------------------------------------------------------------------------
typedef cx<double> cd;

// Self-sorting (Stockham) mixed-radix FFT: for each radix R with Ns = product of earlier radices,
// butterfly j reads a[j + r*n/R], twiddles by w_{Ns*R}^{r*(j%Ns)}, takes an R-point DFT and writes
// b[(j/Ns)*Ns*R + j%Ns + r*Ns]. Radices: 4 and 2 first, then odd primes (direct DFT).
struct FftPlan {
  int n = 0;
  std::vector<int> radix;
  std::vector<cd> tw;  // tw[t] = exp(-2 pi i t / n)
};

static FftPlan make_plan(int n) {
  FftPlan p;
  p.n = n;
  int m = n;
  while (m % 4 == 0) { p.radix.push_back(4); m /= 4; }
  while (m % 2 == 0) { p.radix.push_back(2); m /= 2; }
  for (int f = 3; m > 1; f += 2)
    while (m % f == 0) { p.radix.push_back(f); m /= f; }
  p.tw.resize((size_t)n);
  for (int t = 0; t < n; ++t) {
    const double a = -2.0 * M_PI * (double)t / (double)n;
    p.tw[t] = {std::cos(a), std::sin(a)};
  }
  return p;
}

static const FftPlan& get_plan(int n) {
  thread_local std::vector<FftPlan> cache;
  for (const auto& p : cache)
    if (p.n == n) return p;
  cache.push_back(make_plan(n));
  return cache.back();
}

// Unscaled 1-D FFT of contiguous data (sign -1 forward, +1 inverse), in place.
static void fft_contig(cd* data, int n, int sign) {
  if (n <= 1) return;
  const FftPlan& p = get_plan(n);
  thread_local std::vector<cd> work;
  thread_local std::vector<cd> v;
  if ((int)work.size() < n) work.resize((size_t)n);
  cd* a = data;
  cd* b = work.data();
  int Ns = 1;
  for (int R : p.radix) {
    if ((int)v.size() < R) v.resize((size_t)R);
    const int nb = n / R;
    const int step = n / (Ns * R);  // twiddle-table stride for w_{Ns*R}
    const int rstep = n / R;        // twiddle-table stride for w_R
    for (int j = 0; j < nb; ++j) {
      const int k = j % Ns;
      for (int r = 0; r < R; ++r) {
        cd x = a[j + r * nb];
        cd w = p.tw[(size_t)r * k * step];
        if (sign > 0) w.y = -w.y;
        v[r] = cmul(x, w);
      }
      const int idxD = (j / Ns) * Ns * R + k;
      for (int q = 0; q < R; ++q) {
        double sr = 0, si = 0;
        for (int r = 0; r < R; ++r) {
          cd w = p.tw[(size_t)((r * q) % R) * rstep];
          if (sign > 0) w.y = -w.y;
          sr += v[r].x * w.x - v[r].y * w.y;
          si += v[r].x * w.y + v[r].y * w.x;
        }
        b[idxD + q * Ns] = {sr, si};
      }
    }
    std::swap(a, b);
    Ns *= R;
  }
  if (a != data) std::copy(a, a + n, data);
}

static void fft1(cd* data, size_t stride, int n, int sign) {
  if (stride == 1) { fft_contig(data, n, sign); return; }
  thread_local std::vector<cd> col;
  if ((int)col.size() < n) col.resize((size_t)n);
  for (int i = 0; i < n; ++i) col[i] = data[i * stride];
  fft_contig(col.data(), n, sign);
  for (int i = 0; i < n; ++i) data[i * stride] = col[i];
}

// In-place 2-D FFT over (x: W, y: H) of `nb` stacked planes, scaled by 1/sqrt(W*H).
static void fft2_planes(cd* d, int W, int H, int nb, int sign) {
  const double s = 1.0 / std::sqrt((double)W * (double)H);
#pragma omp parallel for schedule(static)
  for (long long t = 0; t < (long long)nb * H; ++t) fft1(d + (size_t)t * W, 1, W, sign);
#pragma omp parallel for schedule(static)
  for (long long t = 0; t < (long long)nb * W; ++t) {
    const long long b = t / W, x = t % W;
    fft1(d + (size_t)b * W * H + x, (size_t)W, H, sign);
  }
  const size_t n = (size_t)nb * W * H;
  for (size_t i = 0; i < n; ++i) d[i] = d[i] * s;
}

// Shift conventions: the reference's own ifftshift (mricartesianoperator.cu:41-49, 85-93) writes
// dst[(i + mid) % n] = src[i] with mid = int((n + 1.f) / 2.f). ImageUtilities' fftshift2 source is
// absent; it is taken as the numpy fftshift, dst[(i + n/2) % n] = src[i]. Both agree for even n.
inline int mid_ifftshift(int n) { return (int)(((float)n + 1.f) / 2.f); }
inline int mid_fftshift(int n) { return n / 2; }

// ------------------------------------------------------------------------------------------------
// Cartesian multi-coil operator (+ROOS) and single-coil sampling operator.
// kind: 0 = MriCartesianOperator, 1 = MriCartesianRemoveROOSOperator, 2 = MriSamplingOperator.
// ------------------------------------------------------------------------------------------------
enum { K_CART = 0, K_ROOS = 1, K_SAMPLING = 2 };

template <class R>
struct CartOp {
  int kind, W, Hf, C, Hi, y0;
  const cx<R>* sens;  // (W, Hf, C); null for the sampling operator
  const R* mask;      // (W, Hf)
  CartOp(int kind_, int W_, int Hf_, int C_, const cx<R>* sens_, const R* mask_)
      : kind(kind_), W(W_), Hf(Hf_), C(kind_ == K_SAMPLING ? 1 : C_), sens(sens_), mask(mask_) {
    if (kind == K_ROOS) {
      Hi = Hf / 2;
      // mricartesianoperator.cu:341 / :381: `unsigned int FE_idx = size[1] * 0.25f + 1;`
      y0 = (int)(unsigned int)((float)(unsigned int)Hf * 0.25f + 1.f);
    } else {
      Hi = Hf;
      y0 = 0;
    }
  }
  size_t img_n() const { return (size_t)W * Hi; }
  size_t ksp_n() const { return (size_t)W * Hf * C; }
  int img_w() const { return W; }
  int img_h() const { return Hi; }

  // forward: mricartesianoperator.cu:320-365 (ROOS) / 196-225 (plain); mrisamplingoperator.cu:59-70
  void forward(const cx<R>* u, cx<R>* k) const {
    const int mx = mid_ifftshift(W), my = mid_ifftshift(Hf);
    const int ox = mid_fftshift(W), oy = mid_fftshift(Hf);
    std::vector<cd> buf((size_t)W * Hf * C);
#pragma omp parallel for schedule(static)
    for (int c = 0; c < C; ++c)
      for (int y = 0; y < Hf; ++y)
        for (int x = 0; x < W; ++x) {
          // padFOV (mricartesianoperator.cu:145-160): image rows live at [y0, y0 + Hi)
          cx<R> img = {0, 0};
          if (y >= y0 && y < y0 + Hi) img = u[x + (size_t)W * (y - y0)];
          cx<R> v = sens ? cmul(img, sens[x + (size_t)W * (y + (size_t)Hf * c)]) : img;  // prefft_kernel
          const int xd = (x + mx) % W, yd = (y + my) % Hf;
          buf[xd + (size_t)W * (yd + (size_t)Hf * c)] = {(double)v.x, (double)v.y};
        }
    fft2_planes(buf.data(), W, Hf, C, -1);
#pragma omp parallel for schedule(static)
    for (int c = 0; c < C; ++c)
      for (int y = 0; y < Hf; ++y)
        for (int x = 0; x < W; ++x) {
          const cd v = buf[x + (size_t)W * (y + (size_t)Hf * c)];
          const int xd = (x + ox) % W, yd = (y + oy) % Hf;  // fftshift2
          const size_t o = xd + (size_t)W * (yd + (size_t)Hf * c);
          const R m = mask[xd + (size_t)W * yd];
          cx<R> kv = {(R)v.x, (R)v.y};
          k[o] = kv * m;  // applyMask_kernel
        }
  }

  // adjoint: mricartesianoperator.cu:367-414 (ROOS) / 227-265 (plain); mrisamplingoperator.cu:72-88
  void adjoint(const cx<R>* k, cx<R>* u) const {
    const int mx = mid_ifftshift(W), my = mid_ifftshift(Hf);
    const int ox = mid_fftshift(W), oy = mid_fftshift(Hf);
    std::vector<cd> buf((size_t)W * Hf * C);
#pragma omp parallel for schedule(static)
    for (int c = 0; c < C; ++c)
      for (int y = 0; y < Hf; ++y)
        for (int x = 0; x < W; ++x) {
          const size_t i = x + (size_t)W * (y + (size_t)Hf * c);
          cx<R> v = k[i] * mask[x + (size_t)W * y];  // preifft_kernel
          const int xd = (x + mx) % W, yd = (y + my) % Hf;
          buf[xd + (size_t)W * (yd + (size_t)Hf * c)] = {(double)v.x, (double)v.y};
        }
    fft2_planes(buf.data(), W, Hf, C, +1);
    std::vector<cx<R>> g((size_t)W * Hf * C);
    for (int c = 0; c < C; ++c)
      for (int y = 0; y < Hf; ++y)
        for (int x = 0; x < W; ++x) {
          const cd v = buf[x + (size_t)W * (y + (size_t)Hf * c)];
          const int xd = (x + ox) % W, yd = (y + oy) % Hf;
          g[xd + (size_t)W * (yd + (size_t)Hf * c)] = {(R)v.x, (R)v.y};
        }
#pragma omp parallel for schedule(static)
    for (int yi = 0; yi < Hi; ++yi)
      for (int x = 0; x < W; ++x) {
        const int y = yi + y0;  // cropFOV (mricartesianoperator.cu:128-143)
        cx<R> s = {0, 0};
        if (sens) {
          for (int c = 0; c < C; ++c) {  // combineImg_kernel (mricartesianoperator.cu:99-126)
            const size_t i = x + (size_t)W * (y + (size_t)Hf * c);
            s += cmulc(g[i], sens[i]);
          }
        } else {
          s = g[x + (size_t)W * y];
        }
        u[x + (size_t)W * yi] = s;
      }
  }
};


// ------------------------------------------------------------------------------------------------
// Radial operators (MriRadialOperator / MriRadialSinglecoilOperator, mriradialoperator.cu:27-321).
// The reference delegates to gpuNUFFT (github.com/andyschwarzl/gpuNUFFT, submodule pin not recorded,
// .gitmodules:4-6), which is absent here; this restates its published method (Knoll et al., ISMRM 2014:
// Kaiser-Bessel gridding on an osf-oversampled grid, deapodisation, density compensation) with the
// Kaiser-Bessel shape of Beatty et al. (IEEE TMI 2005): beta = pi sqrt((W/osf)^2 (osf - 1/2)^2 - 0.8).
// Convention (parity with gpuNUFFT is unpinned; see the tests):
//   A u [c, j] = w_j / N * sum_{x,y} sens_c(x,y) u(x,y) exp(-2 pi i (k0_j (x - N/2) + k1_j (y - N/2)))
// approximated by: deapodise, zero-pad into G = ceil(osf N) (even), FFT, interpolate with the separable
// kernel at kappa = k G; the adjoint is its exact transpose. Trajectory constant {Ns, 2} is planar
// (k0 for every sample, then k1); k0 pairs with image x (fastest), k1 with y.
// ------------------------------------------------------------------------------------------------
inline int radial_grid_size(int N, double osf) {
  int G = (int)std::ceil(osf * N - 1e-9);
  return G + (G & 1);
}
inline double kb_beta(int kw, double osf) {
  const double a = (double)kw / osf * (osf - 0.5);
  return M_PI * std::sqrt(std::max(a * a - 0.8, 1e-12));
}
inline double kb_kernel(double d, int kw, double beta) {
  const double t = 2.0 * d / kw;
  if (std::fabs(t) > 1.0) return 0.0;
  return std::cyl_bessel_i(0.0, beta * std::sqrt(1.0 - t * t));
}
// deap(m) = integral of the kernel times cos(2 pi t m / G) over its support (composite Simpson, 4000 panels).
inline double kb_deapod(int m, int G, int kw, double beta) {
  const int P = 4000;
  const double a = -0.5 * kw, h = (double)kw / P;
  double s = 0;
  for (int i = 0; i <= P; ++i) {
    const double t = a + i * h;
    const double f = kb_kernel(t, kw, beta) * std::cos(2.0 * M_PI * t * m / G);
    s += f * ((i == 0 || i == P) ? 1.0 : (i & 1) ? 4.0 : 2.0);
  }
  return s * h / 3.0;
}

template <class R>
struct RadialOp {
  int N, G, kw, C, Ns;
  double beta;
  const cx<R>* sens;  // (N, N, C) or null
  std::vector<double> k0, k1, w, deap;
  std::vector<int> gx0, gy0;
  std::vector<double> wx, wy;  // [j][kw]
  RadialOp(int N_, double osf, int kw_, int C_, int Ns_, const R* traj, const R* dcf, const cx<R>* sens_)
      : N(N_), kw(kw_), C(sens_ ? C_ : 1), Ns(Ns_), sens(sens_) {
    G = radial_grid_size(N, osf);
    beta = kb_beta(kw, osf);
    k0.resize(Ns);
    k1.resize(Ns);
    w.resize(Ns);
    gx0.resize(Ns);
    gy0.resize(Ns);
    wx.resize((size_t)Ns * kw);
    wy.resize((size_t)Ns * kw);
    for (int j = 0; j < Ns; ++j) {
      k0[j] = traj[j];
      k1[j] = traj[Ns + j];
      w[j] = dcf[j];
      const double ax = k0[j] * G, ay = k1[j] * G;
      gx0[j] = (int)std::ceil(ax - 0.5 * kw);
      gy0[j] = (int)std::ceil(ay - 0.5 * kw);
      for (int t = 0; t < kw; ++t) {
        wx[(size_t)j * kw + t] = kb_kernel(gx0[j] + t - ax, kw, beta);
        wy[(size_t)j * kw + t] = kb_kernel(gy0[j] + t - ay, kw, beta);
      }
    }
    deap.resize(N);
    for (int x = 0; x < N; ++x) deap[x] = kb_deapod(x - N / 2, G, kw, beta);
  }
  size_t img_n() const { return (size_t)N * N; }
  size_t ksp_n() const { return (size_t)C * Ns; }
  int img_w() const { return N; }
  int img_h() const { return N; }
  int wrap(int g) const { g %= G; return g < 0 ? g + G : g; }

  void forward(const cx<R>* u, cx<R>* k) const {
    std::vector<cd> grid((size_t)G * G * C);
    const double sc = 1.0 / N;
    for (int c = 0; c < C; ++c)
      for (int y = 0; y < N; ++y)
        for (int x = 0; x < N; ++x) {
          const size_t i = x + (size_t)N * y;
          cd v = {(double)u[i].x, (double)u[i].y};
          if (sens) v = cmul(v, cd{(double)sens[i + (size_t)N * N * c].x, (double)sens[i + (size_t)N * N * c].y});
          const double f = sc / (deap[x] * deap[y]);
          grid[wrap(x - N / 2) + (size_t)G * (wrap(y - N / 2) + (size_t)G * c)] = v * f;
        }
    fft2_unscaled(grid.data(), C, -1);
    for (int c = 0; c < C; ++c)
      for (int j = 0; j < Ns; ++j) {
        cd a = {0, 0};
        for (int ty = 0; ty < kw; ++ty)
          for (int tx = 0; tx < kw; ++tx) {
            const double wt = wx[(size_t)j * kw + tx] * wy[(size_t)j * kw + ty];
            a += grid[wrap(gx0[j] + tx) + (size_t)G * (wrap(gy0[j] + ty) + (size_t)G * c)] * wt;
          }
        a = a * w[j];
        k[j + (size_t)Ns * c] = {(R)a.x, (R)a.y};
      }
  }
  void adjoint(const cx<R>* k, cx<R>* u) const {
    std::vector<cd> grid((size_t)G * G * C, cd{0, 0});
    for (int c = 0; c < C; ++c)
      for (int j = 0; j < Ns; ++j) {
        const cd s = cd{(double)k[j + (size_t)Ns * c].x, (double)k[j + (size_t)Ns * c].y} * w[j];
        for (int ty = 0; ty < kw; ++ty)
          for (int tx = 0; tx < kw; ++tx) {
            const double wt = wx[(size_t)j * kw + tx] * wy[(size_t)j * kw + ty];
            grid[wrap(gx0[j] + tx) + (size_t)G * (wrap(gy0[j] + ty) + (size_t)G * c)] += s * wt;
          }
      }
    fft2_unscaled(grid.data(), C, +1);
    const double sc = 1.0 / N;
    for (int y = 0; y < N; ++y)
      for (int x = 0; x < N; ++x) {
        const size_t i = x + (size_t)N * y;
        const double f = sc / (deap[x] * deap[y]);
        cd acc = {0, 0};
        for (int c = 0; c < C; ++c) {
          const cd g = grid[wrap(x - N / 2) + (size_t)G * (wrap(y - N / 2) + (size_t)G * c)] * f;
          acc += sens ? cmulc(g, cd{(double)sens[i + (size_t)N * N * c].x, (double)sens[i + (size_t)N * N * c].y}) : g;
        }
        u[i] = {(R)acc.x, (R)acc.y};
      }
  }
  // exact non-uniform DFT of the same operator (accuracy oracle)
  void ndft_forward(const cx<R>* u, cx<R>* k) const {
#pragma omp parallel for schedule(static)
    for (int j = 0; j < Ns; ++j)
      for (int c = 0; c < C; ++c) {
        double ar = 0, ai = 0;
        for (int y = 0; y < N; ++y)
          for (int x = 0; x < N; ++x) {
            const size_t i = x + (size_t)N * y;
            cd v = {(double)u[i].x, (double)u[i].y};
            if (sens) v = cmul(v, cd{(double)sens[i + (size_t)N * N * c].x, (double)sens[i + (size_t)N * N * c].y});
            const double ph = -2.0 * M_PI * (k0[j] * (x - N / 2) + k1[j] * (y - N / 2));
            ar += v.x * std::cos(ph) - v.y * std::sin(ph);
            ai += v.x * std::sin(ph) + v.y * std::cos(ph);
          }
        k[j + (size_t)Ns * c] = {(R)(ar * w[j] / N), (R)(ai * w[j] / N)};
      }
  }

 private:
  void fft2_unscaled(cd* d, int nb, int sign) const {
#pragma omp parallel for schedule(static)
    for (long long t = 0; t < (long long)nb * G; ++t) fft1(d + (size_t)t * G, 1, G, sign);
#pragma omp parallel for schedule(static)
    for (long long t = 0; t < (long long)nb * G; ++t) {
      const long long b = t / G, x = t % G;
      fft1(d + (size_t)b * G * G + x, (size_t)G, G, sign);
    }
  }
};

// ------------------------------------------------------------------------------------------------
// Solvers.
// ------------------------------------------------------------------------------------------------
template <class P>
struct ImgState {
  int W, H;
  std::vector<P> u, ubar, vx, vy, vbx, vby, px, py, qxx, qyy, qxy;
  ImgState(int W_, int H_) : W(W_), H(H_) {
    const size_t n = (size_t)W * H;
    for (auto* v : {&u, &ubar, &vx, &vy, &vbx, &vby, &px, &py, &qxx, &qyy, &qxy}) v->assign(n, pzero<P>());
  }
};

// TvOptimizer::solve (tvoptimizer.cu:76-125): u0 = f, p = 0, tau = sigma = 1/sqrt(8), k = 0..max_iter.
template <class P, class R>
void tv_solve(int W, int H, const P* f, const P* u0, P* uout, R lambda, unsigned max_iter) {
  ImgState<P> s(W, H);
  const size_t n = (size_t)W * H;
  const P* init = u0 ? u0 : f;
  std::copy(init, init + n, s.u.begin());
  std::copy(init, init + n, s.ubar.begin());
  const R tau = (R)(1.0 / std::sqrt(8.0)), sigma = (R)(1.0 / std::sqrt(8.0));
  for (unsigned k = 0; k <= max_iter; ++k) {
    tv_dual_p(s.px.data(), s.py.data(), s.ubar.data(), W, H, sigma, R(1));
    tv_primal_u(s.u.data(), s.ubar.data(), f, s.px.data(), s.py.data(), W, H, tau, lambda);
  }
  std::copy(s.u.begin(), s.u.end(), uout);
}

// TgvOptimizer::solve (tgvoptimizer.cu:80-141): primal first; tau = sigma = 1/sqrt(12).
template <class P, class R>
void tgv_solve(int W, int H, const P* f, const P* u0, P* uout, R lambda, R alpha0, R alpha1, unsigned max_iter) {
  ImgState<P> s(W, H);
  const size_t n = (size_t)W * H;
  const P* init = u0 ? u0 : f;
  std::copy(init, init + n, s.u.begin());
  std::copy(init, init + n, s.ubar.begin());
  const R tau = (R)(1.0 / std::sqrt(12.0)), sigma = (R)(1.0 / std::sqrt(12.0));
  for (unsigned k = 0; k <= max_iter; ++k) {
    tv_primal_u(s.u.data(), s.ubar.data(), f, s.px.data(), s.py.data(), W, H, tau, lambda);
    tgv_primal_v(s.vx.data(), s.vy.data(), s.vbx.data(), s.vby.data(), s.px.data(), s.py.data(), s.qxx.data(),
                 s.qyy.data(), s.qxy.data(), W, H, tau);
    tgv_dual_p(s.px.data(), s.py.data(), s.ubar.data(), s.vbx.data(), s.vby.data(), W, H, sigma, alpha1);
    tgv_dual_q(s.qxx.data(), s.qyy.data(), s.qxy.data(), s.vbx.data(), s.vby.data(), W, H, sigma, alpha0);
  }
  std::copy(s.u.begin(), s.u.end(), uout);
}

// The geometric alpha continuation of TgvMriOptimizer::solve (tgvmrioptimizer.cu:122-155), evaluated
// in real_type. max_iter = 0 would divide 0/0 in the reference; it is taken as its k/K -> 0 limit.
template <class R>
inline void alpha_schedule(R a0, R a1, R reduction, unsigned max_iter, unsigned k, R& o0, R& o1) {
  const R a00 = a0, a10 = a1, a01 = a0 * reduction, a11 = a1 * reduction;
  if (max_iter == 0) { o0 = a00; o1 = a10; return; }
  const R dmax = (R)max_iter, dk = (R)k;
  o0 = std::exp(dk / dmax * std::log(a01) + (dmax - dk) / dmax * std::log(a00));
  o1 = std::exp(dk / dmax * std::log(a11) + (dmax - dk) / dmax * std::log(a10));
}

// variant: 0 = TgvMriOptimizer (tgvmrioptimizer.cu:93-203), 1 = TgvOptimizerWithOp
// (tgvoptimizerwithop.cu:89-179), 2 = TvOptimizerWithOp (tvoptimizerwithop.cu:86-164).
template <class R, class Op>
void op_solve(const Op& op, const cx<R>* f, const cx<R>* u0, cx<R>* uout, int variant, R alpha0, R alpha1,
              R reduction, R lambda, unsigned max_iter, cx<R>* state_out, const cx<R>* state_in = nullptr) {
  typedef cx<R> P;
  const int W = op.img_w(), H = op.img_h();
  ImgState<P> s(W, H);
  const size_t nk = op.ksp_n(), ni = op.img_n();
  std::vector<P> r(nk, pzero<P>()), tmp(nk);
  if (state_in) {  // a later solve() continues from every primal and dual variable (tgvmrioptimizer.cu:62-91)
    const P* o = state_in;
    for (auto* v : {&s.u, &s.ubar, &s.vx, &s.vy, &s.vbx, &s.vby, &s.px, &s.py, &s.qxx, &s.qyy, &s.qxy}) {
      std::copy(o, o + ni, v->begin());
      o += ni;
    }
    std::copy(o, o + nk, r.begin());
  } else {
    if (u0) {
      std::copy(u0, u0 + ni, s.u.begin());
    } else {
      op.adjoint(f, s.u.data());  // "Initialization with A^T(f)"
    }
    std::copy(s.u.begin(), s.u.end(), s.ubar.begin());
  }
  const R tau = (variant == 0) ? (R)(1.0 / 16.0) : (R)(1.0 / 8.0);
  const R sigma = (R)(1.0 / 8.0);
  const R lam = (variant == 0) ? R(1) : lambda;
  for (unsigned k = 0; k <= max_iter; ++k) {
    R a0 = alpha0, a1 = alpha1;
    if (variant == 0) alpha_schedule(alpha0, alpha1, reduction, max_iter, k, a0, a1);
    op.forward(s.ubar.data(), tmp.data());
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < (long long)nk; ++i) tmp[i] = tmp[i] - f[i];  // addWeighted(tmp, 1, f, -1)
    prox_r(r.data(), tmp.data(), nk, sigma, lam);
    if (variant == 2) {
      tv_dual_p(s.px.data(), s.py.data(), s.ubar.data(), W, H, sigma, R(1));
    } else {
      tgv_dual_p(s.px.data(), s.py.data(), s.ubar.data(), s.vbx.data(), s.vby.data(), W, H, sigma, a1);
      tgv_dual_q(s.qxx.data(), s.qyy.data(), s.qxy.data(), s.vbx.data(), s.vby.data(), W, H, sigma, a0);
    }
    op.adjoint(r.data(), s.ubar.data());
    tgv_primal_u_noprox(s.u.data(), s.ubar.data(), s.px.data(), s.py.data(), W, H, tau);
    if (variant != 2)
      tgv_primal_v(s.vx.data(), s.vy.data(), s.vbx.data(), s.vby.data(), s.px.data(), s.py.data(), s.qxx.data(),
                   s.qyy.data(), s.qxy.data(), W, H, tau);
  }
  std::copy(s.u.begin(), s.u.end(), uout);
  if (state_out) {  // u, ubar, vx, vy, vbx, vby, px, py, qxx, qyy, qxy, then r
    P* o = state_out;
    for (auto* v : {&s.u, &s.ubar, &s.vx, &s.vy, &s.vbx, &s.vby, &s.px, &s.py, &s.qxx, &s.qyy, &s.qxy}) {
      std::copy(v->begin(), v->end(), o);
      o += ni;
    }
    std::copy(r.begin(), r.end(), o);
  }
}

// FP64 TGV-MRI energy at fixed alpha (used for the converged-solution stopping rule and the learned
// warm-start fallback): E(u, v) = 1/2 ||K u - f||^2 + alpha1 ||grad u - v||_{2,1} + alpha0 ||eps(v)||_{F,1}.
template <class R>
double tgv_energy(const CartOp<R>& op, const cx<R>* f, const cx<R>* u, const cx<R>* vx, const cx<R>* vy, R alpha0,
                  R alpha1) {
  typedef cx<R> P;
  const int W = op.W, H = op.Hi;
  std::vector<P> k(op.ksp_n());
  op.forward(u, k.data());
  double data = 0;
  for (size_t i = 0; i < k.size(); ++i) {
    const double dx = (double)k[i].x - f[i].x, dy = (double)k[i].y - f[i].y;
    data += dx * dx + dy * dy;
  }
  double t1 = 0, t0 = 0;
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      const size_t i = x + (size_t)W * y;
      P gx, gy, gxx, gyy, gxy;
      dp(u, W, H, x, y, gx, gy);
      dp_sym(vx, vy, W, H, x, y, gxx, gyy, gxy);
      const P a = gx - vx[i], b = gy - vy[i];
      t1 += std::sqrt((double)a.x * a.x + (double)a.y * a.y + (double)b.x * b.x + (double)b.y * b.y);
      t0 += std::sqrt((double)gxx.x * gxx.x + (double)gxx.y * gxx.y + (double)gyy.x * gyy.x + (double)gyy.y * gyy.y +
                      2.0 * ((double)gxy.x * gxy.x + (double)gxy.y * gxy.y));
    }
  return 0.5 * data + (double)alpha1 * t1 + (double)alpha0 * t0;
}


// ------------------------------------------------------------------------------------------------
// The learned warm-start network (the engine's pdt_cnn.cu), restated for gradient checks: FP64
// arithmetic with BF16 round-to-nearest-even applied exactly where the GPU stores BF16 (weights of the
// 32-channel convolutions, activations, pre-activations, output and hidden gradients).
// Parameter layout (flat): per layer weights [9][COUT][CIN] then bias [COUT]; layers conv_in (2 -> 32),
// six hidden (32 -> 32), conv_out (32 -> 8, channels 6 and 7 unused).
// ------------------------------------------------------------------------------------------------
static bool g_cnn_round = true;  // BF16 rounding emulation (off: exact FP64, for finite-difference checks)
inline float bf16r(float f) {
  if (!g_cnn_round) return f;
  uint32_t u;
  std::memcpy(&u, &f, 4);
  if ((u & 0x7f800000u) == 0x7f800000u) return f;
  u += 0x7fffu + ((u >> 16) & 1u);
  u &= 0xffff0000u;
  std::memcpy(&f, &u, 4);
  return f;
}

struct CnnOracle {
  int B, H, W;
  size_t np;
  static const int L = 8;
  int cin[L], cout[L];
  std::vector<double> w[L], b[L];  // FP32 master values (as double)
  std::vector<double> gw[L], gb[L];
  CnnOracle(int B_, int H_, int W_, const float* params) : B(B_), H(H_), W(W_), np((size_t)B_ * H_ * W_) {
    size_t o = 0;
    for (int l = 0; l < L; ++l) {
      cin[l] = l == 0 ? 2 : 32;
      cout[l] = l == 7 ? 8 : 32;
      const size_t nw = (size_t)9 * cout[l] * cin[l];
      w[l].assign(params + o, params + o + nw);
      o += nw;
      b[l].assign(params + o, params + o + cout[l]);
      o += cout[l];
      if (l >= 1)
        for (auto& v : w[l]) v = bf16r((float)v);  // tensor-core layers use BF16 weights
    }
  }
  // y[p][co] = sum_{tap, ci} x[p + d(tap)][ci] w[tap][co][ci] + bias (zero padding)
  void conv(const std::vector<double>& x, int ci_n, const std::vector<double>& wt, const double* bias, int co_n,
            std::vector<double>& y) const {
    y.assign(np * co_n, 0.0);
#pragma omp parallel for schedule(static)
    for (long long p = 0; p < (long long)np; ++p) {
      const int xx = (int)(p % W), yy = (int)((p / W) % H), bb = (int)(p / ((size_t)W * H));
      for (int co = 0; co < co_n; ++co) {
        double s = bias ? bias[co] : 0.0;
        for (int tap = 0; tap < 9; ++tap) {
          const int gy = yy + tap / 3 - 1, gx = xx + tap % 3 - 1;
          if (gy < 0 || gy >= H || gx < 0 || gx >= W) continue;
          const size_t q = ((size_t)bb * H + gy) * W + gx;
          for (int ci = 0; ci < ci_n; ++ci) s += x[q * ci_n + ci] * wt[((size_t)tap * co_n + co) * ci_n + ci];
        }
        y[p * co_n + co] = s;
      }
    }
  }
  // transposed convolution (data gradient): dx[q][ci] = sum_{tap, co} dy[q - d(tap)][co] w[tap][co][ci]
  void conv_t(const std::vector<double>& dy, int co_n, const std::vector<double>& wt, int ci_n,
              std::vector<double>& dx) const {
    dx.assign(np * ci_n, 0.0);
#pragma omp parallel for schedule(static)
    for (long long q = 0; q < (long long)np; ++q) {
      const int xx = (int)(q % W), yy = (int)((q / W) % H), bb = (int)(q / ((size_t)W * H));
      for (int ci = 0; ci < ci_n; ++ci) {
        double s = 0;
        for (int tap = 0; tap < 9; ++tap) {
          const int py = yy - (tap / 3 - 1), px = xx - (tap % 3 - 1);
          if (py < 0 || py >= H || px < 0 || px >= W) continue;
          const size_t p = ((size_t)bb * H + py) * W + px;
          for (int co = 0; co < co_n; ++co) s += dy[p * co_n + co] * wt[((size_t)tap * co_n + co) * ci_n + ci];
        }
        dx[q * ci_n + ci] = s;
      }
    }
  }
  void wgrad(const std::vector<double>& x, int ci_n, const std::vector<double>& dy, int co_n, std::vector<double>& gw_,
             std::vector<double>& gb_) const {
    gw_.assign((size_t)9 * co_n * ci_n, 0.0);
    gb_.assign(co_n, 0.0);
#pragma omp parallel for schedule(static)
    for (int idx = 0; idx < 9 * co_n; ++idx) {
      const int tap = idx / co_n, co = idx % co_n;
      for (int ci = 0; ci < ci_n; ++ci) {
        double s = 0;
        for (size_t p = 0; p < np; ++p) {
          const int xx = (int)(p % W), yy = (int)((p / W) % H), bb = (int)(p / ((size_t)W * H));
          const int gy = yy + tap / 3 - 1, gx = xx + tap % 3 - 1;
          if (gy < 0 || gy >= H || gx < 0 || gx >= W) continue;
          s += x[(((size_t)bb * H + gy) * W + gx) * ci_n + ci] * dy[p * co_n + co];
        }
        gw_[((size_t)tap * co_n + co) * ci_n + ci] = s;
      }
    }
    for (int co = 0; co < co_n; ++co) {
      double s = 0;
      for (size_t p = 0; p < np; ++p) s += dy[p * co_n + co];
      gb_[co] = s;
    }
  }
  static void round_bf16(std::vector<double>& v) {
    if (!g_cnn_round) return;
    for (auto& x : v) x = bf16r((float)x);
  }
  // loss and gradients; u0, ut complex [B][H][W]; vt [B][2][H][W]
  double run(const float* u0, const float* ut, const float* vt, double* out6 /* nullable: [np][8] */) {
    std::vector<double> s(B);
    for (int bb = 0; bb < B; ++bb) {
      float m = 0.f;
      for (size_t i = 0; i < (size_t)H * W; ++i) {
        const size_t k = (size_t)bb * H * W + i;
        m = std::max(m, std::sqrt(u0[2 * k] * u0[2 * k] + u0[2 * k + 1] * u0[2 * k + 1]));
      }
      s[bb] = m > 0.f ? m : 1.f;
    }
    std::vector<double> x(np * 2), t(np * 6);
    const size_t hw = (size_t)H * W;
    for (size_t p = 0; p < np; ++p) {
      const size_t bb = p / hw, i = p % hw;
      const float inv = 1.f / (float)s[bb];
      x[2 * p] = u0[2 * p] * inv;
      x[2 * p + 1] = u0[2 * p + 1] * inv;
      t[6 * p + 0] = (ut[2 * p] - u0[2 * p]) * inv;
      t[6 * p + 1] = (ut[2 * p + 1] - u0[2 * p + 1]) * inv;
      for (int c = 0; c < 2; ++c) {
        const size_t vi = ((2 * bb + c) * hw + i) * 2;
        t[6 * p + 2 + 2 * c] = vt[vi] * inv;
        t[6 * p + 3 + 2 * c] = vt[vi + 1] * inv;
      }
    }
    // forward
    std::vector<double> z[7], h[7], o;
    conv(x, 2, w[0], b[0].data(), 32, z[0]);
    h[0] = z[0];
    for (auto& v : h[0]) v = bf16r((float)std::max(v, 0.0));
    round_bf16(z[0]);
    for (int l = 1; l <= 6; ++l) {
      conv(h[l - 1], 32, w[l], b[l].data(), 32, z[l]);
      h[l].resize(np * 32);
      for (size_t i = 0; i < np * 32; ++i) h[l][i] = bf16r((float)(h[l - 1][i] + std::max(z[l][i], 0.0)));
      round_bf16(z[l]);
    }
    conv(h[6], 32, w[7], b[7].data(), 8, o);
    if (g_cnn_round)
      for (auto& v : o) v = (float)v;
    if (out6) std::copy(o.begin(), o.end(), out6);
    // loss
    double loss = 0;
    std::vector<double> go(np * 8, 0.0);
    for (size_t p = 0; p < np; ++p)
      for (int c = 0; c < 6; ++c) {
        const double d = o[p * 8 + c] - t[p * 6 + c];
        loss += d * d;
        go[p * 8 + c] = bf16r((float)(2.0 * d / (double)np));
      }
    // backward
    wgrad(h[6], 32, go, 8, gw[7], gb[7]);
    std::vector<double> g, tmp;
    conv_t(go, 8, w[7], 32, tmp);
    round_bf16(tmp);
    g = tmp;
    for (int l = 6; l >= 1; --l) {
      std::vector<double> gz(np * 32);
      for (size_t i = 0; i < np * 32; ++i) {
        const double gi = bf16r((float)g[i]);
        gz[i] = z[l][i] > 0 ? gi : 0.0;
      }
      wgrad(h[l - 1], 32, gz, 32, gw[l], gb[l]);
      conv_t(gz, 32, w[l], 32, tmp);
      round_bf16(tmp);
      for (size_t i = 0; i < np * 32; ++i) g[i] += tmp[i];
    }
    std::vector<double> gz(np * 32);
    for (size_t i = 0; i < np * 32; ++i) gz[i] = z[0][i] > 0 ? bf16r((float)g[i]) : 0.0;
    wgrad(x, 2, gz, 32, gw[0], gb[0]);
    return loss / (double)np;
  }
};

}  // namespace

// ==================================================================================================
// C entry points (ctypes). Complex arrays are interleaved real pairs; `prec` 32 or 64 selects the
// FP32-mirror or FP64 path; pointers for prec 32 are float*, for 64 double*.
// ==================================================================================================
extern "C" {

int orc_version(void) { return 1; }

void orc_set_threads(int n) {
#ifdef _OPENMP
  omp_set_num_threads(n > 0 ? n : 1);
#else
  (void)n;
#endif
}

int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

// 1-D complex FFT (double, unscaled), sign -1 forward / +1 inverse. Test hook for the FFT restatement.
void orc_fft1d(double* data, int n, int sign) { fft1(reinterpret_cast<cd*>(data), 1, n, sign); }

#define ORC_DISPATCH_REAL(prec, F32CALL, F64CALL) \
  do {                                           \
    if ((prec) == 32) { F32CALL; }               \
    else { F64CALL; }                            \
  } while (0)

// TvOptimizer / TgvOptimizer denoising. is_complex selects the *_2c (complex) or *_2f (real) variant.
void orc_tv_solve(int prec, int is_complex, int W, int H, const void* f, const void* u0, void* uout, double lambda,
                  unsigned max_iter) {
  if (prec == 32) {
    if (is_complex)
      tv_solve<cx<float>, float>(W, H, (const cx<float>*)f, (const cx<float>*)u0, (cx<float>*)uout, (float)lambda, max_iter);
    else
      tv_solve<float, float>(W, H, (const float*)f, (const float*)u0, (float*)uout, (float)lambda, max_iter);
  } else {
    if (is_complex)
      tv_solve<cx<double>, double>(W, H, (const cx<double>*)f, (const cx<double>*)u0, (cx<double>*)uout, lambda, max_iter);
    else
      tv_solve<double, double>(W, H, (const double*)f, (const double*)u0, (double*)uout, lambda, max_iter);
  }
}

void orc_tgv_solve(int prec, int is_complex, int W, int H, const void* f, const void* u0, void* uout, double lambda,
                   double alpha0, double alpha1, unsigned max_iter) {
  if (prec == 32) {
    if (is_complex)
      tgv_solve<cx<float>, float>(W, H, (const cx<float>*)f, (const cx<float>*)u0, (cx<float>*)uout, (float)lambda,
                                  (float)alpha0, (float)alpha1, max_iter);
    else
      tgv_solve<float, float>(W, H, (const float*)f, (const float*)u0, (float*)uout, (float)lambda, (float)alpha0,
                              (float)alpha1, max_iter);
  } else {
    if (is_complex)
      tgv_solve<cx<double>, double>(W, H, (const cx<double>*)f, (const cx<double>*)u0, (cx<double>*)uout, lambda,
                                    alpha0, alpha1, max_iter);
    else
      tgv_solve<double, double>(W, H, (const double*)f, (const double*)u0, (double*)uout, lambda, alpha0, alpha1,
                                max_iter);
  }
}

// Operator application. kind 0/1/2 as above; sens may be null for kind 2. C is ignored for kind 2.
void orc_op_apply(int prec, int kind, int adjoint, int W, int Hf, int C, const void* sens, const void* mask,
                  const void* src, void* dst) {
  if (prec == 32) {
    CartOp<float> op(kind, W, Hf, C, (const cx<float>*)sens, (const float*)mask);
    if (adjoint) op.adjoint((const cx<float>*)src, (cx<float>*)dst);
    else op.forward((const cx<float>*)src, (cx<float>*)dst);
  } else {
    CartOp<double> op(kind, W, Hf, C, (const cx<double>*)sens, (const double*)mask);
    if (adjoint) op.adjoint((const cx<double>*)src, (cx<double>*)dst);
    else op.forward((const cx<double>*)src, (cx<double>*)dst);
  }
}

// TgvMriOptimizer / TgvOptimizerWithOp / TvOptimizerWithOp with a Cartesian-family operator.
void orc_op_solve(int prec, int kind, int W, int Hf, int C, const void* sens, const void* mask, const void* f,
                  const void* u0, void* uout, int variant, double alpha0, double alpha1, double reduction,
                  double lambda, unsigned max_iter, void* state_out, const void* state_in) {
  if (prec == 32) {
    CartOp<float> op(kind, W, Hf, C, (const cx<float>*)sens, (const float*)mask);
    op_solve<float, CartOp<float>>(op, (const cx<float>*)f, (const cx<float>*)u0, (cx<float>*)uout, variant, (float)alpha0,
                    (float)alpha1, (float)reduction, (float)lambda, max_iter, (cx<float>*)state_out,
                    (const cx<float>*)state_in);
  } else {
    CartOp<double> op(kind, W, Hf, C, (const cx<double>*)sens, (const double*)mask);
    op_solve<double, CartOp<double>>(op, (const cx<double>*)f, (const cx<double>*)u0, (cx<double>*)uout, variant, alpha0, alpha1,
                     reduction, lambda, max_iter, (cx<double>*)state_out, (const cx<double>*)state_in);
  }
}

// Alpha schedule of TgvMriOptimizer in float (the value the GPU engine must reproduce).
void orc_alpha_schedule_f32(float a0, float a1, float reduction, unsigned max_iter, unsigned k, float* o0, float* o1) {
  alpha_schedule<float>(a0, a1, reduction, max_iter, k, *o0, *o1);
}

double orc_tgv_energy_f64(int kind, int W, int Hf, int C, const double* sens, const double* mask, const double* f,
                          const double* u, const double* vx, const double* vy, double alpha0, double alpha1) {
  CartOp<double> op(kind, W, Hf, C, (const cx<double>*)sens, mask);
  return tgv_energy<double>(op, (const cx<double>*)f, (const cx<double>*)u, (const cx<double>*)vx,
                            (const cx<double>*)vy, alpha0, alpha1);
}

// Primal-dual gap of the with-operator saddle problems from a full state, in FP64 (the engine's
// pdt_opt_gap). state = {u, ubar, vx, vy, vbx, vby, px, py, qxx, qyy, qxy} (image planes) then r (k-space),
// as op_solve returns it. The r-prox (r + sigma (K u - f)) / (1 + sigma lambda) (tgv_kernels.cuh:213-223)
// is the resolvent of F*(r) = <f, r> + lambda/2 |r|^2, so F(z) = |z - f|^2 / (2 lambda) and the dual value
// is -F*(r) when K^H r = div- p and p = -div_h- q. Phase-encode columns without a sampled entry contribute
// |f|^2 / (2 lambda) to both sides (r -> -f / lambda there) and are taken at that limit.
// out = {gap, primal, dual, |div- p - K^H r|, |p + div_h- q|, |K^H r|}; variant as op_solve (2 = TV).
void orc_op_gap(int kind, int W, int Hf, int C, const double* sens, const double* mask, const double* f,
                const double* state, int variant, double alpha0, double alpha1, double lambda, double* out) {
  typedef cx<double> P;
  CartOp<double> op(kind, W, Hf, C, (const P*)sens, mask);
  const size_t ni = op.img_n(), nk = op.ksp_n();
  const int H = op.img_h();
  const double lam = variant == 0 ? 1.0 : lambda;
  const P* st = (const P*)state;
  const P *u = st, *vx = st + 2 * ni, *vy = st + 3 * ni, *px = st + 6 * ni, *py = st + 7 * ni;
  const P *qxx = st + 8 * ni, *qyy = st + 9 * ni, *qxy = st + 10 * ni, *r = st + 11 * ni;
  const P* F = (const P*)f;
  std::vector<P> k(nk), khr(ni);
  op.forward(u, k.data());
  double data = 0;
  for (size_t i = 0; i < nk; ++i) {
    const double dx = k[i].x - F[i].x, dy = k[i].y - F[i].y;
    data += dx * dx + dy * dy;
  }
  data *= 0.5 / lam;
  double t1 = 0, t0 = 0, ru = 0, rv = 0;
  op.adjoint(r, khr.data());
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      const size_t i = x + (size_t)W * y;
      P gx, gy;
      dp(u, W, H, x, y, gx, gy);
      if (variant != 2) {
        P gxx, gyy, gxy, dx, dy;
        dp_sym(vx, vy, W, H, x, y, gxx, gyy, gxy);
        gx = gx - vx[i];
        gy = gy - vy[i];
        t0 += std::sqrt(gxx.x * gxx.x + gxx.y * gxx.y + gyy.x * gyy.x + gyy.y * gyy.y +
                        2.0 * (gxy.x * gxy.x + gxy.y * gxy.y));
        dm_sym(qxx, qyy, qxy, W, H, x, y, dx, dy);
        const P a = px[i] + dx, b = py[i] + dy;
        rv += a.x * a.x + a.y * a.y + b.x * b.x + b.y * b.y;
      }
      t1 += std::sqrt(gx.x * gx.x + gx.y * gx.y + gy.x * gy.x + gy.y * gy.y);
      const P d = dm(px, py, W, H, x, y) - khr[i];
      ru += d.x * d.x + d.y * d.y;
    }
  const double primal = data + (variant == 2 ? t1 : alpha1 * t1 + alpha0 * t0);
  std::vector<char> sampled(W, 0);
  for (int y = 0; y < Hf; ++y)
    for (int x = 0; x < W; ++x)
      if (mask[(size_t)y * W + x] != 0.0) sampled[x] = 1;
  double fr = 0, rr = 0, fu = 0;
  for (size_t i = 0; i < nk; ++i) {
    if (sampled[i % W]) {
      fr += F[i].x * r[i].x + F[i].y * r[i].y;
      rr += r[i].x * r[i].x + r[i].y * r[i].y;
    } else {
      fu += F[i].x * F[i].x + F[i].y * F[i].y;
    }
  }
  double nkhr = 0;
  for (size_t i = 0; i < ni; ++i) nkhr += khr[i].x * khr[i].x + khr[i].y * khr[i].y;
  const double dual = -fr - 0.5 * lam * rr + 0.5 * fu / lam;
  out[0] = primal - dual;
  out[1] = primal;
  out[2] = dual;
  out[3] = std::sqrt(ru);
  out[4] = std::sqrt(rv);
  out[5] = std::sqrt(nkhr);
}

// Radial operators. mode: 0 forward (NUFFT), 1 adjoint, 2 exact NDFT forward. sens may be null (single coil).
// traj {Ns, 2} planar, dcf {Ns}. Pointers are float (prec 32) or double (prec 64).
void orc_radial_apply(int prec, int mode, int N, double osf, int kw, int C, int Ns, const void* traj, const void* dcf,
                      const void* sens, const void* src, void* dst) {
  if (prec == 32) {
    RadialOp<float> op(N, osf, kw, C, Ns, (const float*)traj, (const float*)dcf, (const cx<float>*)sens);
    if (mode == 0) op.forward((const cx<float>*)src, (cx<float>*)dst);
    else if (mode == 1) op.adjoint((const cx<float>*)src, (cx<float>*)dst);
    else op.ndft_forward((const cx<float>*)src, (cx<float>*)dst);
  } else {
    RadialOp<double> op(N, osf, kw, C, Ns, (const double*)traj, (const double*)dcf, (const cx<double>*)sens);
    if (mode == 0) op.forward((const cx<double>*)src, (cx<double>*)dst);
    else if (mode == 1) op.adjoint((const cx<double>*)src, (cx<double>*)dst);
    else op.ndft_forward((const cx<double>*)src, (cx<double>*)dst);
  }
}

void orc_radial_solve(int prec, int N, double osf, int kw, int C, int Ns, const void* traj, const void* dcf,
                      const void* sens, const void* f, const void* u0, void* uout, int variant, double alpha0,
                      double alpha1, double reduction, double lambda, unsigned max_iter) {
  if (prec == 32) {
    RadialOp<float> op(N, osf, kw, C, Ns, (const float*)traj, (const float*)dcf, (const cx<float>*)sens);
    op_solve<float, RadialOp<float>>(op, (const cx<float>*)f, (const cx<float>*)u0, (cx<float>*)uout, variant,
                                     (float)alpha0, (float)alpha1, (float)reduction, (float)lambda, max_iter, nullptr);
  } else {
    RadialOp<double> op(N, osf, kw, C, Ns, (const double*)traj, (const double*)dcf, (const cx<double>*)sens);
    op_solve<double, RadialOp<double>>(op, (const cx<double>*)f, (const cx<double>*)u0, (cx<double>*)uout, variant,
                                       alpha0, alpha1, reduction, lambda, max_iter, nullptr);
  }
}

// Kaiser-Bessel helpers exposed for tests: grid size, beta, deapodisation.
int orc_radial_grid_size(int N, double osf) { return radial_grid_size(N, osf); }
double orc_kb_beta(int kw, double osf) { return kb_beta(kw, osf); }
double orc_kb_deapod(int m, int G, int kw, double beta) { return kb_deapod(m, G, kw, beta); }

// The same network without any BF16 rounding (every value FP64 except the FP32 inputs and parameters).
double orc_cnn_grad_exact(int B, int H, int W, const float* params, const float* u0, const float* ut,
                          const float* vt, double* grads) {
  g_cnn_round = false;
  CnnOracle net(B, H, W, params);
  const double loss = net.run(u0, ut, vt, nullptr);
  g_cnn_round = true;
  size_t o = 0;
  for (int l = 0; l < CnnOracle::L; ++l) {
    for (double v : net.gw[l]) grads[o++] = v;
    for (double v : net.gb[l]) grads[o++] = v;
  }
  return loss;
}

// Loss and gradients of the warm-start network (flat layout as pdt_cnn_get_grads); returns the loss.
double orc_cnn_grad(int B, int H, int W, const float* params, const float* u0, const float* ut, const float* vt,
                    double* grads, double* out8) {
  g_cnn_round = true;
  CnnOracle net(B, H, W, params);
  const double loss = net.run(u0, ut, vt, out8);
  size_t o = 0;
  for (int l = 0; l < CnnOracle::L; ++l) {
    for (double v : net.gw[l]) grads[o++] = v;
    for (double v : net.gb[l]) grads[o++] = v;
  }
  return loss;
}

}  // extern "C"
