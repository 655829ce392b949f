// pdt_iu_shim.h -- a host-only stand-in for the parts of ImageUtilities (github.com/VLOGroup/imageutilities,
// an empty submodule in the reference checkout, pin unknown) that the reference's optimizer and Cartesian
// operator sources use, so that those sources compile with g++ and run on the CPU.
//
// TEST INFRASTRUCTURE ONLY: used by oracle/ref_build.py to build oracle/_ref/libpdtref.so, which tests
// use to pin the oracle restatement (oracle/pdt_oracle.cpp) and to write golden vectors. Nothing of the
// product includes it.
//
// What it provides, restated from ImageUtilities' documented behaviour and its call sites in the
// reference (mricartesianoperator.cu:196-414, tgvmrioptimizer.cu, tvoptimizer.cu, tgvoptimizer.cu,
// t*optimizerwithop.cu, optimizer_helper.h, operatorbase.h):
//   * CUDA's launch vocabulary for sequential host execution: a kernel is an ordinary function and
//     pdtref::launch runs it once per (block, thread), setting the thread-local blockIdx / threadIdx.
//     The reference's kernels on this path use no shared memory and no __syncthreads, and none reads a
//     value that another thread of the same launch writes, so any execution order gives the GPU's result.
//   * float2 / double2 arithmetic (element-wise, scalar multiples) and complex_multiply(_conjugate);
//   * iu::Size, iu::LinearHostMemory, iu::LinearDeviceMemory (host memory here) and its KernelData
//     accessors (x fastest: idx = x + size[0] (y + size[1] z));
//   * iu::copy, iu::math::fill, iu::math::addWeighted, the dot products;
//   * iu::math::fft::fft2 / ifft2 (batched over the third dimension, exp(-+2 pi i jk/n), scaled by
//     1/sqrt(W H) when asked) computed in double precision and rounded to the pixel type, and fftshift2
//     (a shift by n/2 along both dimensions, numpy's fftshift);
//   * iu::type_trait, iu::divUp, iu::IuCudaTimer, IuException, IU_CUDA_CHECK, IU_SIZE_CHECK.
#pragma once

#include <chrono>
#include <cmath>
#include <complex>
#include <cstring>
#include <initializer_list>
#include <map>
#include <iostream>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

// ---- CUDA vocabulary ---------------------------------------------------------------------------------
#define __global__
#define __device__
#define __host__
#define __forceinline__ inline

struct uint3 {
  unsigned x, y, z;
};
struct dim3 {
  unsigned x, y, z;
  dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};
inline thread_local uint3 threadIdx, blockIdx;
inline thread_local dim3 blockDim, gridDim;

namespace pdtref {
// Runs `body` (a call of a kernel with its arguments) once for every thread of every block; blocks are
// spread over the host's OpenMP threads (the kernels' threads write disjoint elements and read nothing
// another thread of the launch writes, so the order is immaterial).
template <class F>
void launch(dim3 grid, dim3 block, F&& body) {
  const long long nblocks = (long long)grid.x * grid.y * grid.z;
#pragma omp parallel for schedule(static)
  for (long long b = 0; b < nblocks; ++b) {
    gridDim = grid;
    blockDim = block;
    blockIdx = {(unsigned)(b % grid.x), (unsigned)((b / grid.x) % grid.y), (unsigned)(b / ((long long)grid.x * grid.y))};
    for (unsigned tz = 0; tz < block.z; ++tz)
      for (unsigned ty = 0; ty < block.y; ++ty)
        for (unsigned tx = 0; tx < block.x; ++tx) {
          threadIdx = {tx, ty, tz};
          body();
        }
  }
}
}  // namespace pdtref

// ---- vector types ------------------------------------------------------------------------------------
struct float2 {
  float x, y;
};
struct double2 {
  double x, y;
};
inline float2 make_float2(float x, float y) { return {x, y}; }
inline double2 make_double2(double x, double y) { return {x, y}; }

#define PDTREF_VEC_OPS(V, S)                                                                     \
  inline V operator+(V a, V b) { return {a.x + b.x, a.y + b.y}; }                                \
  inline V operator-(V a, V b) { return {a.x - b.x, a.y - b.y}; }                                \
  inline V operator-(V a) { return {-a.x, -a.y}; }                                               \
  inline V operator*(V a, V b) { return {a.x * b.x, a.y * b.y}; }                                \
  inline V operator*(V a, S s) { return {a.x * s, a.y * s}; }                                    \
  inline V operator*(S s, V a) { return {s * a.x, s * a.y}; }                                    \
  inline V operator/(V a, S s) { return {a.x / s, a.y / s}; }                                    \
  inline V& operator+=(V& a, V b) { a.x += b.x; a.y += b.y; return a; }                          \
  inline V& operator-=(V& a, V b) { a.x -= b.x; a.y -= b.y; return a; }                          \
  inline V& operator*=(V& a, S s) { a.x *= s; a.y *= s; return a; }                              \
  inline V& operator/=(V& a, S s) { a.x /= s; a.y /= s; return a; }                              \
  inline bool operator==(V a, V b) { return a.x == b.x && a.y == b.y; }                          \
  inline std::ostream& operator<<(std::ostream& o, V a) { return o << "(" << a.x << "," << a.y << ")"; }
PDTREF_VEC_OPS(float2, float)
PDTREF_VEC_OPS(double2, double)
#undef PDTREF_VEC_OPS

template <class T>
inline T sqr(T x) {
  return x * x;
}

namespace iu {

// ---- type traits -------------------------------------------------------------------------------------
template <class T>
struct type_trait;
template <>
struct type_trait<float> {
  typedef float real_type;
  typedef float2 complex_type;
  static float make(float v) { return v; }
  static float2 make_complex(float v) { return {v, 0.f}; }
  static float2 make_complex(float re, float im) { return {re, im}; }
  static float abs(float v) { return std::fabs(v); }
  static float max(float a, float b) { return a > b ? a : b; }
  static const char* name() { return "float"; }
};
template <>
struct type_trait<double> {
  typedef double real_type;
  typedef double2 complex_type;
  static double make(double v) { return v; }
  static double2 make_complex(double v) { return {v, 0.0}; }
  static double2 make_complex(double re, double im) { return {re, im}; }
  static double abs(double v) { return std::fabs(v); }
  static double max(double a, double b) { return a > b ? a : b; }
  static const char* name() { return "double"; }
};
template <>
struct type_trait<float2> {
  typedef float real_type;
  typedef float2 complex_type;
  static float2 make(float v) { return {v, v}; }
  static float2 make_complex(float v) { return {v, 0.f}; }
  static float2 make_complex(float re, float im) { return {re, im}; }
  static float abs(float2 v) { return std::sqrt(v.x * v.x + v.y * v.y); }
  static float max(float a, float b) { return a > b ? a : b; }
  static const char* name() { return "float2"; }
};
template <>
struct type_trait<double2> {
  typedef double real_type;
  typedef double2 complex_type;
  static double2 make(double v) { return {v, v}; }
  static double2 make_complex(double v) { return {v, 0.0}; }
  static double2 make_complex(double re, double im) { return {re, im}; }
  static double abs(double2 v) { return std::sqrt(v.x * v.x + v.y * v.y); }
  static double max(double a, double b) { return a > b ? a : b; }
  static const char* name() { return "double2"; }
};

inline unsigned divUp(unsigned a, unsigned b) { return (a + b - 1) / b; }

// ---- sizes and memory --------------------------------------------------------------------------------
template <unsigned N>
struct Size {
  unsigned v[N];
  Size() {
    for (unsigned i = 0; i < N; ++i) v[i] = 0;
  }
  Size(std::initializer_list<unsigned> l) {
    unsigned i = 0;
    for (unsigned x : l)
      if (i < N) v[i++] = x;
    for (; i < N; ++i) v[i] = 1;
  }
  template <class... A, class = typename std::enable_if<sizeof...(A) == N && (N > 1)>::type>
  Size(A... a) : Size({static_cast<unsigned>(a)...}) {}
  unsigned& operator[](unsigned i) { return v[i]; }
  unsigned operator[](unsigned i) const { return v[i]; }
  size_t numel() const {
    size_t n = 1;
    for (unsigned i = 0; i < N; ++i) n *= v[i];
    return n;
  }
  bool operator==(const Size& o) const { return std::memcmp(v, o.v, sizeof v) == 0; }
  bool operator!=(const Size& o) const { return !(*this == o); }
  friend std::ostream& operator<<(std::ostream& os, const Size& s) {
    os << "(";
    for (unsigned i = 0; i < N; ++i) os << (i ? "," : "") << s.v[i];
    return os << ")";
  }
};

template <typename T, unsigned N>
class LinearMemoryBase {
 public:
  typedef T pixel_type;
  static const unsigned ndim = N;
  explicit LinearMemoryBase(const Size<N>& s) : size_(s), own_(s.numel()), data_(own_.data()) {}
  LinearMemoryBase(T* data, const Size<N>& s, bool ext_data = true) : size_(s), data_(data) {
    if (!ext_data) {
      own_.assign(data, data + s.numel());
      data_ = own_.data();
    }
  }
  T* data() { return data_; }
  const T* data() const { return data_; }
  Size<N> size() const { return size_; }
  size_t numel() const { return size_.numel(); }
  size_t bytes() const { return numel() * sizeof(T); }

  // Device-side accessor (by value in kernel launches): x fastest.
  struct KernelData {
    T* data_;
    unsigned size_[N];
    unsigned numel_;
    KernelData(const LinearMemoryBase& m) : data_(const_cast<T*>(m.data_)), numel_((unsigned)m.numel()) {
      for (unsigned i = 0; i < N; ++i) size_[i] = m.size_[i];
    }
    T& operator()(unsigned idx) { return data_[idx]; }
    T& operator()(unsigned x, unsigned y) { return data_[x + (size_t)size_[0] * y]; }
    T& operator()(unsigned x, unsigned y, unsigned z) {
      return data_[x + (size_t)size_[0] * (y + (size_t)size_[1] * z)];
    }
  };

 protected:
  Size<N> size_;
  std::vector<T> own_;
  T* data_;
};

template <typename T, unsigned N>
class LinearHostMemory : public LinearMemoryBase<T, N> {
 public:
  using LinearMemoryBase<T, N>::LinearMemoryBase;
};
template <typename T, unsigned N>
class LinearDeviceMemory : public LinearMemoryBase<T, N> {
 public:
  using LinearMemoryBase<T, N>::LinearMemoryBase;
};

template <typename T, unsigned N>
void copy(const LinearMemoryBase<T, N>* src, LinearMemoryBase<T, N>* dst) {
  if (src->size() != dst->size()) throw std::runtime_error("iu::copy: size mismatch");
  std::memcpy(dst->data(), src->data(), src->bytes());
}

class IuCudaTimer {
 public:
  void start() { t0_ = std::chrono::steady_clock::now(); }
  double elapsed() const {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0_).count();
  }

 private:
  std::chrono::steady_clock::time_point t0_;
};

// ---- math --------------------------------------------------------------------------------------------
namespace math {
template <typename T, unsigned N>
void fill(LinearMemoryBase<T, N>& m, T v) {
  for (size_t i = 0; i < m.numel(); ++i) m.data()[i] = v;
}
// dst = a * wa + b * wb, element-wise
template <typename T, unsigned N>
void addWeighted(const LinearMemoryBase<T, N>& a, T wa, const LinearMemoryBase<T, N>& b, T wb,
                 LinearMemoryBase<T, N>& dst) {
  for (size_t i = 0; i < dst.numel(); ++i) dst.data()[i] = a.data()[i] * wa + b.data()[i] * wb;
}
template <typename T, unsigned N>
void dotProduct(const LinearMemoryBase<T, N>& a, const LinearMemoryBase<T, N>& b, T& out) {
  double s = 0;
  for (size_t i = 0; i < a.numel(); ++i) s += (double)a.data()[i] * (double)b.data()[i];
  out = (T)s;
}
namespace complex {
// sum a * conj(b)
template <typename T, unsigned N>
void dotProduct(const LinearMemoryBase<T, N>& a, const LinearMemoryBase<T, N>& b, T& out) {
  double re = 0, im = 0;
  for (size_t i = 0; i < a.numel(); ++i) {
    const T p = a.data()[i], q = b.data()[i];
    re += (double)p.x * q.x + (double)p.y * q.y;
    im += (double)p.y * q.x - (double)p.x * q.y;
  }
  out.x = re;
  out.y = im;
}
}  // namespace complex

namespace fft {
namespace detail {
// exp(sign 2 pi i k / n) for k < n, computed once per (n, sign) and thread
inline const std::vector<std::complex<double>>& roots(int n, int sign) {
  thread_local std::map<long long, std::vector<std::complex<double>>> cache;  // references stay valid
  auto& w = cache[2LL * n + (sign > 0)];
  if (w.empty()) {
    const double tau = 6.283185307179586476925286766559;
    w.resize(n);
    for (int k = 0; k < n; ++k) w[k] = std::polar(1.0, sign * tau * k / n);
  }
  return w;
}
// In-place DFT of n values in double: radix-2 recursion, direct DFT for odd n.
inline void dft(std::complex<double>* a, int n, int sign, std::vector<std::complex<double>>& tmp) {
  if (n == 1) return;
  const std::vector<std::complex<double>>& w = roots(n, sign);
  if (n % 2 == 0) {
    const int h = n / 2;
    std::vector<std::complex<double>> e(h), o(h);
    for (int i = 0; i < h; ++i) {
      e[i] = a[2 * i];
      o[i] = a[2 * i + 1];
    }
    dft(e.data(), h, sign, tmp);
    dft(o.data(), h, sign, tmp);
    for (int k = 0; k < h; ++k) {
      const std::complex<double> t = w[k] * o[k];
      a[k] = e[k] + t;
      a[k + h] = e[k] - t;
    }
    return;
  }
  tmp.assign(a, a + n);
  for (int k = 0; k < n; ++k) {
    std::complex<double> s = 0;
    for (int j = 0; j < n; ++j) s += tmp[j] * w[(long long)j * k % n];
    a[k] = s;
  }
}
template <typename T, unsigned N>
void fft2_impl(const LinearMemoryBase<T, N>& src, LinearMemoryBase<T, N>& dst, bool scale, int sign) {
  const unsigned W = src.size()[0], H = src.size()[1];
  const long long S = (long long)(src.numel() / ((size_t)W * H));
  const double sc = scale ? 1.0 / std::sqrt((double)W * H) : 1.0;
#pragma omp parallel for schedule(static)
  for (long long s = 0; s < S; ++s) {
    std::vector<std::complex<double>> img((size_t)W * H), line, tmp;
    const T* in = src.data() + s * W * H;
    for (size_t i = 0; i < (size_t)W * H; ++i) img[i] = {(double)in[i].x, (double)in[i].y};
    line.resize(W);
    for (unsigned y = 0; y < H; ++y) dft(img.data() + (size_t)y * W, W, sign, tmp);
    line.resize(H);
    for (unsigned x = 0; x < W; ++x) {
      for (unsigned y = 0; y < H; ++y) line[y] = img[x + (size_t)W * y];
      dft(line.data(), H, sign, tmp);
      for (unsigned y = 0; y < H; ++y) img[x + (size_t)W * y] = line[y];
    }
    T* out = dst.data() + s * W * H;
    for (size_t i = 0; i < (size_t)W * H; ++i) {
      out[i].x = (decltype(out[i].x))(img[i].real() * sc);
      out[i].y = (decltype(out[i].y))(img[i].imag() * sc);
    }
  }
}
}  // namespace detail

template <typename T, unsigned N>
void fft2(const LinearMemoryBase<T, N>& src, LinearMemoryBase<T, N>& dst, bool scale_sqrt = false) {
  detail::fft2_impl(src, dst, scale_sqrt, -1);
}
template <typename T, unsigned N>
void ifft2(const LinearMemoryBase<T, N>& src, LinearMemoryBase<T, N>& dst, bool scale_sqrt = false) {
  detail::fft2_impl(src, dst, scale_sqrt, +1);
}
// dst(x + W/2 mod W, y + H/2 mod H) = src(x, y), for every slice of the third dimension
template <typename T, unsigned N>
void fftshift2(const LinearMemoryBase<T, N>& src, LinearMemoryBase<T, N>& dst) {
  const unsigned W = src.size()[0], H = src.size()[1];
  const size_t S = src.numel() / ((size_t)W * H);
  for (size_t s = 0; s < S; ++s)
    for (unsigned y = 0; y < H; ++y)
      for (unsigned x = 0; x < W; ++x)
        dst.data()[s * W * H + (x + W / 2) % W + (size_t)W * ((y + H / 2) % H)] =
            src.data()[s * W * H + x + (size_t)W * y];
}
}  // namespace fft
}  // namespace math
}  // namespace iu

// ---- complex helpers of iuhelpermath -----------------------------------------------------------------
template <typename PixelType>
inline typename iu::type_trait<PixelType>::complex_type complex_multiply(
    typename iu::type_trait<PixelType>::complex_type a, typename iu::type_trait<PixelType>::complex_type b) {
  return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
template <typename PixelType>
inline typename iu::type_trait<PixelType>::complex_type complex_multiply_conjugate(
    typename iu::type_trait<PixelType>::complex_type a, typename iu::type_trait<PixelType>::complex_type b) {
  return {a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y};
}

// ---- errors ------------------------------------------------------------------------------------------
class IuException : public std::runtime_error {
 public:
  IuException(const std::string& msg, const char* file = "", const char* func = "", int line = 0)
      : std::runtime_error(msg) {
    (void)file;
    (void)func;
    (void)line;
  }
};
#define IU_CUDA_CHECK ((void)0)
#define IU_SIZE_CHECK(a, b)                                                                     \
  do {                                                                                          \
    if ((a) != (b)) {                                                                           \
      std::stringstream pdtref_ss;                                                              \
      pdtref_ss << "size mismatch " << (a) << " vs " << (b);                                    \
      throw IuException(pdtref_ss.str(), __FILE__, __FUNCTION__, __LINE__);                     \
    }                                                                                           \
  } while (0)
