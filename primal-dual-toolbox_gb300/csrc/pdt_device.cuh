// pdt_device.cuh -- device helpers shared by the engine's kernels: complex arithmetic on float2 and the
// batched shared-memory mixed-radix FFT used by the Cartesian / sampling operators.
#pragma once

#ifndef PDT_HOST_EMULATION
#include <cuda_runtime.h>
#endif
#include <cstdint>

namespace pdt {

// ------------------------------------------------------------------------------------------------
// complex64 arithmetic (float2), the ImageUtilities iuhelpermath operations used by the reference.
// ------------------------------------------------------------------------------------------------
__host__ __device__ __forceinline__ float2 c2(float a, float b) { return make_float2(a, b); }
__host__ __device__ __forceinline__ float2 operator+(float2 a, float2 b) { return c2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ float2 operator-(float2 a, float2 b) { return c2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ float2 operator-(float2 a) { return c2(-a.x, -a.y); }
__host__ __device__ __forceinline__ float2 operator*(float s, float2 a) { return c2(s * a.x, s * a.y); }
__host__ __device__ __forceinline__ float2 operator*(float2 a, float s) { return c2(a.x * s, a.y * s); }
__host__ __device__ __forceinline__ float2 operator/(float2 a, float s) { return c2(a.x / s, a.y / s); }
__host__ __device__ __forceinline__ float2& operator+=(float2& a, float2 b) { a.x += b.x; a.y += b.y; return a; }
// a * b and a * conj(b): complex_multiply / complex_multiply_conjugate of mricartesianoperator.cu
__host__ __device__ __forceinline__ float2 cmul(float2 a, float2 b) { return c2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__host__ __device__ __forceinline__ float2 cmulc(float2 a, float2 b) { return c2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y); }
__host__ __device__ __forceinline__ float2 conjf2(float2 a) { return c2(a.x, -a.y); }

#ifndef PDT_HOST_EMULATION
// Programmatic dependent launch: a kernel launched with programmatic stream serialisation may be
// launched while its predecessor in the stream finishes; pdl_wait() blocks until the predecessor grid
// has completed and its writes are visible (it returns at once for an ordinary launch).
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Lets the next kernel in the stream launch once every block of this grid has executed it (or exited), so
// that its blocks take SMs as they free up and run their set-up before their own pdl_wait(). Called right
// after pdl_wait(): only the next grid is launched early, and it still waits for this one to complete.
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// Asynchronous global -> shared copies (cp.async; completion per thread by commit groups).
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
#endif

// |z|^2 of a pixel (real or complex).
__device__ __forceinline__ float abs2(float a) { return a * a; }
__device__ __forceinline__ float abs2(float2 a) { return a.x * a.x + a.y * a.y; }
template <class P> __device__ __forceinline__ P pzero();
template <> __device__ __forceinline__ float pzero<float>() { return 0.f; }
template <> __device__ __forceinline__ float2 pzero<float2>() { return c2(0.f, 0.f); }

// x * (s*i) for s = +-1
__device__ __forceinline__ float2 mul_si(float2 x, float s) { return c2(-s * x.y, s * x.x); }

// ------------------------------------------------------------------------------------------------
// FFT plan: length n = prod(radix[i]); radices 8, 4, 2, 3, 5 have dedicated butterflies, 7..31 odd
// primes a compile-time direct DFT, anything else a runtime direct DFT.
// ------------------------------------------------------------------------------------------------
constexpr int kMaxStages = 24;
struct FftPlan {
  int n;
  int nst;
  int radix[kMaxStages];
};

// Direct-DFT butterflies for compile-time radix RAD. `w` holds w_RAD^m, m = 0..RAD-1 (conjugated for
// the inverse).
template <int RAD>
__device__ __forceinline__ void dft_small(float2 (&v)[RAD], const float2* __restrict__ w) {
  float2 o[RAD];
#pragma unroll
  for (int q = 0; q < RAD; ++q) {
    float2 acc = v[0];
#pragma unroll
    for (int r = 1; r < RAD; ++r) {
      const float2 t = w[(r * q) % RAD];
      acc.x += v[r].x * t.x - v[r].y * t.y;
      acc.y += v[r].x * t.y + v[r].y * t.x;
    }
    o[q] = acc;
  }
#pragma unroll
  for (int q = 0; q < RAD; ++q) v[q] = o[q];
}

__device__ __forceinline__ void dft2(float2& a0, float2& a1) {
  const float2 t = a0;
  a0 = t + a1;
  a1 = t - a1;
}

// 4-point DFT, sign s = -1 forward / +1 inverse.
__device__ __forceinline__ void dft4(float2& a0, float2& a1, float2& a2, float2& a3, float s) {
  const float2 t0 = a0 + a2, t1 = a0 - a2, t2 = a1 + a3, t3 = mul_si(a1 - a3, s);
  a0 = t0 + t2;
  a2 = t0 - t2;
  a1 = t1 + t3;
  a3 = t1 - t3;
}

__device__ __forceinline__ void dft8(float2 (&v)[8], float s) {
  float2 e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
  float2 o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
  dft4(e0, e1, e2, e3, s);
  dft4(o0, o1, o2, o3, s);
  const float h = 0.70710678118654752440f;
  // w8^1 = h(1 + s i), w8^2 = s i, w8^3 = h(-1 + s i)
  const float2 w1o1 = c2(h * (o1.x - s * o1.y), h * (o1.y + s * o1.x));
  const float2 w2o2 = mul_si(o2, s);
  const float2 w3o3 = c2(h * (-o3.x - s * o3.y), h * (-o3.y + s * o3.x));
  v[0] = e0 + o0;
  v[4] = e0 - o0;
  v[1] = e1 + w1o1;
  v[5] = e1 - w1o1;
  v[2] = e2 + w2o2;
  v[6] = e2 - w2o2;
  v[3] = e3 + w3o3;
  v[7] = e3 - w3o3;
}

__device__ __forceinline__ void dft3(float2 (&v)[3], float s) {
  const float c = -0.5f, sn = 0.86602540378443864676f;
  const float2 t = v[1] + v[2], d = v[1] - v[2];
  const float2 m = v[0] + c * t;
  const float2 j = mul_si(d, s * sn);
  v[0] = v[0] + t;
  v[1] = m + j;
  v[2] = m - j;
}

__device__ __forceinline__ void dft5(float2 (&v)[5], float s) {
  const float c1 = 0.30901699437494742410f, c2v = -0.80901699437494742410f;
  const float s1 = 0.95105651629515357212f, s2 = 0.58778525229247312917f;
  const float2 t1 = v[1] + v[4], t2 = v[2] + v[3], d1 = v[1] - v[4], d2 = v[2] - v[3];
  const float2 a = v[0] + c1 * t1 + c2v * t2;
  const float2 b = v[0] + c2v * t1 + c1 * t2;
  const float2 ja = mul_si(s1 * d1 + s2 * d2, s);
  const float2 jb = mul_si(s2 * d1 - s1 * d2, s);
  v[0] = v[0] + t1 + t2;
  v[1] = a + ja;
  v[4] = a - ja;
  v[2] = b + jb;
  v[3] = b - jb;
}

// One Stockham pass for compile-time radix RAD over one butterfly: reads src[r*nb], twiddles by
// w_{Ns*RAD}^{r*k} = tw[r*kstep], takes the RAD-point DFT and writes dst[r*Ns].
template <int RAD>
__device__ __forceinline__ void stockham_bfly(const float2* __restrict__ src, float2* __restrict__ dst, int nb,
                                              int Ns, int kstep, const float2* __restrict__ tw, int n, float s) {
  float2 v[RAD];
#pragma unroll
  for (int r = 0; r < RAD; ++r) {
    float2 x = src[r * nb];
    if (r > 0) {
      float2 w = tw[r * kstep];
      w.y *= -s;  // tw holds exp(-2 pi i t/n); the inverse (s = +1) conjugates
      x = cmul(x, w);
    }
    v[r] = x;
  }
  if constexpr (RAD == 2) {
    dft2(v[0], v[1]);
  } else if constexpr (RAD == 4) {
    dft4(v[0], v[1], v[2], v[3], s);
  } else if constexpr (RAD == 8) {
    dft8(v, s);
  } else if constexpr (RAD == 3) {
    dft3(v, s);
  } else if constexpr (RAD == 5) {
    dft5(v, s);
  } else {
    float2 w[RAD];
    const int step = n / RAD;
#pragma unroll
    for (int m = 0; m < RAD; ++m) {
      float2 t = tw[m * step];
      t.y *= -s;
      w[m] = t;
    }
    dft_small<RAD>(v, w);
  }
#pragma unroll
  for (int r = 0; r < RAD; ++r) dst[r * Ns] = v[r];
}

// Runtime-radix butterfly (direct DFT read straight from shared memory) for radices without a
// compile-time instance.
__device__ __forceinline__ void stockham_bfly_dyn(const float2* __restrict__ src, float2* __restrict__ dst, int RAD,
                                                  int nb, int Ns, int kstep, const float2* __restrict__ tw, int n,
                                                  float s) {
  const int step = n / RAD;
  for (int q = 0; q < RAD; ++q) {
    float2 acc = c2(0.f, 0.f);
    for (int r = 0; r < RAD; ++r) {
      float2 x = src[r * nb];
      float2 w = tw[(r * kstep) % n];
      w.y = s > 0 ? -w.y : w.y;
      x = cmul(x, w);
      float2 t = tw[((r * q) % RAD) * step];
      t.y = s > 0 ? -t.y : t.y;
      acc += cmul(x, t);
    }
    dst[q * Ns] = acc;
  }
}

// Batched in-shared-memory FFT: `nseq` sequences of length plan.n, sequence b at a[b*ld ... b*ld+n).
// `b` is scratch of the same shape. The whole block participates; the call ends with a barrier.
// Returns the buffer that holds the result (a or b). inverse: exp(+2 pi i ...), unscaled.
static __device__ __noinline__ float2* smem_fft(float2* a, float2* b, int nseq, int ld, const FftPlan& pl,
                                         const float2* __restrict__ tw, bool inverse) {
  const float s = inverse ? 1.f : -1.f;
  const int n = pl.n;
  int Ns = 1;
  for (int st = 0; st < pl.nst; ++st) {
    const int RAD = pl.radix[st];
    const int nb = n / RAD;
    const int kstep_unit = n / (Ns * RAD);
    const int total = nb * nseq;
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
      const int sq = t / nb;
      const int j = t - sq * nb;
      const int k = j % Ns;
      const float2* src = a + (size_t)sq * ld + j;
      float2* dst = b + (size_t)sq * ld + (j / Ns) * Ns * RAD + k;
      const int kstep = k * kstep_unit;
      switch (RAD) {
        case 2: stockham_bfly<2>(src, dst, nb, Ns, kstep, tw, n, s); break;
        case 3: stockham_bfly<3>(src, dst, nb, Ns, kstep, tw, n, s); break;
        case 4: stockham_bfly<4>(src, dst, nb, Ns, kstep, tw, n, s); break;
        case 5: stockham_bfly<5>(src, dst, nb, Ns, kstep, tw, n, s); break;
        case 7: stockham_bfly<7>(src, dst, nb, Ns, kstep, tw, n, s); break;
        case 8: stockham_bfly<8>(src, dst, nb, Ns, kstep, tw, n, s); break;
        case 11: stockham_bfly<11>(src, dst, nb, Ns, kstep, tw, n, s); break;
        case 13: stockham_bfly<13>(src, dst, nb, Ns, kstep, tw, n, s); break;
        case 17: stockham_bfly<17>(src, dst, nb, Ns, kstep, tw, n, s); break;
        case 19: stockham_bfly<19>(src, dst, nb, Ns, kstep, tw, n, s); break;
        case 23: stockham_bfly<23>(src, dst, nb, Ns, kstep, tw, n, s); break;
        default: stockham_bfly_dyn(src, dst, RAD, nb, Ns, kstep, tw, n, s); break;
      }
    }
    __syncthreads();
    float2* t = a;
    a = b;
    b = t;
    Ns *= RAD;
  }
  return a;
}

}  // namespace pdt
