// pdt_cnn.cu -- the learned warm start: a small residual CNN with BF16 weights and activations and FP32
// accumulation, trained and run by the engine's own kernels.
//
// Network (fully convolutional, 3 x 3 convolutions, zero padding, channel-last BF16 activations):
//   x  = [Re u0, Im u0] / s                       (u0 = A^H f, s = max |u0|)
//   h1 = relu(conv_in(x))                          2 -> 32
//   h_{l+1} = h_l + relu(conv_l(h_l)), l = 1..6    32 -> 32
//   o  = conv_out(h7)                              32 -> 8 (6 used)
//   u  = u0 + s (o0 + i o1),  v = s (o2 + i o3, o4 + i o5)
// Eight convolutions in all. The 32-channel convolutions run as implicit GEMMs on the tensor cores
// (mma.sync m16n8k16, BF16 in, FP32 accumulate): pixels are the M dimension, output channels N, and
// (tap, input channel) K. The data gradient is the same kernel with flipped taps and transposed channels;
// the weight gradient is a second implicit GEMM with pixels as K, reduced over blocks in block order.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <memory>
#include <vector>

#include "pdt_device.cuh"
#include "pdt_internal.h"
#include "pdt_tc.cuh"

namespace pdt {
namespace {

typedef __nv_bfloat16 bf16;

constexpr int CH = 32;    // hidden channels
constexpr int TW = 16;    // pixel tile width (one mma M tile)
constexpr int TH = 8;     // pixel tile height (one row per warp)
constexpr int NTAP = 9;

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t*>(&v);
}

__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

enum Epi {
  EPI_RELU_RES = 2,  // zsave = z, out = in + relu(z)   (CIN == COUT)
  EPI_F32 = 3,       // out32 = z (FP32)
  EPI_ACC = 4,       // acc32 += bf16(z)  (a residual stream's FP32 gradient; the BF16 rounding of a stored z)
  EPI_F32_BF16 = 5   // out32 = bf16(z), stored as FP32 (starts a residual stream's gradient)
};

// 32 -> 32 channel 3 x 3 convolution on the fifth-generation tensor cores (tcgen05 kind::f16, BF16
// operands, FP32 accumulator in tensor memory), as an implicit GEMM without an im2col copy. One CTA computes
// a tile of 8 x 16 pixels (x, y) = the 128 rows of one MMA tile, rows ordered y-major. The input tile with
// its one-pixel zero halo (10 x 18 pixels) sits in shared memory in the no-swizzle K-major layout: channel
// group g (8 channels, 16 bytes) of pixel p at byte g 2912 + 16 p, so eight consecutive pixels form a core
// matrix (the group stride, two pixels more than the 180 of a group, puts the four groups of a pixel in
// four different bank quarters, so the halo's 16-byte stores do not conflict); the 8-pixel groups of the M tile are one halo row (160 bytes) apart, and tap (ky, kx) is the
// same layout started 16 (10 ky + kx) bytes in. The weights sit the same way ([tap][g][co] x 16 bytes).
// K = (tap, channel) = 288 in 18 MMAs of K = 16 (two channel groups), N = 32 output channels. One thread
// issues the MMAs and commits them to an mbarrier; the epilogue reads pixel rows from tensor memory
// (warps q and q + 4 share lane quarter q, 16 output channels each).
constexpr int kConvTcThreads = 256;
constexpr int kConvTcTW = 8, kConvTcTH = 16;                      // tile: 8 pixels wide, 16 rows
constexpr int kConvTcHaloPix = (kConvTcTW + 2) * (kConvTcTH + 2);  // 180
constexpr uint32_t kConvTcGroup = 16 * (kConvTcHaloPix + 2);       // 2912: one channel group of the tile
constexpr uint32_t kConvTcIn = 4 * kConvTcGroup;                   // 11,648 bytes
constexpr uint32_t kConvTcW = NTAP * 4 * 32 * 16;                   // 18,432 bytes
// The farthest operand byte an MMA reads: A at tap (2, 2), channel groups 2, 3: 16 (2 10 + 2) + 2 2912 +
// 2912 (second K core matrix) + 15 160 (last 8-pixel group) + 128 = 11,616 <= kConvTcIn; B at tap 8, groups
// 2, 3: (8 4 + 2) 512 + 512 + 3 128 + 128 = 18,432 = kConvTcW. The mbarrier, the tensor-memory slot and
// the 32 biases (FP32) follow the weights.
constexpr size_t kConvTcSmem = 1024 + kConvTcIn + kConvTcW + 16 + 128;
constexpr int kConvTcItems = kConvTcHaloPix * 4;                                 // 720 16-byte items per tile
constexpr int kConvTcPre = (kConvTcItems + kConvTcThreads - 1) / kConvTcThreads;  // 3 per thread

__device__ __forceinline__ void ld_shared_v4(uint32_t addr, uint32_t (&v)[4]) {
  asm volatile("ld.shared.v4.b32 {%0, %1, %2, %3}, [%4];" : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]) : "r"(addr));
}

// Persistent: a CTA loads the weights once and walks tiles t = blockIdx.x, + gridDim.x, ... of the
// (x tiles) x (y tiles) x B grid; the completion barrier's phase alternates per tile. The next tile's halo
// is loaded into registers right after this tile's MMAs are issued, so its global-load latency overlaps
// the MMAs and the epilogue; it is stored to shared memory once the tile buffer is free.
template <int EPI>
__global__ void __launch_bounds__(kConvTcThreads, 4) conv3x3_tc(const bf16* __restrict__ in, const bf16* __restrict__ w,
                                                            const float* __restrict__ bias, int B, int H, int W,
                                                            bf16* __restrict__ out, bf16* __restrict__ zsave,
                                                            int* __restrict__ err, float* __restrict__ acc32) {
  static_assert(EPI == EPI_RELU_RES || EPI == EPI_ACC, "epilogues of the 32 -> 32 layers");
  extern __shared__ unsigned char conv_smem_raw[];
  const uint32_t off = tc::smem_addr(conv_smem_raw);
  unsigned char* sm = conv_smem_raw + ((1024u - (off & 1023u)) & 1023u);
  const uint32_t in_base = tc::smem_addr(sm), w_base = in_base + kConvTcIn;
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + kConvTcIn + kConvTcW);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 1);
  float* bias_s = reinterpret_cast<float*>(sm + kConvTcIn + kConvTcW + 16);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int ntx = (W + kConvTcTW - 1) / kConvTcTW, nty = (H + kConvTcTH - 1) / kConvTcTH;
  const int ntiles = ntx * nty * B;
  if (tid < CH) bias_s[tid] = bias ? bias[tid] : 0.f;
  if (tid == 0) {
    tc::mbar_init(bar, 1);
    tc::fence_mbar_init();
  }
  if (warp == 0) tc::tmem_alloc(tslot, 32);
  // weights: item (tap, group, co) at byte ((tap 4 + g) 32 + co) 16
  for (int i = tid; i < NTAP * 4 * 32; i += kConvTcThreads) {
    const int co = i & 31, g = (i >> 5) & 3, tap = i >> 7;
    const uint4 v = __ldg(reinterpret_cast<const uint4*>(w + ((size_t)tap * CH + co) * CH) + g);
    asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(w_base + 16 * i), "r"(v.x), "r"(v.y), "r"(v.z),
                 "r"(v.w)
                 : "memory");
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;
  const int q = warp & 3, h = warp >> 2;
  // the halo of tile t: item i = (pixel, channel group) of 16 bytes, zero outside the image
  uint4 pre[kConvTcPre];
  auto fetch = [&](int t) {
    const int bx = t % ntx, by = (t / ntx) % nty, b = t / (ntx * nty);
    const int x0 = bx * kConvTcTW, y0 = by * kConvTcTH;
    const bf16* inb = in + (size_t)b * H * W * CH;
#pragma unroll
    for (int j = 0; j < kConvTcPre; ++j) {
      const int i = tid + j * kConvTcThreads;
      const int g = i & 3, pix = i >> 2;
      const int hy = pix / (kConvTcTW + 2), hx = pix - hy * (kConvTcTW + 2);
      const int gy = y0 + hy - 1, gx = x0 + hx - 1;
      pre[j] = make_uint4(0u, 0u, 0u, 0u);
      if (i < kConvTcItems && gy >= 0 && gy < H && gx >= 0 && gx < W)
        pre[j] = __ldg(reinterpret_cast<const uint4*>(inb + ((size_t)gy * W + gx) * CH) + g);
    }
  };
  bool ok = true;
  int it = 0;
  if (blockIdx.x < ntiles) fetch(blockIdx.x);
  for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x, ++it) {
    const int bx = t % ntx, by = (t / ntx) % nty, b = t / (ntx * nty);
    const int x0 = bx * kConvTcTW, y0 = by * kConvTcTH;
    // the tile buffer is free (the previous tile's MMAs and epilogue are done)
#pragma unroll
    for (int j = 0; j < kConvTcPre; ++j) {
      const int i = tid + j * kConvTcThreads;
      if (i < kConvTcItems)
        asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(in_base + (i & 3) * kConvTcGroup + 16 * (i >> 2)),
                     "r"(pre[j].x), "r"(pre[j].y), "r"(pre[j].z), "r"(pre[j].w)
                     : "memory");
    }
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    // (the test hook withholds block 0's first tile: no MMAs and no commit, so the wait below runs out)
    if (tid == 0 && !(it == 0 && blockIdx.x == 0 && tc::g_drop_arrival)) {
      const uint32_t idesc = tc::idesc_bf16(128, CH);
      for (int tap = 0; tap < NTAP; ++tap) {
        const uint32_t a0 = in_base + 16 * ((tap / 3) * (kConvTcTW + 2) + tap % 3);
        for (int k = 0; k < 2; ++k)  // channel groups 2k, 2k + 1
          tc::mma_bf16(tmem, tc::desc_interleave(a0 + 2 * k * kConvTcGroup, kConvTcGroup, 16 * (kConvTcTW + 2)),
                       tc::desc_interleave(w_base + (tap * 4 + 2 * k) * 512, 512, 128), idesc, (tap | k) ? 1u : 0u);
      }
      tc::mma_commit(bar);
    }
    if (t + (int)gridDim.x < ntiles) fetch(t + gridDim.x);
    const int m = 32 * q + lane, gy = y0 + (m >> 3), gx = x0 + (m & 7);  // row m = pixel (m % 8, m / 8)
    const bool inside = gy < H && gx < W;
    const size_t pix = ((size_t)b * H + gy) * W + gx;
    float4 acc_in[4];  // the accumulated gradient, loaded while the MMAs run
    if constexpr (EPI == EPI_ACC) {
      if (inside) {
        const float4* ap = reinterpret_cast<const float4*>(acc32 + pix * CH + 16 * h);
#pragma unroll
        for (int q4 = 0; q4 < 4; ++q4) acc_in[q4] = ap[q4];
      }
    }
    ok = tc::mbar_wait(bar, it & 1);  // every thread waits each phase in turn
    // after a give-up, wait once more (bounded) for MMAs still in flight before the tile buffer, the
    // accumulator and finally the tensor memory are released
    if (!ok) tc::mbar_wait(bar, it & 1);
    tc::fence_after_sync();
    float v[16];
    tc::tmem_ld16(tmem + ((uint32_t)(32 * q) << 16) + 16 * h, v);
    if (ok && inside) {
      uint32_t o[8], zz[8], res[8];
      float bs[16];
      if constexpr (EPI == EPI_RELU_RES) {
#pragma unroll
        for (int q4 = 0; q4 < 4; ++q4) {
          uint32_t r[4];
          ld_shared_v4(tc::smem_addr(bias_s) + 64 * h + 16 * q4, r);
#pragma unroll
          for (int e = 0; e < 4; ++e) bs[4 * q4 + e] = __uint_as_float(r[e]);
        }
      }
      if constexpr (EPI == EPI_RELU_RES) {  // the residual input: this pixel's channels 16 h .. 16 h + 15 in the tile
        const uint32_t hp = in_base + 16 * (((m >> 3) + 1) * (kConvTcTW + 2) + (m & 7) + 1);
        ld_shared_v4(hp + 2 * h * kConvTcGroup, *reinterpret_cast<uint32_t(*)[4]>(&res[0]));
        ld_shared_v4(hp + (2 * h + 1) * kConvTcGroup, *reinterpret_cast<uint32_t(*)[4]>(&res[4]));
      }
#pragma unroll
      for (int j = 0; j < 8; ++j) {  // output channels 16 h + 2 j, + 1
        float z0 = v[2 * j], z1 = v[2 * j + 1];
        if constexpr (EPI == EPI_RELU_RES) {
          z0 += bs[2 * j];
          z1 += bs[2 * j + 1];
        }
        if constexpr (EPI == EPI_ACC) {
          o[j] = pack_bf16(z0, z1);
        } else {
          zz[j] = pack_bf16(z0, z1);
          const __nv_bfloat162 hv = *reinterpret_cast<const __nv_bfloat162*>(&res[j]);
          o[j] = pack_bf16(__bfloat162float(hv.x) + fmaxf(z0, 0.f), __bfloat162float(hv.y) + fmaxf(z1, 0.f));
        }
      }
      if constexpr (EPI == EPI_ACC) {
        float4* ap = reinterpret_cast<float4*>(acc32 + pix * CH + 16 * h);
#pragma unroll
        for (int q4 = 0; q4 < 4; ++q4) {
          float4 a = acc_in[q4];
          const __nv_bfloat162 lo = *reinterpret_cast<const __nv_bfloat162*>(&o[2 * q4]);
          const __nv_bfloat162 hi = *reinterpret_cast<const __nv_bfloat162*>(&o[2 * q4 + 1]);
          a.x += __bfloat162float(lo.x);
          a.y += __bfloat162float(lo.y);
          a.z += __bfloat162float(hi.x);
          a.w += __bfloat162float(hi.y);
          ap[q4] = a;
        }
      } else {
        uint4* op = reinterpret_cast<uint4*>(out + pix * CH + 16 * h);
        op[0] = make_uint4(o[0], o[1], o[2], o[3]);
        op[1] = make_uint4(o[4], o[5], o[6], o[7]);
      }
      if constexpr (EPI == EPI_RELU_RES) {
        uint4* zp = reinterpret_cast<uint4*>(zsave + pix * CH + 16 * h);
        zp[0] = make_uint4(zz[0], zz[1], zz[2], zz[3]);
        zp[1] = make_uint4(zz[4], zz[5], zz[6], zz[7]);
      }
    }
    ok = __syncthreads_and(ok);  // the tile buffer and the accumulator are free for the next tile
  }
  if (!ok && tid == 0) atomicExch(err, 0x2000);
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, 32);
  }
}

// 3 x 3 convolution as an implicit GEMM on warp-level MMAs, for the layers tcgen05 does not take (N = 8
// output channels; the 16-channel padded output gradient): in: [B][H][W][CIN] BF16; w: [9][COUT][CIN] BF16;
// bias: [COUT] FP32 (may be null); FP32 output. Each block computes a 16 x 8 pixel tile; warp w owns tile
// row w (16 pixels = one M tile).
template <int CIN, int COUT, int EPI>
__global__ void __launch_bounds__(32 * TH) conv3x3_mma(const bf16* __restrict__ in, const bf16* __restrict__ w,
                                                       const float* __restrict__ bias, int H, int W,
                                                       float* __restrict__ out32) {
  static_assert(CIN % 16 == 0 && COUT % 8 == 0, "channel counts");
  static_assert(EPI == EPI_F32 || EPI == EPI_F32_BF16, "epilogues of the 32 -> 8 layer and the first data gradient");
  constexpr int PS = CIN + 4;       // smem pixel stride (bf16): spreads the fragment loads over all banks
  constexpr int WS = CIN + 8;       // smem weight row stride (bf16)
  __shared__ __align__(16) bf16 s_in[(TH + 2) * (TW + 2) * PS];
  __shared__ __align__(16) bf16 s_w[NTAP * COUT * WS];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int gid = lane >> 2, tig = lane & 3;
  const int x0 = blockIdx.x * TW, y0 = blockIdx.y * TH, b = blockIdx.z;
  const bf16* inb = in + (size_t)b * H * W * CIN;
  // stage weights and the input tile with a one-pixel halo (zero outside the image), 4-byte granules
  for (int i = tid; i < NTAP * COUT * (CIN / 2); i += blockDim.x) {
    const int row = i / (CIN / 2), c2 = i - row * (CIN / 2);
    reinterpret_cast<uint32_t*>(s_w + row * WS)[c2] = reinterpret_cast<const uint32_t*>(w + (size_t)row * CIN)[c2];
  }
  for (int i = tid; i < (TH + 2) * (TW + 2) * (CIN / 2); i += blockDim.x) {
    const int pix = i / (CIN / 2), c2 = i - pix * (CIN / 2);
    const int ty = pix / (TW + 2), tx = pix - ty * (TW + 2);
    const int gy = y0 - 1 + ty, gx = x0 - 1 + tx;
    uint32_t v = 0;
    if (gy >= 0 && gy < H && gx >= 0 && gx < W)
      v = reinterpret_cast<const uint32_t*>(inb + ((size_t)gy * W + gx) * CIN)[c2];
    reinterpret_cast<uint32_t*>(s_in + pix * PS)[c2] = v;
  }
  __syncthreads();
  float acc[COUT / 8][4];
#pragma unroll
  for (int n = 0; n < COUT / 8; ++n) acc[n][0] = acc[n][1] = acc[n][2] = acc[n][3] = 0.f;
#pragma unroll
  for (int tap = 0; tap < NTAP; ++tap) {
    const int ky = tap / 3, kx = tap % 3;
    const bf16* arow0 = s_in + ((warp + ky) * (TW + 2) + gid + kx) * PS;  // pixel gid of this warp's row
    const bf16* arow1 = arow0 + 8 * PS;                                    // pixel gid + 8
#pragma unroll
    for (int kk = 0; kk < CIN / 16; ++kk) {
      uint32_t a[4];
      const int c = kk * 16 + tig * 2;
      a[0] = *reinterpret_cast<const uint32_t*>(arow0 + c);
      a[1] = *reinterpret_cast<const uint32_t*>(arow1 + c);
      a[2] = *reinterpret_cast<const uint32_t*>(arow0 + c + 8);
      a[3] = *reinterpret_cast<const uint32_t*>(arow1 + c + 8);
#pragma unroll
      for (int n = 0; n < COUT / 8; ++n) {
        const bf16* brow = s_w + (tap * COUT + n * 8 + gid) * WS + c;
        mma16816(acc[n], a, *reinterpret_cast<const uint32_t*>(brow), *reinterpret_cast<const uint32_t*>(brow + 8));
      }
    }
  }
  // epilogue: rows gid and gid + 8 of the M tile are pixels x0 + gid (+ 8) of image row y0 + warp
  const int gy = y0 + warp;
  if (gy >= H) return;
#pragma unroll
  for (int half = 0; half < 2; ++half) {
    const int gx = x0 + gid + 8 * half;
    if (gx >= W) continue;
    const size_t pix = ((size_t)b * H + gy) * W + gx;
#pragma unroll
    for (int n = 0; n < COUT / 8; ++n) {
      const int co = n * 8 + tig * 2;
      float z0 = acc[n][2 * half], z1 = acc[n][2 * half + 1];
      if (bias) {
        z0 += bias[co];
        z1 += bias[co + 1];
      }
      if constexpr (EPI == EPI_F32) {
        out32[pix * COUT + co] = z0;
        out32[pix * COUT + co + 1] = z1;
      } else {
        out32[pix * COUT + co] = __bfloat162float(__float2bfloat16(z0));
        out32[pix * COUT + co + 1] = __bfloat162float(__float2bfloat16(z1));
      }
    }
  }
}

// Weight gradient dW[tap][co][ci] = sum_p x[p + d(tap)][ci] dy[p][co] for CIN = 32 and COUT = 32 or 8:
// a persistent grid, each block walking 16 x 8 tiles and warp `tap` accumulating that tap's 32 x 32 (or
// 8 x 32) block in registers; partial[block] is summed by wgrad_reduce in block order.
template <int COUT>
__global__ void __launch_bounds__(32 * NTAP) wgrad_mma(const bf16* __restrict__ x, const bf16* __restrict__ dy, int B,
                                                       int H, int W, float* __restrict__ partial) {
  constexpr int CIN = CH;
  constexpr int XS = TW + 2 + 2;  // smem row stride of the transposed input tile (pixels)
  constexpr int DS = TW + 8;      // smem row stride of the transposed output-gradient tile
  __shared__ __align__(16) bf16 s_x[CIN * (TH + 2) * XS];  // [ci][ty][tx]
  __shared__ __align__(16) bf16 s_dy[COUT * TH * DS];       // [co][ty][tx]
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int gid = lane >> 2, tig = lane & 3;
  const int tap = warp, ky = tap / 3, kx = tap % 3;
  constexpr int MT = COUT >= 16 ? COUT / 16 : 1;  // M tiles over co (COUT 8: one padded tile)
  float acc[MT][CIN / 8][4];
#pragma unroll
  for (int m = 0; m < MT; ++m)
#pragma unroll
    for (int n = 0; n < CIN / 8; ++n) acc[m][n][0] = acc[m][n][1] = acc[m][n][2] = acc[m][n][3] = 0.f;
  const int tiles_x = (W + TW - 1) / TW, tiles_y = (H + TH - 1) / TH;
  const int ntiles = B * tiles_x * tiles_y;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int b = t / (tiles_x * tiles_y), r = t - b * tiles_x * tiles_y;
    const int y0 = (r / tiles_x) * TH, x0 = (r % tiles_x) * TW;
    __syncthreads();
    for (int i = tid; i < (TH + 2) * (TW + 2) * CIN; i += blockDim.x) {
      const int pix = i / CIN, ci = i - pix * CIN;
      const int ty = pix / (TW + 2), tx = pix - ty * (TW + 2);
      const int gy = y0 - 1 + ty, gx = x0 - 1 + tx;
      bf16 v = __float2bfloat16(0.f);
      if (gy >= 0 && gy < H && gx >= 0 && gx < W) v = x[(((size_t)b * H + gy) * W + gx) * CIN + ci];
      s_x[(ci * (TH + 2) + ty) * XS + tx] = v;
    }
    for (int i = tid; i < TH * TW * COUT; i += blockDim.x) {
      const int pix = i / COUT, co = i - pix * COUT;
      const int ty = pix / TW, tx = pix - ty * TW;
      const int gy = y0 + ty, gx = x0 + tx;
      bf16 v = __float2bfloat16(0.f);
      if (gy < H && gx < W) v = dy[(((size_t)b * H + gy) * W + gx) * COUT + co];
      s_dy[(co * TH + ty) * DS + tx] = v;
    }
    __syncthreads();
    // K = pixels: one k-step per tile row (16 pixels)
    for (int ty = 0; ty < TH; ++ty) {
#pragma unroll
      for (int m = 0; m < MT; ++m) {
        uint32_t a[4];
        const int co0 = m * 16 + gid, co1 = co0 + 8;
        const bf16* d0 = s_dy + (co0 * TH + ty) * DS + tig * 2;
        a[0] = *reinterpret_cast<const uint32_t*>(d0);
        a[2] = *reinterpret_cast<const uint32_t*>(d0 + 8);
        if (COUT >= 16) {
          const bf16* d1 = s_dy + (co1 * TH + ty) * DS + tig * 2;
          a[1] = *reinterpret_cast<const uint32_t*>(d1);
          a[3] = *reinterpret_cast<const uint32_t*>(d1 + 8);
        } else {
          a[1] = a[3] = 0u;  // rows 8..15 of the padded 8-channel tile
        }
#pragma unroll
        for (int n = 0; n < CIN / 8; ++n) {
          const bf16* xr = s_x + ((n * 8 + gid) * (TH + 2) + ty + ky) * XS + kx + tig * 2;
          const uint32_t b0 = (uint32_t)__bfloat16_as_ushort(xr[0]) | ((uint32_t)__bfloat16_as_ushort(xr[1]) << 16);
          const uint32_t b1 = (uint32_t)__bfloat16_as_ushort(xr[8]) | ((uint32_t)__bfloat16_as_ushort(xr[9]) << 16);
          mma16816(acc[m][n], a, b0, b1);
        }
      }
    }
  }
  // partial[block][tap][co][ci]
  float* pb = partial + ((size_t)blockIdx.x * NTAP + tap) * COUT * CIN;
#pragma unroll
  for (int m = 0; m < MT; ++m)
#pragma unroll
    for (int n = 0; n < CIN / 8; ++n)
#pragma unroll
      for (int hh = 0; hh < 2; ++hh) {
        const int co = m * 16 + gid + 8 * hh;
        if (co >= COUT) continue;
        const int ci = n * 8 + tig * 2;
        pb[co * CIN + ci] = acc[m][n][2 * hh];
        pb[co * CIN + ci + 1] = acc[m][n][2 * hh + 1];
      }
}

// Weight gradient of a 32 -> 32 layer on the tensor cores (tcgen05, kind::f16 BF16, FP32 in TMEM):
//   dW[ky 3 + kx][co][ci] = sum_p x[p + (ky - 1, kx - 1)][ci] dy[p][co]
// as D_ky[m = kx 32 + ci][n = co] = sum_k A[m][k] B[n][k] with K = the 16 pixels of one tile row: A is the
// input tile shifted by kx (rows 96..127 zero), B the output gradient. Per 16 x 8 tile and tile row py,
// three MMAs (ky = 0, 1, 2: A from halo row py + ky) of M = 128, N = 32, K = 16 into three accumulators
// (TMEM columns 32 ky). Operands in shared memory in the no-swizzle K-major layout (a core matrix is 8
// rows x 8 pixels, 16 bytes per row; the tile is staged transposed from the [pixel][channel] activations):
//   A: [halo row 10][pixel half 2][row group 16][128 B], row group = 4 kx + ci / 8  (LBO 2048, SBO 128)
//   B: [tile row 8][pixel half 2][channel group 4][128 B]                          (LBO 512, SBO 128)
// CTAs are persistent over tiles and accumulate in TMEM; each writes partial[block][tap][co][ci], which
// wgrad_reduce adds in block order.
constexpr int kWgThreads = 256;
constexpr uint32_t kWgA = 20 * 2048;  // 40 KB
constexpr uint32_t kWgB = 16 * 512;   // 8 KB
constexpr size_t kWgSmem = 1024 + kWgA + kWgB + 64;

__device__ __forceinline__ void st_shared_b16(uint32_t addr, uint16_t v) {
  asm volatile("st.shared.b16 [%0], %1;" ::"r"(addr), "h"(v) : "memory");
}
__device__ __forceinline__ uint16_t u4_elem(const uint4& v, int e) {
  const uint32_t w = e < 2 ? v.x : e < 4 ? v.y : e < 6 ? v.z : v.w;
  return (uint16_t)((e & 1) ? (w >> 16) : (w & 0xFFFFu));
}

__global__ void __launch_bounds__(kWgThreads) wgrad_tc(const bf16* __restrict__ x, const bf16* __restrict__ dy, int B,
                                                       int H, int W, float* __restrict__ partial, int* __restrict__ err) {
  extern __shared__ unsigned char wg_smem_raw[];
  const uint32_t off = tc::smem_addr(wg_smem_raw);
  unsigned char* sm = wg_smem_raw + ((1024u - (off & 1023u)) & 1023u);
  const uint32_t a_base = tc::smem_addr(sm), b_base = a_base + kWgA;
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + kWgA + kWgB);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int ntx = (W + TW - 1) / TW, nty = (H + TH - 1) / TH;
  const int ntiles = ntx * nty * B;
  if (tid == 0) {
    tc::mbar_init(bar, 1);
    tc::fence_mbar_init();
  }
  if (warp == 0) tc::tmem_alloc(tslot, 128);
  // the zero rows 96..127 of A (row groups 12..15 of every block), written once
  for (int i = tid; i < 20 * 4 * 8; i += kWgThreads) {
    const int blk = i >> 5, g = 12 + ((i >> 3) & 3), q = i & 7;
    asm volatile("st.shared.v4.b32 [%0], {%1, %1, %1, %1};" ::"r"(a_base + (blk * 16 + g) * 128 + q * 16), "r"(0u)
                 : "memory");
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;
  const bool drop = tc::g_drop_arrival != 0;
  bool ok = true;
  int it = 0;
  for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x, ++it) {
    const int bx = t % ntx, by = (t / ntx) % nty, b = t / (ntx * nty);
    const int x0 = bx * TW, y0 = by * TH;
    // x halo tile -> A, transposed and shifted: item (halo row, halo column, channel group of 8)
    for (int i = tid; i < (TH + 2) * (TW + 2) * 4; i += kWgThreads) {
      const int cg = i & 3, col = (i >> 2) % (TW + 2), hy = (i >> 2) / (TW + 2);
      const int gy = y0 + hy - 1, gx = x0 + col - 1;
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if (gy >= 0 && gy < H && gx >= 0 && gx < W)
        v = __ldg(reinterpret_cast<const uint4*>(x + (((size_t)b * H + gy) * W + gx) * CH) + cg);
#pragma unroll
      for (int kx = 0; kx < 3; ++kx) {
        const int px = col - kx;
        if (px < 0 || px >= TW) continue;
        const uint32_t base = a_base + ((hy * 2 + (px >> 3)) * 16 + kx * 4 + cg) * 128 + (px & 7) * 2;
#pragma unroll
        for (int e = 0; e < 8; ++e) st_shared_b16(base + e * 16, u4_elem(v, e));
      }
    }
    // dy tile -> B, transposed: item (tile row, pixel, channel group)
    for (int i = tid; i < TH * TW * 4; i += kWgThreads) {
      const int cg = i & 3, px = (i >> 2) % TW, py = (i >> 2) / TW;
      const int gy = y0 + py, gx = x0 + px;
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if (gy < H && gx < W) v = __ldg(reinterpret_cast<const uint4*>(dy + (((size_t)b * H + gy) * W + gx) * CH) + cg);
      const uint32_t base = b_base + ((py * 2 + (px >> 3)) * 4 + cg) * 128 + (px & 7) * 2;
#pragma unroll
      for (int e = 0; e < 8; ++e) st_shared_b16(base + e * 16, u4_elem(v, e));
    }
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    // (the test hook withholds block 0's first tile: no MMAs and no commit, so the wait below runs out)
    if (tid == 0 && !(it == 0 && blockIdx.x == 0 && drop)) {
      const uint32_t idesc = tc::idesc_bf16(128, CH);
      for (int py = 0; py < TH; ++py)
        for (int ky = 0; ky < 3; ++ky)
          tc::mma_bf16(tmem + 32 * ky, tc::desc_interleave(a_base + (py + ky) * 2 * 2048, 2048, 128),
                       tc::desc_interleave(b_base + py * 2 * 512, 512, 128), idesc, (it > 0 || py > 0) ? 1u : 0u);
      tc::mma_commit(bar);
    }
    ok = tc::mbar_wait(bar, it & 1);
    if (!ok) tc::mbar_wait(bar, it & 1);  // wait (bounded) for MMAs still in flight before the tiles are reused
    tc::fence_after_sync();
    ok = __syncthreads_and(ok);
  }
  // epilogue: TMEM lane m = kx 32 + ci (warps 0..3 own lanes 32 w .. 32 w + 31), column 32 ky + co
  if (ok && warp < 4) {
    const int m = 32 * warp + lane;
    const uint32_t taddr = tmem + ((uint32_t)(32 * warp) << 16);
    float* pb = partial + (size_t)blockIdx.x * NTAP * CH * CH;
#pragma unroll
    for (int ky = 0; ky < 3; ++ky) {
      float v[16];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        tc::tmem_ld16(taddr + 32 * ky + 16 * h, v);
        if (m < 96) {
          const int kx = m >> 5, ci = m & 31, tap = ky * 3 + kx;
#pragma unroll
          for (int j = 0; j < 16; ++j) pb[((size_t)tap * CH + 16 * h + j) * CH + ci] = v[j];
        }
      }
    }
  }
  if (!ok && tid == 0) atomicCAS(err, 0, 0x2100);
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, 128);
  }
}

// Two-level fixed-order sum of partial[b][i] over the blocks b: stage 1 adds block range s (blockIdx.y) into
// tmp[s][i], stage 2 (wgrad_reduce with nblocks = the range count) adds the ranges in order.
constexpr int kWgRanges = 16;
__global__ void wgrad_reduce_ranges(const float* __restrict__ partial, int nblocks, int n, float* __restrict__ tmp) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, r = blockIdx.y;
  if (i >= n) return;
  const int b0 = (int)((long long)r * nblocks / gridDim.y), b1 = (int)((long long)(r + 1) * nblocks / gridDim.y);
  float s = 0.f;
  for (int b = b0; b < b1; ++b) s += partial[(size_t)b * n + i];
  tmp[(size_t)r * n + i] = s;
}

// grad[i] = sum_b partial[b][i] (block order)
__global__ void wgrad_reduce(const float* __restrict__ partial, int nblocks, int n, float* __restrict__ grad) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int b = 0; b < nblocks; ++b) s += partial[(size_t)b * n + i];
    grad[i] = s;
  }
}

// Per-channel sums of dy [npix][C] (the bias gradient), stage 1: block b sums the pixels of its contiguous
// chunk -- C / 2 threads per pixel, two channels each, so that a warp reads consecutive bytes -- and writes
// partial[b][C]; sum_partials adds the blocks' partials in block order (deterministic).
template <int C>
__global__ void __launch_bounds__(256) bias_grad_partial(const bf16* __restrict__ dy, size_t npix,
                                                         float* __restrict__ partial) {
  constexpr int TPP = C / 2, PPB = 256 / TPP;  // threads per pixel, pixels per pass
  __shared__ float2 sh[256];
  const int t = threadIdx.x, cp = t % TPP, pr = t / TPP;
  const size_t chunk = (npix + gridDim.x - 1) / gridDim.x;
  const size_t p0 = (size_t)blockIdx.x * chunk, p1 = min(npix, p0 + chunk);
  float2 acc = c2(0.f, 0.f);
  for (size_t p = p0 + pr; p < p1; p += PPB) {
    const __nv_bfloat162 v = reinterpret_cast<const __nv_bfloat162*>(dy + p * C)[cp];
    acc.x += __low2float(v);
    acc.y += __high2float(v);
  }
  sh[t] = acc;
  __syncthreads();
  if (t < TPP) {
    float2 a = c2(0.f, 0.f);
    for (int r = 0; r < PPB; ++r) {
      a.x += sh[r * TPP + t].x;
      a.y += sh[r * TPP + t].y;
    }
    partial[(size_t)blockIdx.x * C + 2 * t] = a.x;
    partial[(size_t)blockIdx.x * C + 2 * t + 1] = a.y;
  }
}

// out[i] = sum over blocks b of partial[b * stride + i], i < n: one CUDA block per output, its 128 threads
// sum fixed strided subsets of the partials, then a fixed-order tree (the same order on every run).
__global__ void __launch_bounds__(128) sum_partials(const float* __restrict__ partial, int nblocks, int stride, int n,
                                                   float* __restrict__ out) {
  __shared__ float sh[128];
  const int i = blockIdx.x;
  if (i >= n) return;
  float s = 0.f;
  for (int b = threadIdx.x; b < nblocks; b += 128) s += partial[(size_t)b * stride + i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = 64; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[i] = sh[0];
}

// w'[tap'][ci][co] = w[8 - tap'][co][ci] (padded to COP output / CIP input channels) for the data gradient.
__global__ void flip_transpose(const bf16* __restrict__ w, int cout, int cin, int cop, int cip, bf16* __restrict__ wt) {
  const int n = NTAP * cip * cop;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int tap = i / (cip * cop), r = i - tap * cip * cop;
    const int ci = r / cop, co = r - ci * cop;  // wt[tap][ci (as out)][co (as in)]
    bf16 v = __float2bfloat16(0.f);
    if (ci < cin && co < cout) v = w[((size_t)(8 - tap) * cout + co) * cin + ci];
    wt[i] = v;
  }
}

// First layer, 2 -> 32 channels (too narrow for the tensor cores): SIMT, relu, saves z.
__global__ void conv_in_fwd(const float* __restrict__ x, const float* __restrict__ w, const float* __restrict__ bias,
                            int B, int H, int W, bf16* __restrict__ out, bf16* __restrict__ zsave) {
  const size_t n = (size_t)B * H * W;
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n; p += (size_t)gridDim.x * blockDim.x) {
    const int xx = (int)(p % W), yy = (int)((p / W) % H), b = (int)(p / ((size_t)W * H));
    float in[NTAP][2];
    for (int tap = 0; tap < NTAP; ++tap) {
      const int gy = yy + tap / 3 - 1, gx = xx + tap % 3 - 1;
      const bool ok = gy >= 0 && gy < H && gx >= 0 && gx < W;
      const size_t q = ((size_t)b * H + gy) * W + gx;
      in[tap][0] = ok ? x[q * 2] : 0.f;
      in[tap][1] = ok ? x[q * 2 + 1] : 0.f;
    }
    for (int co = 0; co < CH; co += 2) {
      float z[2];
      for (int j = 0; j < 2; ++j) {
        float s = bias[co + j];
        for (int tap = 0; tap < NTAP; ++tap)
          s += w[(tap * CH + co + j) * 2] * in[tap][0] + w[(tap * CH + co + j) * 2 + 1] * in[tap][1];
        z[j] = s;
      }
      reinterpret_cast<uint32_t*>(zsave + p * CH)[co / 2] = pack_bf16(z[0], z[1]);
      reinterpret_cast<uint32_t*>(out + p * CH)[co / 2] = pack_bf16(fmaxf(z[0], 0.f), fmaxf(z[1], 0.f));
    }
  }
}

// First-layer weight gradient: dW[tap][co][cj] = sum_p x[p + d][cj] g[p][co]; block per (tap, co).
// Weight and bias gradients of the 2 -> 32 input layer, stage 1: block b takes a contiguous chunk of
// pixels; lane = output channel co, the eight warps take every eighth pixel of the chunk; for each pixel a
// warp reads g[p][0..31] once (64 consecutive bytes) and the two input channels at the nine neighbours
// (broadcast), and accumulates all 9 x 2 weight terms and the bias term. The warps' sums are added in warp
// order in shared memory: partial[b][(tap CH + co) 2 + ci] = sum x[p + d(tap)][ci] g[p][co],
// partial[b][NTAP CH 2 + co] = sum g[p][co]. sum_partials adds the blocks in a fixed order.
constexpr int kConvInPartial = NTAP * CH * 2 + CH;
constexpr int kPartialBlocksPerSm = 8;  // blocks per SM of the input-layer gradient (short chunks, more in flight)
constexpr int kConvInWarps = 8;
__global__ void __launch_bounds__(32 * kConvInWarps) conv_in_wgrad_partial(const float* __restrict__ x,
                                                                           const bf16* __restrict__ g, int B, int H,
                                                                           int W, float* __restrict__ partial) {
  __shared__ float sh[kConvInWarps][2 * NTAP + 1][CH];
  const int co = threadIdx.x & 31, w = threadIdx.x >> 5;
  const size_t n = (size_t)B * H * W;
  const size_t chunk = (n + gridDim.x - 1) / gridDim.x;
  const size_t p0 = (size_t)blockIdx.x * chunk, p1 = min(n, p0 + chunk);
  const float2* x2 = reinterpret_cast<const float2*>(x);
  float acc[NTAP][2], sb = 0.f;
#pragma unroll
  for (int t = 0; t < NTAP; ++t) acc[t][0] = acc[t][1] = 0.f;
  for (size_t p = p0 + w; p < p1; p += kConvInWarps) {
    const int xx = (int)(p % W), yy = (int)((p / W) % H), b = (int)(p / ((size_t)W * H));
    const float gv = __bfloat162float(g[p * CH + co]);
    sb += gv;
#pragma unroll
    for (int t = 0; t < NTAP; ++t) {
      const int gy = yy + t / 3 - 1, gx = xx + t % 3 - 1;
      if (gy >= 0 && gy < H && gx >= 0 && gx < W) {
        const float2 xv = x2[((size_t)b * H + gy) * W + gx];
        acc[t][0] += xv.x * gv;
        acc[t][1] += xv.y * gv;
      }
    }
  }
#pragma unroll
  for (int t = 0; t < NTAP; ++t) {
    sh[w][2 * t][co] = acc[t][0];
    sh[w][2 * t + 1][co] = acc[t][1];
  }
  sh[w][2 * NTAP][co] = sb;
  __syncthreads();
  float* out = partial + (size_t)blockIdx.x * kConvInPartial;
  for (int i = threadIdx.x; i < (2 * NTAP + 1) * CH; i += blockDim.x) {
    const int j = i / CH, c = i - j * CH;  // j = 2 tap + ci, or 2 NTAP for the bias
    float s = 0.f;
    for (int ww = 0; ww < kConvInWarps; ++ww) s += sh[ww][j][c];
    if (j < 2 * NTAP)
      out[((j >> 1) * CH + c) * 2 + (j & 1)] = s;
    else
      out[NTAP * CH * 2 + c] = s;
  }
}

// g = bf16(acc) * relu'(z): the residual stream's FP32 gradient rounded to BF16 (the same rounding as a
// separate conversion) and masked by the ReLU's derivative, four elements per thread.
__global__ void relu_bwd_acc(const float* __restrict__ acc, const bf16* __restrict__ z, size_t n, bf16* __restrict__ g) {
  const size_t n4 = n / 4;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n4; i += (size_t)gridDim.x * blockDim.x) {
    const float4 a = reinterpret_cast<const float4*>(acc)[i];
    const uint2 zz = reinterpret_cast<const uint2*>(z)[i];
    const __nv_bfloat162 z01 = *reinterpret_cast<const __nv_bfloat162*>(&zz.x);
    const __nv_bfloat162 z23 = *reinterpret_cast<const __nv_bfloat162*>(&zz.y);
    const bf16 zero = __float2bfloat16(0.f);
    const bf16 g0 = __bfloat162float(z01.x) > 0.f ? __float2bfloat16(a.x) : zero;
    const bf16 g1 = __bfloat162float(z01.y) > 0.f ? __float2bfloat16(a.y) : zero;
    const bf16 g2 = __bfloat162float(z23.x) > 0.f ? __float2bfloat16(a.z) : zero;
    const bf16 g3 = __bfloat162float(z23.y) > 0.f ? __float2bfloat16(a.w) : zero;
    uint2 o;
    __nv_bfloat162 o01, o23;
    o01.x = g0;
    o01.y = g1;
    o23.x = g2;
    o23.y = g3;
    o.x = *reinterpret_cast<const uint32_t*>(&o01);
    o.y = *reinterpret_cast<const uint32_t*>(&o23);
    reinterpret_cast<uint2*>(g)[i] = o;
  }
}

__global__ void to_bf16(const float* __restrict__ a, size_t n, bf16* __restrict__ out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = __float2bfloat16(a[i]);
}

// Mean squared error over the 6 used output channels and its gradient (padded to 8 channels, BF16).
__global__ void mse_loss(const float* __restrict__ y, const float* __restrict__ t, size_t npix, float scale,
                         bf16* __restrict__ g, double* __restrict__ partial) {
  __shared__ double sh[256];
  double s = 0;
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < npix; p += (size_t)gridDim.x * blockDim.x) {
    for (int c = 0; c < 8; ++c) {
      float d = 0.f;
      if (c < 6) {
        d = y[p * 8 + c] - t[p * 6 + c];
        s += (double)d * d;
      }
      g[p * 8 + c] = __float2bfloat16(2.f * d * scale);
    }
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

// Adam on FP32 master weights, BF16 copy refreshed.
__global__ void adam_step(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                          float* __restrict__ v, int n, float lr, float b1, float b2, float eps, float c1, float c2,
                          bf16* __restrict__ wb) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    if (wb) wb[i] = __float2bfloat16(wi);
  }
}

// x = [Re, Im] of the complex input / s per image (s = max |u0| of that image, given).
__global__ void prep_input(const float2* __restrict__ u0, const float* __restrict__ inv_s, int B, size_t npix,
                           float* __restrict__ x) {
  const size_t n = (size_t)B * npix;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float s = inv_s[i / npix];
    x[2 * i] = u0[i].x * s;
    x[2 * i + 1] = u0[i].y * s;
  }
}

// u = u0 + s (o0 + i o1), vx = s (o2 + i o3), vy = s (o4 + i o5)
__global__ void assemble_output(const float2* __restrict__ u0, const float* __restrict__ o, const float* __restrict__ s,
                                int B, size_t npix, float2* __restrict__ u, float2* __restrict__ v) {
  const size_t n = (size_t)B * npix;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const size_t b = i / npix, p = i - b * npix;
    const float sc = s[b];
    u[i] = u0[i] + sc * c2(o[i * 8], o[i * 8 + 1]);
    v[(2 * b) * npix + p] = sc * c2(o[i * 8 + 2], o[i * 8 + 3]);
    v[(2 * b + 1) * npix + p] = sc * c2(o[i * 8 + 4], o[i * 8 + 5]);
  }
}

// training target: t = [(u* - u0)/s, v*/s] in 6 channels
__global__ void prep_target(const float2* __restrict__ u0, const float2* __restrict__ ut, const float2* __restrict__ vt,
                            const float* __restrict__ inv_s, int B, size_t npix, float* __restrict__ t) {
  const size_t n = (size_t)B * npix;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const size_t b = i / npix, p = i - b * npix;
    const float s = inv_s[b];
    const float2 du = (ut[i] - u0[i]) * s;
    const float2 vx = vt[(2 * b) * npix + p] * s, vy = vt[(2 * b + 1) * npix + p] * s;
    t[i * 6 + 0] = du.x;
    t[i * 6 + 1] = du.y;
    t[i * 6 + 2] = vx.x;
    t[i * 6 + 3] = vx.y;
    t[i * 6 + 4] = vy.x;
    t[i * 6 + 5] = vy.y;
  }
}

// s[b] = max |u0| over image b; inv_s[b] = 1 / s[b] (1 for an all-zero image). Block per image.
// max |u0| of image blockIdx.y over the pixels of block column blockIdx.x, combined across blocks with an
// integer atomicMax on the float's bits (non-negative floats order like their bit patterns, so the result
// does not depend on the order); image_scale_finish turns the maxima into the scale and its inverse.
__global__ void image_scale_max(const float2* __restrict__ u0, size_t npix, int* __restrict__ imax) {
  __shared__ float sh[256];
  const float2* img = u0 + (size_t)blockIdx.y * npix;
  float m = 0.f;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < npix; i += (size_t)gridDim.x * blockDim.x)
    m = fmaxf(m, sqrtf(abs2(img[i])));
  sh[threadIdx.x] = m;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] = fmaxf(sh[threadIdx.x], sh[threadIdx.x + o]);
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicMax(imax + blockIdx.y, __float_as_int(sh[0]));
}

__global__ void image_scale_finish(const int* __restrict__ imax, int B, float* __restrict__ s,
                                   float* __restrict__ inv_s) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const float m = __int_as_float(imax[b]);
  const float v = m > 0.f ? m : 1.f;
  s[b] = v;
  inv_s[b] = 1.f / v;
}

inline int grid_for(size_t n) { return (int)std::min<size_t>((n + 255) / 256, 4096); }

}  // namespace

// ------------------------------------------------------------------------------------------------
// Host side: parameters, activations for a batch, forward / backward / Adam.
// ------------------------------------------------------------------------------------------------
struct CnnParam {
  int n = 0;          // elements
  DevBuf w, g, m, v;  // FP32 master, gradient, Adam moments
  DevBuf wb;          // BF16 copy used by the tensor-core kernels (null for the SIMT first layer)
};

class WarmStartCnn {
 public:
  static constexpr int kLayers = 8;  // conv_in, 6 hidden, conv_out
  explicit WarmStartCnn(uint64_t seed) {
    std::mt19937_64 gen(seed);
    // conv_in: [9][32][2] + bias 32; hidden: [9][32][32] + 32; conv_out: [9][8][32] + 8
    const int sizes[kLayers] = {NTAP * CH * 2, NTAP * CH * CH, NTAP * CH * CH, NTAP * CH * CH, NTAP * CH * CH,
                                NTAP * CH * CH, NTAP * CH * CH, NTAP * 8 * CH};
    const int fan_in[kLayers] = {NTAP * 2, NTAP * CH, NTAP * CH, NTAP * CH, NTAP * CH, NTAP * CH, NTAP * CH, NTAP * CH};
    const int nb[kLayers] = {CH, CH, CH, CH, CH, CH, CH, 8};
    for (int l = 0; l < kLayers; ++l) {
      std::vector<float> w(sizes[l]);
      // He initialisation; the hidden residual branches start small so the net begins near identity
      const float sd = std::sqrt(2.0f / fan_in[l]) * ((l >= 1 && l <= 6) ? 0.25f : (l == 7 ? 0.1f : 1.0f));
      std::normal_distribution<float> dis(0.f, sd);
      for (auto& x : w) x = dis(gen);
      if (l == 7)  // output channels 6, 7 are padding
        for (int tap = 0; tap < NTAP; ++tap)
          for (int co = 6; co < 8; ++co)
            for (int ci = 0; ci < CH; ++ci) w[((size_t)tap * 8 + co) * CH + ci] = 0.f;
      init_param(W_[l], w, l >= 1);
      init_param(B_[l], std::vector<float>(nb[l], 0.f), false);
    }
    for (auto fn : {conv3x3_tc<EPI_ACC>, conv3x3_tc<EPI_RELU_RES>}) {
      PDT_CUDA_CHECK(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kConvTcSmem));
      // all of the unified L1 / shared storage as shared memory, so that several CTAs fit on an SM
      PDT_CUDA_CHECK(cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
    }
    PDT_CUDA_CHECK(cudaFuncSetAttribute(wgrad_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kWgSmem));
    err_.ensure(sizeof(int));
    PDT_CUDA_CHECK(cudaMemset(err_.p, 0, sizeof(int)));
    int dev = 0;
    PDT_CUDA_CHECK(cudaGetDevice(&dev));
    PDT_CUDA_CHECK(cudaDeviceGetAttribute(&sms_, cudaDevAttrMultiProcessorCount, dev));
    // resident CTAs per SM from the register file, shared memory and thread limits (256-register allocation
    // granules per warp, the per-block shared memory reservation)
    int regs_sm = 0, smem_sm = 0, smem_rsv = 0, thr_sm = 0;
    PDT_CUDA_CHECK(cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev));
    PDT_CUDA_CHECK(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
    PDT_CUDA_CHECK(cudaDeviceGetAttribute(&smem_rsv, cudaDevAttrReservedSharedMemoryPerBlock, dev));
    PDT_CUDA_CHECK(cudaDeviceGetAttribute(&thr_sm, cudaDevAttrMaxThreadsPerMultiProcessor, dev));
    for (auto fn : {conv3x3_tc<EPI_ACC>, conv3x3_tc<EPI_RELU_RES>}) {
      cudaFuncAttributes fa{};
      PDT_CUDA_CHECK(cudaFuncGetAttributes(&fa, fn));
      const int warp_regs = ((fa.numRegs * 32 + 255) / 256) * 256;
      const int by_regs = regs_sm / (warp_regs * (kConvTcThreads / 32));
      const int by_smem = smem_sm / ((int)kConvTcSmem + (int)fa.sharedSizeBytes + smem_rsv);
      const int by_thr = thr_sm / kConvTcThreads;
      conv_tc_per_sm_ = std::min({conv_tc_per_sm_, by_regs, by_smem, by_thr});
    }
    conv_tc_per_sm_ = std::max(conv_tc_per_sm_, 1);
  }

  // Raises (and clears) the error word of the tensor-core convolutions: set when an MMA completion wait
  // gave up, after which that launch's output is not valid.
  void check_error() {
    int e = 0;
    PDT_CUDA_CHECK(cudaMemcpy(&e, err_.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (e) {
      PDT_CUDA_CHECK(cudaMemset(err_.p, 0, sizeof(int)));
      throw Error(PDT_ERR_TIMEOUT, "warm-start network: a tensor-core convolution gave up waiting for its MMAs");
    }
  }

  // Parameters as one flat FP32 vector (weights then biases per layer) for saving / loading.
  std::vector<float> get_params() const {
    std::vector<float> out;
    for (int l = 0; l < kLayers; ++l)
      for (const CnnParam* p : {&W_[l], &B_[l]}) {
        const size_t o = out.size();
        out.resize(o + p->n);
        PDT_CUDA_CHECK(cudaMemcpy(out.data() + o, p->w.p, p->n * sizeof(float), cudaMemcpyDeviceToHost));
      }
    return out;
  }
  void set_params(const float* src, size_t n) {
    size_t o = 0;
    for (int l = 0; l < kLayers; ++l)
      for (CnnParam* p : {&W_[l], &B_[l]}) {
        if (o + p->n > n) throw Error(PDT_ERR_SIZE, "parameter vector too short");
        PDT_CUDA_CHECK(cudaMemcpy(p->w.p, src + o, p->n * sizeof(float), cudaMemcpyHostToDevice));
        if (p->wb.p) refresh_bf16(*p, 0);
        o += p->n;
      }
    if (o != n) throw Error(PDT_ERR_SIZE, "parameter vector length mismatch");
    PDT_CUDA_CHECK(cudaDeviceSynchronize());
  }
  size_t num_params() const {
    size_t n = 0;
    for (int l = 0; l < kLayers; ++l) n += W_[l].n + B_[l].n;
    return n;
  }

  // Forward pass for B images of H x W; u0 complex [B][H][W], s = per-image scale. Writes o (FP32, 8 ch).
  void forward(const float2* u0, const float* inv_s, int B, int H, int W, cudaStream_t st) {
    alloc(B, H, W);
    const size_t npix = (size_t)B * H * W;
    prep_input<<<grid_for(npix), 256, 0, st>>>(u0, inv_s, B, (size_t)H * W, x_.as<float>());
    PDT_LAUNCH_CHECK();
    conv_in_fwd<<<grid_for(npix), 256, 0, st>>>(x_.as<float>(), W_[0].w.as<float>(), B_[0].w.as<float>(), B, H, W,
                                               h_[0].as<bf16>(), z_[0].as<bf16>());
    PDT_LAUNCH_CHECK();
    count_launch(2);
    const dim3 grid((W + TW - 1) / TW, (H + TH - 1) / TH, B);
    const int tgrid = conv_tc_grid(B, H, W);
    for (int l = 1; l <= 6; ++l) {
      conv3x3_tc<EPI_RELU_RES><<<tgrid, kConvTcThreads, kConvTcSmem, st>>>(h_[l - 1].as<bf16>(), W_[l].wb.as<bf16>(),
                                                                         B_[l].w.as<float>(), B, H, W, h_[l].as<bf16>(),
                                                                         z_[l].as<bf16>(), err_.as<int>(), nullptr);
      PDT_LAUNCH_CHECK();
      count_launch();
    }
    conv3x3_mma<CH, 8, EPI_F32><<<grid, 32 * TH, 0, st>>>(h_[6].as<bf16>(), W_[7].wb.as<bf16>(), B_[7].w.as<float>(),
                                                          H, W, o_.as<float>());
    PDT_LAUNCH_CHECK();
    count_launch();
  }

  // Backward pass after forward(): loss = mean over pixels of sum_c (o_c - t_c)^2 (t: 6 channels FP32).
  double backward(const float* target, int B, int H, int W, cudaStream_t st) {
    const size_t npix = (size_t)B * H * W;
    const float scale = 1.0f / (float)npix;
    const int lb = grid_for(npix);
    part_.ensure(sizeof(double) * lb);
    mse_loss<<<lb, 256, 0, st>>>(o_.as<float>(), target, npix, scale, go_.as<bf16>(), part_.as<double>());
    PDT_LAUNCH_CHECK();
    count_launch();
    const dim3 grid((W + TW - 1) / TW, (H + TH - 1) / TH, B);
    const int tgrid = conv_tc_grid(B, H, W);
    // conv_out: dW, db, and dh6 = conv(go, W7') (8 -> 32 channels, padded to 16 input channels)
    wgrad(8, h_[6].as<bf16>(), go_.as<bf16>(), B, H, W, W_[7].g.as<float>(), st);
    bias_gradient(go_.as<bf16>(), npix, 8, B_[7].g.as<float>(), st);
    // go is [npix][8]; the data-gradient kernel needs 16 input channels: pad into go16_
    pad8to16(go_.as<bf16>(), npix, st);
    flip_transpose<<<64, 256, 0, st>>>(W_[7].wb.as<bf16>(), 8, CH, 16, CH, wt_.as<bf16>());
    PDT_LAUNCH_CHECK();
    // the residual stream's FP32 gradient starts as G = dh6 (the BF16 rounding of the convolution's output)
    conv3x3_mma<16, CH, EPI_F32_BF16><<<grid, 32 * TH, 0, st>>>(go16_.as<bf16>(), wt_.as<bf16>(), nullptr, H, W,
                                                                gacc_.as<float>());
    PDT_LAUNCH_CHECK();
    count_launch(3);  // mse_loss, flip_transpose, conv3x3_mma (the bias gradient counts its own)
    for (int l = 6; l >= 1; --l) {
      // h_l = h_{l-1} + relu(z_l), z_l = conv_l(h_{l-1}):  dz = G * relu'(z_l); dh_{l-1} = G + conv_l^T(dz)
      relu_bwd_acc<<<grid_for(npix * CH / 4), 256, 0, st>>>(gacc_.as<float>(), z_[l].as<bf16>(), npix * CH,
                                                             gz_.as<bf16>());
      PDT_LAUNCH_CHECK();
      wgrad(CH, h_[l - 1].as<bf16>(), gz_.as<bf16>(), B, H, W, W_[l].g.as<float>(), st);
      bias_gradient(gz_.as<bf16>(), npix, CH, B_[l].g.as<float>(), st);
      flip_transpose<<<64, 256, 0, st>>>(W_[l].wb.as<bf16>(), CH, CH, CH, CH, wt_.as<bf16>());
      // dh_{l-1} += conv_l^T(dz), added into the FP32 residual gradient in the convolution's epilogue
      conv3x3_tc<EPI_ACC><<<tgrid, kConvTcThreads, kConvTcSmem, st>>>(gz_.as<bf16>(), wt_.as<bf16>(), nullptr, B, H, W,
                                                                    nullptr, nullptr, err_.as<int>(), gacc_.as<float>());
      PDT_LAUNCH_CHECK();
      count_launch(3);  // relu_bwd_acc, flip_transpose, conv3x3_tc
    }
    // conv_in: h1 = relu(z_0): dz0 = G * relu'(z0)
    relu_bwd_acc<<<grid_for(npix * CH / 4), 256, 0, st>>>(gacc_.as<float>(), z_[0].as<bf16>(), npix * CH,
                                                           gz_.as<bf16>());
    {
      const int nb = kPartialBlocksPerSm * sms_;
      bpart_.ensure(sizeof(float) * (size_t)nb * kConvInPartial);
      conv_in_wgrad_partial<<<nb, 32 * kConvInWarps, 0, st>>>(x_.as<float>(), gz_.as<bf16>(), B, H, W,
                                                              bpart_.as<float>());
      sum_partials<<<NTAP * CH * 2, 128, 0, st>>>(bpart_.as<float>(), nb, kConvInPartial, NTAP * CH * 2,
                                                  W_[0].g.as<float>());
      sum_partials<<<CH, 128, 0, st>>>(bpart_.as<float>() + NTAP * CH * 2, nb, kConvInPartial, CH, B_[0].g.as<float>());
      PDT_LAUNCH_CHECK();
    }
    count_launch(4);  // relu_bwd_acc, conv_in_wgrad_partial, two sum_partials
    std::vector<double> h(lb);
    PDT_CUDA_CHECK(cudaMemcpyAsync(h.data(), part_.p, sizeof(double) * lb, cudaMemcpyDeviceToHost, st));
    PDT_CUDA_CHECK(cudaStreamSynchronize(st));
    check_error();
    double loss = 0;
    for (double v : h) loss += v;
    return loss / (double)npix;
  }

  void adam(float lr, cudaStream_t st) {
    ++step_;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float c1 = 1.f - std::pow(b1, (float)step_), c2 = 1.f - std::pow(b2, (float)step_);
    for (int l = 0; l < kLayers; ++l)
      for (CnnParam* p : {&W_[l], &B_[l]}) {
        adam_step<<<grid_for(p->n), 256, 0, st>>>(p->w.as<float>(), p->g.as<float>(), p->m.as<float>(),
                                                  p->v.as<float>(), p->n, lr, b1, b2, eps, c1, c2,
                                                  p->wb.p ? p->wb.as<bf16>() : nullptr);
        PDT_LAUNCH_CHECK();
        count_launch();
      }
  }

  const float* output() const { return o_.as<float>(); }
  // per-image scales of u0 (device): s, 1/s
  void scales(const float2* u0, int B, size_t npix_img, cudaStream_t st) {
    sc_.ensure(3 * sizeof(float) * std::max(B, 1));  // scale [B], inverse [B], maxima as int bits [B]
    int* imax = reinterpret_cast<int*>(sc_.as<float>() + 2 * B);
    PDT_CUDA_CHECK(cudaMemsetAsync(imax, 0, sizeof(int) * B, st));
    const int nbx = (int)std::max<size_t>(1, std::min<size_t>((npix_img + 255) / 256, (size_t)sms_));
    image_scale_max<<<dim3(nbx, B), 256, 0, st>>>(u0, npix_img, imax);
    image_scale_finish<<<(B + 127) / 128, 128, 0, st>>>(imax, B, sc_.as<float>(), sc_.as<float>() + B);
    PDT_LAUNCH_CHECK();
    count_launch(2);
  }
  const float* scale_ptr() const { return sc_.as<float>(); }
  const float* inv_scale_ptr(int B) const { return sc_.as<float>() + B; }
  std::vector<float> get_grads() const {
    std::vector<float> out;
    for (int l = 0; l < kLayers; ++l)
      for (const CnnParam* p : {&W_[l], &B_[l]}) {
        const size_t o = out.size();
        out.resize(o + p->n);
        PDT_CUDA_CHECK(cudaMemcpy(out.data() + o, p->g.p, p->n * sizeof(float), cudaMemcpyDeviceToHost));
      }
    return out;
  }
  float* target_buf(size_t npix) {
    t_.ensure(npix * 6 * sizeof(float));
    return t_.as<float>();
  }

  void make_target(const float2* u0, const float2* ut, const float2* vt, const float* inv_s, int B, size_t npix_img,
                   cudaStream_t st) {
    float* t = target_buf((size_t)B * npix_img);
    prep_target<<<grid_for((size_t)B * npix_img), 256, 0, st>>>(u0, ut, vt, inv_s, B, npix_img, t);
    PDT_LAUNCH_CHECK();
    count_launch();
  }
  void assemble(const float2* u0, const float* s, int B, size_t npix_img, float2* u, float2* v, cudaStream_t st) {
    assemble_output<<<grid_for((size_t)B * npix_img), 256, 0, st>>>(u0, o_.as<float>(), s, B, npix_img, u, v);
    PDT_LAUNCH_CHECK();
    count_launch();
  }

 private:
  void init_param(CnnParam& p, const std::vector<float>& w, bool bf) {
    p.n = (int)w.size();
    p.w.ensure(w.size() * sizeof(float));
    p.g.ensure(w.size() * sizeof(float));
    p.m.ensure(w.size() * sizeof(float));
    p.v.ensure(w.size() * sizeof(float));
    PDT_CUDA_CHECK(cudaMemcpy(p.w.p, w.data(), w.size() * sizeof(float), cudaMemcpyHostToDevice));
    PDT_CUDA_CHECK(cudaMemset(p.g.p, 0, p.g.bytes));
    PDT_CUDA_CHECK(cudaMemset(p.m.p, 0, p.m.bytes));
    PDT_CUDA_CHECK(cudaMemset(p.v.p, 0, p.v.bytes));
    if (bf) {
      p.wb.ensure(w.size() * sizeof(bf16));
      refresh_bf16(p, 0);
    }
  }
  // persistent tensor-core convolutions: three CTAs per SM (66 KB of shared memory each), at most one tile each
  int conv_tc_grid(int B, int H, int W) const {
    const long long tiles = (long long)((W + kConvTcTW - 1) / kConvTcTW) * ((H + kConvTcTH - 1) / kConvTcTH) * B;
    return (int)std::min<long long>(tiles, (long long)conv_tc_per_sm_ * sms_);
  }
  void refresh_bf16(CnnParam& p, cudaStream_t st) {
    to_bf16<<<grid_for(p.n), 256, 0, st>>>(p.w.as<float>(), p.n, p.wb.as<bf16>());
    PDT_LAUNCH_CHECK();
  }
  void alloc(int B, int H, int W) {
    if (B == B_n_ && H == H_n_ && W == W_n_) return;
    const size_t npix = (size_t)B * H * W;
    x_.ensure(npix * 2 * sizeof(float));
    for (int l = 0; l < 7; ++l) {
      h_[l].ensure(npix * CH * sizeof(bf16));
      z_[l].ensure(npix * CH * sizeof(bf16));
    }
    o_.ensure(npix * 8 * sizeof(float));
    go_.ensure(npix * 8 * sizeof(bf16));
    go16_.ensure(npix * 16 * sizeof(bf16));
    gz_.ensure(npix * CH * sizeof(bf16));
    gacc_.ensure(npix * CH * sizeof(float));
    wt_.ensure(NTAP * CH * CH * sizeof(bf16));
    B_n_ = B;
    H_n_ = H;
    W_n_ = W;
  }
  void pad8to16(const bf16* g8, size_t npix, cudaStream_t st) {
    PDT_CUDA_CHECK(cudaMemsetAsync(go16_.p, 0, npix * 16 * sizeof(bf16), st));
    PDT_CUDA_CHECK(cudaMemcpy2DAsync(go16_.p, 16 * sizeof(bf16), g8, 8 * sizeof(bf16), 8 * sizeof(bf16), npix,
                                     cudaMemcpyDeviceToDevice, st));
  }
  void wgrad(int cout, const bf16* x, const bf16* dy, int B, int H, int W, float* grad, cudaStream_t st) {
    int sms = 0, dev = 0;
    PDT_CUDA_CHECK(cudaGetDevice(&dev));
    PDT_CUDA_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int tiles = B * ((W + TW - 1) / TW) * ((H + TH - 1) / TH);
    // the tensor-core kernel: three persistent CTAs per SM (128 TMEM columns, 50 KB shared memory each)
    const int nb = std::max(1, std::min(sms * (cout == CH ? 3 : 2), tiles));
    const int n = NTAP * cout * CH;
    wpart_.ensure((size_t)std::max(1, std::min(sms * 3, tiles)) * NTAP * CH * CH * sizeof(float));
    if (cout == CH)
      wgrad_tc<<<nb, kWgThreads, kWgSmem, st>>>(x, dy, B, H, W, wpart_.as<float>(), err_.as<int>());
    else
      wgrad_mma<8><<<nb, 32 * NTAP, 0, st>>>(x, dy, B, H, W, wpart_.as<float>());
    PDT_LAUNCH_CHECK();
    wtmp_.ensure(sizeof(float) * (size_t)kWgRanges * NTAP * CH * CH);
    wgrad_reduce_ranges<<<dim3((n + 255) / 256, kWgRanges), 256, 0, st>>>(wpart_.as<float>(), nb, n, wtmp_.as<float>());
    wgrad_reduce<<<grid_for(n), 256, 0, st>>>(wtmp_.as<float>(), kWgRanges, n, grad);
    PDT_LAUNCH_CHECK();
    count_launch(3);
  }

  CnnParam W_[kLayers], B_[kLayers];
  DevBuf x_, h_[7], z_[7], o_, go_, go16_, gz_, gacc_, wt_, wpart_, part_, t_, sc_, err_, bpart_, wtmp_;

  // Bias gradient db[c] = sum over pixels of dy[p][c] (C = 8 or 32): chunked partial sums, then the
  // partials in block order.
  void bias_gradient(const bf16* dy, size_t npix, int C, float* db, cudaStream_t st) {
    const int nb = 2 * sms_;
    bpart_.ensure(sizeof(float) * (size_t)kPartialBlocksPerSm * sms_ * kConvInPartial);
    if (C == 8)
      bias_grad_partial<8><<<nb, 256, 0, st>>>(dy, npix, bpart_.as<float>());
    else
      bias_grad_partial<CH><<<nb, 256, 0, st>>>(dy, npix, bpart_.as<float>());
    sum_partials<<<C, 128, 0, st>>>(bpart_.as<float>(), nb, C, C, db);
    PDT_LAUNCH_CHECK();
    count_launch(2);
  }
  int sms_ = 1;
  int conv_tc_per_sm_ = 8;  // resident conv3x3_tc CTAs per SM (each holds 32 TMEM columns: 8 x 32 <= 512)
  int B_n_ = 0, H_n_ = 0, W_n_ = 0;
  long step_ = 0;
};

void cnn_set_drop_arrival(int on) { PDT_CUDA_CHECK(tc::set_drop_arrival(on)); }

}  // namespace pdt

// ==================================================================================================
// C ABI of the warm-start network
// ==================================================================================================
struct pdt_cnn {
  std::unique_ptr<pdt::WarmStartCnn> impl;
};

namespace {
template <class F>
pdt_status cnn_guard(F&& fn) {
  try {
    fn();
    return PDT_OK;
  } catch (const pdt::Error& e) {
    pdt::set_last_error(e.what());
    return e.code;
  } catch (const std::exception& e) {
    pdt::set_last_error(e.what());
    return PDT_ERR_INVALID_ARGUMENT;
  }
}
void cnn_check(pdt_cnn* c, int B, int H, int W) {
  if (!c) throw pdt::Error(PDT_ERR_INVALID_ARGUMENT, "null network");
  if (B < 1 || H < 1 || W < 1) throw pdt::Error(PDT_ERR_INVALID_ARGUMENT, "B, H and W must be positive");
}
}  // namespace

extern "C" {

pdt_status pdt_cnn_create(uint64_t seed, pdt_cnn** out) {
  return cnn_guard([&] {
    if (!out) throw pdt::Error(PDT_ERR_INVALID_ARGUMENT, "null out");
    auto h = std::make_unique<pdt_cnn>();
    h->impl = std::make_unique<pdt::WarmStartCnn>(seed);
    *out = h.release();
  });
}

pdt_status pdt_cnn_destroy(pdt_cnn* c) {
  return cnn_guard([&] { delete c; });
}

pdt_status pdt_cnn_num_params(pdt_cnn* c, size_t* n) {
  return cnn_guard([&] {
    cnn_check(c, 1, 1, 1);
    *n = c->impl->num_params();
  });
}

pdt_status pdt_cnn_get_params(pdt_cnn* c, float* dst, size_t n) {
  return cnn_guard([&] {
    cnn_check(c, 1, 1, 1);
    auto v = c->impl->get_params();
    if (n != v.size()) throw pdt::Error(PDT_ERR_SIZE, "parameter count mismatch");
    std::memcpy(dst, v.data(), n * sizeof(float));
  });
}

pdt_status pdt_cnn_set_params(pdt_cnn* c, const float* src, size_t n) {
  return cnn_guard([&] {
    cnn_check(c, 1, 1, 1);
    c->impl->set_params(src, n);
  });
}

pdt_status pdt_cnn_get_grads(pdt_cnn* c, float* dst, size_t n) {
  return cnn_guard([&] {
    cnn_check(c, 1, 1, 1);
    auto v = c->impl->get_grads();
    if (n != v.size()) throw pdt::Error(PDT_ERR_SIZE, "parameter count mismatch");
    std::memcpy(dst, v.data(), n * sizeof(float));
  });
}

pdt_status pdt_cnn_train_step(pdt_cnn* c, const void* u0, const void* ut, const void* vt, int B, int H, int W,
                              float lr, void* stream, double* loss) {
  return cnn_guard([&] {
    cnn_check(c, B, H, W);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    auto& n = *c->impl;
    const size_t np = (size_t)H * W;
    n.scales(static_cast<const float2*>(u0), B, np, st);
    n.make_target(static_cast<const float2*>(u0), static_cast<const float2*>(ut), static_cast<const float2*>(vt),
                  n.inv_scale_ptr(B), B, np, st);
    n.forward(static_cast<const float2*>(u0), n.inv_scale_ptr(B), B, H, W, st);
    const double l = n.backward(n.target_buf((size_t)B * np), B, H, W, st);
    if (lr > 0.f) n.adam(lr, st);
    if (loss) *loss = l;
  });
}

pdt_status pdt_cnn_predict(pdt_cnn* c, const void* u0, int B, int H, int W, void* u, void* v, void* stream) {
  return cnn_guard([&] {
    cnn_check(c, B, H, W);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    auto& n = *c->impl;
    const size_t np = (size_t)H * W;
    n.scales(static_cast<const float2*>(u0), B, np, st);
    n.forward(static_cast<const float2*>(u0), n.inv_scale_ptr(B), B, H, W, st);
    n.assemble(static_cast<const float2*>(u0), n.scale_ptr(), B, np, static_cast<float2*>(u), static_cast<float2*>(v),
               st);
    if (!stream) {
      PDT_CUDA_CHECK(cudaStreamSynchronize(st));
      n.check_error();
    }
  });
}

}  // extern "C"
