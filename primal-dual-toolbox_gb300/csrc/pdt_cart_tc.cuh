// pdt_cart_tc.cuh -- the row passes of the Cartesian operator as pruned DFTs on the tensor cores.
//
// Along W only the ns sampled phase-encode columns are needed (forward output, adjoint input), so the
// row transforms are pruned DFTs. With the shift index maps of the FFT kernels folded in:
//   forward  t1[c][s][y] = sum_x (ubar . sens_c)[y][x] w^(q(x) f_s),   q(x)  = (x + mid_W) mod W
//   adjoint  g_c[y][x]   = sum_s t2[c][s][y] w^(-p_s q'(x)),           q'(x) = (x - W/2) mod W
// with w = exp(-2 pi i / W), f_s the forward-FFT output slot and p_s the inverse-FFT input slot of
// sampled column s (the same maps as rows_fwd_kernel / rows_adj_kernel). Both are complex GEMMs over the
// rows (c, y), flattened to M = C Hi and cut into tiles of 128 (the tensor-memory lanes). A complex
// product becomes a real one by interleaving re/im along K and expanding the DFT factor e into the 2 x 2
// block [[Re e, -Im e], [Im e, Re e]] along (N, K), so D[row][2 j + o] is part o of output j.
//
// Operands are TF32 hi/lo pairs in 128-byte-swizzled K-major tiles; one thread issues three kind::tf32
// MMAs per K step (hi.hi + hi.lo + lo.hi, FP32 accumulate in tensor memory) and commits them to the
// stage's mbarrier.
//
//   tc_rows_adj  grid (N ranges, row tiles). Both operands arrive by bulk copy (cp.async.bulk): the data
//                tiles as the column kernel wrote them, the DFT factor from tiles precomputed per operator.
//                A row tile holds a few image rows of every coil, and each CTA writes the coil sum
//                sum_c conj(sens_c) . g_c of its rows and output columns (coil order: deterministic).
//   tc_rows_fwd  grid (row tiles, KS, s tiles), clusters of (1, KS, 1). The threads stage the data operand
//                (ubar . sens_c, split) and generate the DFT factor from the twiddle table; the KS CTAs of
//                a cluster take disjoint K (x) ranges and reduce their accumulators through distributed
//                shared memory in rank order (deterministic) before writing t1.
#pragma once

#include <cooperative_groups.h>

#include "pdt_tc.cuh"

namespace pdt {
namespace {

constexpr int kTcThreads = 256;
constexpr int kTcRows = 128;
constexpr uint32_t kTcTmemCols = 256;
constexpr uint32_t kTcTileA = 128 * 128;  // bytes of one 128-row x 32-element FP32 tile
constexpr int kTcMaxW = 1024;             // twiddle table and index products (< 2^20) sized for this
constexpr int kTcMaxStages = 4;

__device__ __forceinline__ unsigned char* tc_align1024(unsigned char* raw) {
  const uint32_t off = tc::smem_addr(raw);
  return raw + ((1024u - (off & 1023u)) & 1023u);
}

// (a b) mod W for 0 <= a, b < W <= 1024: the product is exact in FP32, the quotient estimate is off by
// at most one and corrected.
__device__ __forceinline__ int tc_mod_mul(int a, int b, int W, float invW) {
  const int p = a * b;
  const int q = __float2int_rz(__int2float_rn(p) * invW);
  int m = p - q * W;
  if (m < 0) m += W;
  if (m >= W) m -= W;
  return m;
}

__device__ __forceinline__ float4 tc_cmul2(float4 a, float4 b) {
  return make_float4(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x, a.z * b.z - a.w * b.w, a.z * b.w + a.w * b.z);
}
__device__ __forceinline__ float4 tc_cmulc2(float4 a, float4 b) {  // a . conj(b), two complex values
  return make_float4(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y, a.z * b.z + a.w * b.w, a.w * b.z - a.z * b.w);
}

// Stage layout in shared memory (bytes from the 1024-aligned base): [A hi | A lo | B hi | B lo] per
// stage, two stages, then the kernel's tables.
__host__ __device__ inline uint32_t tc_stage_bytes(int nbmax) { return 2 * kTcTileA + 2u * (uint32_t)nbmax * 128u; }
inline size_t tc_adj_smem(int NB, int nst) { return 1024 + (size_t)nst * tc_stage_bytes(NB) + 16 * kTcMaxStages + 32; }
inline size_t tc_fwd_smem(int W, int nb) { return 1024 + 2 * (size_t)tc_stage_bytes(nb) + 8 * (size_t)W + 4 * 128 + 64; }

// Issues the MMAs of one staged K chunk (ksteps <= 4 steps of K = 8) and commits them to `bar`.
__device__ __forceinline__ void tc_issue_chunk(uint32_t tmem, uint32_t a_hi, uint32_t a_lo, uint32_t b_hi,
                                               uint32_t b_lo, int ksteps, uint32_t idesc, bool first, uint64_t* bar) {
  tc::fence_after_sync();
#pragma unroll 1
  for (int k = 0; k < ksteps; ++k) {
    const uint32_t o = 32u * (uint32_t)k;
    tc::mma_tf32(tmem, tc::desc_sw128(a_hi + o), tc::desc_sw128(b_hi + o), idesc, (first && k == 0) ? 0u : 1u);
    tc::mma_tf32(tmem, tc::desc_sw128(a_hi + o), tc::desc_sw128(b_lo + o), idesc, 1u);
    tc::mma_tf32(tmem, tc::desc_sw128(a_lo + o), tc::desc_sw128(b_hi + o), idesc, 1u);
  }
  tc::mma_commit(bar);
}

// ------------------------------------------------------------------------------------------------
// Adjoint rows and coil combination: out[y][x] = sum_c conj(sens_c[y0 + y][x]) sum_s t2[c][s][y] w^(-p_s q'(x)).
// K = 2 ns (s, re/im); N = 2 W (x, re/im) cut into ranges of NB; M: a tile holds yb image rows of all
// C coils (row m = c yb + yl), so that the coil sum stays inside the CTA and one image is written.
// Both operands arrive by bulk copy: the data tiles as the column kernel wrote them (tc_put_a), the DFT
// factor from the operator's precomputed tiles. Thread 0 copies, thread 32 issues the MMAs; the
// epilogue (1) moves TMEM lanes 32 q .. + 31 (warps q, q + 4, ...: one row per thread, column groups of
// 8) to shared memory, (2) sums the coils: item (yl, four real columns) per thread, coalesced along x.
// `nst` stages of [A hi | A lo | B hi | B lo].
// ------------------------------------------------------------------------------------------------
constexpr int kTcAdjThreads = 512;  // 16 warps
constexpr int kTcAdjMaxNB = 256;    // output columns (re/im) per CTA
constexpr int kTcCoilUnroll = 16;   // coil-sum loads issued together

template <bool SENS>
__global__ void __launch_bounds__(kTcAdjThreads, 1) tc_rows_adj(CartDev d, const float* __restrict__ atiles,
                                                             const unsigned char* __restrict__ btiles,
                                                             float2* __restrict__ out, int NB, int nst,
                                                             int* __restrict__ err) {
  extern __shared__ unsigned char tc_smem_raw[];
  unsigned char* sm = tc_align1024(tc_smem_raw);
  const int W = d.W, ns = d.ns, Hi = d.Hi, C = d.C, yb = d.tc_yb;
  const uint32_t stage_bytes = tc_stage_bytes(NB);
  uint64_t* full = reinterpret_cast<uint64_t*>(sm + nst * stage_bytes);  // copies of a stage landed
  uint64_t* empty = full + kTcMaxStages;                                  // MMAs of a stage done
  uint64_t* accb = empty + kTcMaxStages;                                  // every MMA done (one phase)
  uint32_t* tslot = reinterpret_cast<uint32_t*>(accb + 1);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int n0 = blockIdx.x * NB;
  const int nb = min(NB, (2 * W - n0 + 15) & ~15);
  const int T = blockIdx.y, ybase = T * yb;
  const int K = 2 * ns;
  const int nch = (K + 31) >> 5;
  const int F4 = nb >> 2;  // float4 groups (two outputs) per row

  if (tid == 0) {
    for (int i = 0; i < nst; ++i) {
      tc::mbar_init(&full[i], 1);
      tc::mbar_init(&empty[i], 1);
    }
    tc::mbar_init(accb, 1);
    tc::fence_mbar_init();
  }
  if (warp == 0) tc::tmem_alloc(tslot, kTcTmemCols);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;

  const uint32_t base = tc::smem_addr(sm);
  const uint32_t bbytes = 2u * (uint32_t)nb * 128u;
  const unsigned char* bsrc = btiles + (size_t)blockIdx.x * nch * 2 * NB * 128;
  const int pre = min(nst, nch);
  if (tid == 0) {  // the DFT-factor tiles are constants: their first copies start before the column kernel ends
    for (int j = 0; j < pre; ++j) {
      tc::mbar_arrive_expect_tx(&full[j], 2 * kTcTileA + bbytes);
      tc::bulk_g2s(base + j * stage_bytes + 2 * kTcTileA, bsrc + (size_t)j * 2 * NB * 128, bbytes, &full[j]);
    }
  }
  pdl_wait();  // every thread: the data tiles come from the column kernel

  bool ok = true;
  if (tid == 0) {
    const float* asrc = atiles + (size_t)T * nch * (2 * 128 * 32);
    tc::fence_async_global();
    for (int j = 0; j < pre; ++j)
      tc::bulk_g2s(base + j * stage_bytes, asrc + (size_t)j * (2 * 128 * 32), 2 * kTcTileA, &full[j]);
    for (int j = pre; j < nch && ok; ++j) {
      const int b = j % nst;
      ok = tc::mbar_wait(&empty[b], ((j / nst) - 1) & 1);  // the MMAs of chunk j - nst are done
      if (!ok) {
        atomicCAS(err, 0, 0x100 | j);  // the copy thread gave up at chunk j
        break;
      }
      const uint32_t dst = base + b * stage_bytes;
      tc::mbar_arrive_expect_tx(&full[b], 2 * kTcTileA + bbytes);
      tc::bulk_g2s(dst, asrc + (size_t)j * (2 * 128 * 32), 2 * kTcTileA, &full[b]);
      tc::bulk_g2s(dst + 2 * kTcTileA, bsrc + (size_t)j * 2 * NB * 128, bbytes, &full[b]);
    }
  } else if (tid == 32) {
    const uint32_t idesc = tc::idesc_tf32(kTcRows, nb);
    for (int j = 0; j < nch && ok; ++j) {
      const int b = j % nst;
      ok = tc::mbar_wait(&full[b], (j / nst) & 1);
      if (!ok) {
        atomicCAS(err, 0, 0x200 | j);  // the MMA thread gave up waiting for chunk j's copies
        break;
      }
      const uint32_t a_hi = base + b * stage_bytes, a_lo = a_hi + kTcTileA;
      const uint32_t b_hi = a_lo + kTcTileA, b_lo = b_hi + (uint32_t)nb * 128u;
      tc_issue_chunk(tmem, a_hi, a_lo, b_hi, b_lo, min(4, (K - 32 * j + 7) >> 3), idesc, j == 0, &empty[b]);
    }
    tc::mma_commit(accb);  // also after a timeout
    // a single-phase barrier (the stage barriers run through several phases, and a parity wait only
    // distinguishes the current phase from the one before it); the other threads wait in the block
    // barrier below without taking issue slots
    if (!tc::mbar_wait(accb, 0)) {
      atomicCAS(err, 0, 0x300);  // the MMAs did not complete
      ok = false;
    }
    tc::fence_before_sync();
  }

  // coil-map values of this thread's first output item: the other threads load them while the MMAs run
  const int yrows = min(yb, Hi - ybase);  // image rows of this tile
  const int nitems = yrows * F4;
  float4 sv[kTcCoilUnroll];
  {
    const int yl = tid / F4, f = tid - yl * F4;
    const int x = (n0 >> 1) + 2 * f;  // even; W even, so x + 1 < W as well
    const bool iv = tid < nitems && x < W;
#pragma unroll
    for (int c = 0; c < kTcCoilUnroll; ++c) {
      sv[c] = make_float4(1.f, 0.f, 1.f, 0.f);
      if (SENS && iv && c < C)
        sv[c] = *reinterpret_cast<const float4*>(d.sens + ((size_t)c * d.Hf + ybase + yl + d.y0) * W + x);
    }
  }
  const bool done = __syncthreads_and(ok);
  tc::fence_after_sync();
  float* dt = reinterpret_cast<float*>(sm);  // the stage buffers are free: every MMA has completed
  const int ld = nb + 4;                      // row stride: 16-byte row-per-thread stores conflict-free
  if (done) {
    const int q = warp & 3, h = warp >> 2;
    const int G8 = nb >> 3, gb = h * G8 / 4, ge = (h + 1) * G8 / 4;
    const uint32_t taddr = tmem + ((uint32_t)(32 * q) << 16);
    float* drow = dt + (size_t)(32 * q + lane) * ld;
    for (int g = gb; g < ge; ++g) {  // warp-uniform bounds
      float v[8];
      tc::tmem_ld8(taddr + (uint32_t)(8 * g), v);
      *reinterpret_cast<float4*>(drow + 8 * g) = make_float4(v[0], v[1], v[2], v[3]);
      *reinterpret_cast<float4*>(drow + 8 * g + 4) = make_float4(v[4], v[5], v[6], v[7]);
    }
  }
  __syncthreads();
  if (done) {
    for (int i = tid; i < nitems; i += kTcAdjThreads) {
      const int yl = i / F4, f = i - yl * F4;
      const int x = (n0 >> 1) + 2 * f;
      if (x >= W) continue;
      const int y = ybase + yl;
      const float* drow = dt + (size_t)yl * ld + 4 * f;  // row c yb + yl of coil c
      const float2* srow = d.sens + ((size_t)y + d.y0) * W + x;  // coil c at + c Hf W
      const size_t sstride = (size_t)d.Hf * W;
      float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
      auto add = [&](int c, float4 sc) {
        const float4 v = *reinterpret_cast<const float4*>(drow + (size_t)c * yb * ld);
        const float4 p = SENS ? tc_cmulc2(v, sc) : v;  // D . conj(sens_c) for two outputs
        acc.x += p.x;
        acc.y += p.y;
        acc.z += p.z;
        acc.w += p.w;
      };
      if (i == tid) {  // this thread's first item: the coil-map values of the first coils are loaded
#pragma unroll
        for (int c = 0; c < kTcCoilUnroll; ++c)
          if (c < C) add(c, sv[c]);
      } else {
        float4 s4[kTcCoilUnroll];
#pragma unroll
        for (int c = 0; c < kTcCoilUnroll; ++c)
          s4[c] = (SENS && c < C) ? *reinterpret_cast<const float4*>(srow + c * sstride) : make_float4(1.f, 0.f, 1.f, 0.f);
#pragma unroll
        for (int c = 0; c < kTcCoilUnroll; ++c)
          if (c < C) add(c, s4[c]);
      }
      for (int c = kTcCoilUnroll; c < C; ++c)
        add(c, SENS ? *reinterpret_cast<const float4*>(srow + c * sstride) : make_float4(1.f, 0.f, 1.f, 0.f));
      *reinterpret_cast<float4*>(out + (size_t)y * W + x) = acc;  // coils summed in coil order
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, kTcTmemCols);
  }
}

// ------------------------------------------------------------------------------------------------
// Forward rows: t1[c][s][y] = sum_x (ubar . sens_c)[y][x] w^(q(x) f_s) for the 128 sampled columns of
// s tile blockIdx.z. K = 2 W (x, re/im) split over the KS CTAs of a cluster; N = 2 (s, re/im) <= 256.
// ------------------------------------------------------------------------------------------------
template <bool SENS>
__global__ void __launch_bounds__(kTcThreads, 1) tc_rows_fwd(CartDev d, const float2* __restrict__ ubar,
                                                             float2* __restrict__ t1, int* __restrict__ tick,
                                                             int* __restrict__ err) {
  namespace cg = cooperative_groups;
  extern __shared__ unsigned char tc_smem_raw[];
  unsigned char* sm = tc_align1024(tc_smem_raw);
  const int W = d.W, ns = d.ns, Hi = d.Hi;
  const int s0 = blockIdx.z * 128, nsl = min(128, ns - s0);
  const int nb = (2 * nsl + 15) & ~15;
  const uint32_t stage_bytes = tc_stage_bytes(nb);
  float2* tw = reinterpret_cast<float2*>(sm + 2 * stage_bytes);
  int* fs = reinterpret_cast<int*>(tw + W);
  uint64_t* bars = reinterpret_cast<uint64_t*>((reinterpret_cast<uintptr_t>(fs + 128) + 15) & ~(uintptr_t)15);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 2);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int R = d.C * Hi;
  const int r0 = blockIdx.x * kTcRows;
  const int KS = gridDim.y, ks = blockIdx.y;
  const int K = 2 * W;
  const int nchT = (K + 31) >> 5;
  const int jb = ks * nchT / KS, je = (ks + 1) * nchT / KS;
  const float invW = 1.0f / (float)W;

  if (tid == 0) {
    tc::mbar_init(&bars[0], 1);
    tc::mbar_init(&bars[1], 1);
    tc::fence_mbar_init();
  }
  if (warp == 0) tc::tmem_alloc(tslot, kTcTmemCols);
  for (int i = tid; i < W; i += kTcThreads) tw[i] = d.twW[i];
  for (int i = tid; i < nsl; i += kTcThreads) fs[i] = d.fwd_slot[s0 + i];
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;
  pdl_wait();  // ubar comes from the previous kernel; t1 may still be read by it
  if (tick && blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && tid == 0) atomicAdd(tick, 1);

  const uint32_t base = tc::smem_addr(sm);
  const uint32_t idesc = tc::idesc_tf32(kTcRows, nb);
  int issued = 0;
  bool good = true;
  for (int j = jb; j < je; ++j) {
    const int jl = j - jb, b = jl & 1;
    const uint32_t a_hi = base + b * stage_bytes, a_lo = a_hi + kTcTileA;
    const uint32_t b_hi = a_lo + kTcTileA, b_lo = b_hi + (uint32_t)nb * 128u;
    bool ok = jl < 2 || tc::mbar_wait(&bars[b], ((jl >> 1) - 1) & 1);
    const int x0 = 16 * j;
    // A: rows (c, y) x 16 image columns (re, im) of ubar . sens_c; 8 threads cover one row's 128 bytes
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int it = tid + kTcThreads * i;
      const int p = it & 7, row = it >> 3;
      const int r = r0 + row, x = x0 + 2 * p;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (r < R && x < W) {  // x even and W even: x + 1 < W
        const int c = r / Hi, y = r - c * Hi;
        v = *reinterpret_cast<const float4*>(ubar + (size_t)y * W + x);
        if (SENS) v = tc_cmul2(v, *reinterpret_cast<const float4*>(d.sens + ((size_t)c * d.Hf + y + d.y0) * W + x));
      }
      float4 hi, lo;
      tc::split4(v, hi, lo);
      const uint32_t o = tc::sw128(row, p);
      tc::st_shared4(a_hi + o, hi);
      tc::st_shared4(a_lo + o, lo);
    }
    // B: output columns (s, re/im) x the same 16 image columns, from the twiddles
    const int nitems = (nb >> 1) * 8;
    for (int it = tid; it < nitems; it += kTcThreads) {
      const int p = it & 7, sl = it >> 3;
      const int x = x0 + 2 * p;
      float2 e0 = c2(0.f, 0.f), e1 = c2(0.f, 0.f);
      if (sl < nsl && x < W) {
        const int f = fs[sl];
        int q = x + d.mxW;
        if (q >= W) q -= W;
        e0 = tw[tc_mod_mul(q, f, W, invW)];
        if (++q == W) q = 0;
        e1 = tw[tc_mod_mul(q, f, W, invW)];
      }
      float4 hi, lo;
      tc::split4(make_float4(e0.x, -e0.y, e1.x, -e1.y), hi, lo);
      uint32_t o = tc::sw128(2 * sl, p);
      tc::st_shared4(b_hi + o, hi);
      tc::st_shared4(b_lo + o, lo);
      tc::split4(make_float4(e0.y, e0.x, e1.y, e1.x), hi, lo);
      o = tc::sw128(2 * sl + 1, p);
      tc::st_shared4(b_hi + o, hi);
      tc::st_shared4(b_lo + o, lo);
    }
    tc::fence_async_smem();
    if (!__syncthreads_and(ok)) {
      good = false;
      break;
    }
    if (tid == 0) tc_issue_chunk(tmem, a_hi, a_lo, b_hi, b_lo, min(4, (K - 32 * j + 7) >> 3), idesc, jl == 0, &bars[b]);
    ++issued;
  }
  bool done = issued > 0 && tc::mbar_wait(&bars[(issued - 1) & 1], ((issued - 1) >> 1) & 1);
  done = __syncthreads_and(done) && good;
  tc::fence_after_sync();
  const int q = warp & 3, h = warp >> 2;
  const int half = nb >> 1;  // a multiple of 8
  const int row = 32 * q + lane, r = r0 + row;
  const bool rv = r < R;
  const uint32_t taddr = tmem + ((uint32_t)(32 * q) << 16);
  if (KS == 1) {
    if (done) {
      const int c = rv ? r / Hi : 0, y = rv ? r - c * Hi : 0;
      float2* out = t1 + ((size_t)c * ns + s0) * Hi + y;
      for (int col = h * half; col < (h + 1) * half; col += 8) {
        float v[8];
        tc::tmem_ld8(taddr + (uint32_t)col, v);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int sl = (col >> 1) + i;
          if (rv && sl < nsl) out[(size_t)sl * Hi] = c2(v[2 * i], v[2 * i + 1]);
        }
      }
    }
  } else {
    // accumulator -> shared memory red[sl][row] (the stage buffers are free: every MMA has completed)
    float2* red = reinterpret_cast<float2*>(sm);
    if (done) {
      for (int col = h * half; col < (h + 1) * half; col += 8) {
        float v[8];
        tc::tmem_ld8(taddr + (uint32_t)col, v);
#pragma unroll
        for (int i = 0; i < 4; ++i) red[((col >> 1) + i) * kTcRows + row] = c2(v[2 * i], v[2 * i + 1]);
      }
    }
    cg::cluster_group cluster = cg::this_cluster();
    const int anybad = __syncthreads_or(!done);
    cluster.sync();  // every CTA's partial sums are in its shared memory (executed by all CTAs)
    const int sb = ks * nsl / KS, se = (ks + 1) * nsl / KS;
    if (!anybad) {
      for (int i = tid; i < (se - sb) * kTcRows; i += kTcThreads) {
        const int rr = i & (kTcRows - 1), sl = sb + (i >> 7);
        float2 acc = c2(0.f, 0.f);
        for (int qq = 0; qq < KS; ++qq) acc += cluster.map_shared_rank(red, qq)[sl * kTcRows + rr];  // rank order
        const int rg = r0 + rr;
        if (rg < R) {
          const int c = rg / Hi, y = rg - c * Hi;
          t1[((size_t)c * ns + s0 + sl) * Hi + y] = acc;
        }
      }
    }
    cluster.sync();  // keep this CTA's shared memory alive until the other CTAs have read it
  }
  if (!done && tid == 0) atomicExch(err, 2);
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, kTcTmemCols);
  }
}

}  // namespace
}  // namespace pdt
