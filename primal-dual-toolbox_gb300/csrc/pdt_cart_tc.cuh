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
//   tc_rows_adj  grid (N ranges, row tiles). The DFT factor arrives by bulk copy (cp.async.bulk) from
//                tiles precomputed per operator; the threads stage the data operand from t2. A row tile
//                holds a few image rows of every coil, and each CTA writes the coil sum
//                sum_c conj(sens_c) . g_c of its rows and output columns (coil order: deterministic).
//                Rows of blocks past the row tiles, when the launch has them, run the solver's dual
//                update on the SMs the row tiles leave free.
//   tc_rows_fwd  grid (row tiles, KS, s tiles), clusters of (1, KS, 1). The DFT factor arrives by bulk
//                copy, the threads form the data operand (ubar . sens_c, split); the KS CTAs of a cluster
//                take disjoint K (x) ranges and reduce their accumulators through distributed shared
//                memory in rank order (deterministic) before writing t1.
#pragma once

#include <cooperative_groups.h>

#include "pdt_primal.cuh"
#include "pdt_tc.cuh"

namespace pdt {
namespace {

constexpr int kTcRows = 128;
constexpr uint32_t kTcTmemCols = 256;
constexpr uint32_t kTcTileA = 128 * 128;  // bytes of one 128-row x 32-element FP32 tile
constexpr int kTcMaxStages = 4;

__device__ __forceinline__ unsigned char* tc_align1024(unsigned char* raw) {
  const uint32_t off = tc::smem_addr(raw);
  return raw + ((1024u - (off & 1023u)) & 1023u);
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
// barriers after the stages: full, empty and copy (8 bytes each per stage), accb, the TMEM slot
inline size_t tc_adj_smem(int NB, int nst) { return 1024 + (size_t)nst * tc_stage_bytes(NB) + 24 * kTcMaxStages + 32; }
inline size_t tc_fwd_smem(int nb, int nst) { return 1024 + (size_t)nst * tc_stage_bytes(nb) + 24 * kTcMaxStages + 32; }

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
// Thread 0 bulk-copies the DFT factor from the operator's precomputed tiles; warps 2..15 stage the data
// operand from t2 (split into TF32 hi/lo) and arrive on the stage's barrier; thread 32 issues the MMAs.
// The epilogue (1) moves TMEM lanes 32 q .. + 31 (warps q, q + 4, ...: one row per thread, column
// groups of 8) to shared memory, (2) sums the coils: item (yl, four real columns) per thread, coalesced
// along x. `nst` stages of [A hi | A lo | B hi | B lo].
// ------------------------------------------------------------------------------------------------
constexpr int kTcAdjThreads = 512;  // 16 warps: copy thread (warp 0), MMA thread (warp 1), 14 staging warps
constexpr int kTcStagers = kTcAdjThreads - 64;
constexpr int kTcStageItems = (kTcRows * 8 + kTcStagers - 1) / kTcStagers;  // staging items per thread
constexpr int kTcAdjMaxNB = 256;    // output columns (re/im) per CTA
constexpr int kTcCoilUnroll = 16;   // coil-sum loads issued together

// Thread 0 waits until the DFT-factor copies it started (chunks 0 .. issued-1, stage j % nst) have
// landed, so that no copy into this CTA's shared memory is still in flight when the CTA reuses it or
// exits -- after a wait gave up the MMA thread may not have consumed them. A copy into a stage starts
// only after the MMAs of the stage's previous chunk, hence after that chunk's copy phase completed, so
// only each stage's last phase can be pending.
__device__ __forceinline__ void copies_drain(uint64_t* copied, int issued, int nst, int* err) {
  for (int b = 0; b < nst && b < issued; ++b) {
    const int j = b + ((issued - 1 - b) / nst) * nst;  // last chunk copied into stage b
    if (!tc::mbar_wait(&copied[b], (j / nst) & 1)) atomicCAS(err, 0, 0x600 | j);
  }
}

template <bool SENS>
__global__ void __launch_bounds__(kTcAdjThreads, 1) tc_rows_adj(CartDev d, const float2* __restrict__ t2,
                                                             const unsigned char* __restrict__ btiles,
                                                             float2* __restrict__ out, int NB, int nst,
                                                             int* __restrict__ err, int ntiles, DualStep ds) {
  if ((int)blockIdx.y >= ntiles) {
    // rows of blocks past the row tiles run the solver's dual update (no TMEM, no barriers); its inputs
    // come from before the previous launch, its outputs are read only after this launch completes
    pdl_wait();
    pdl_trigger();
    const int db = (blockIdx.y - ntiles) * gridDim.x + blockIdx.x, nd = (gridDim.y - ntiles) * gridDim.x;
    if (ds.tgv)
      mri_dual_blocks<true>(ds, db, nd);
    else
      mri_dual_blocks<false>(ds, db, nd);
    return;
  }
  extern __shared__ unsigned char tc_smem_raw[];
  unsigned char* sm = tc_align1024(tc_smem_raw);
  const int W = d.W, ns = d.ns, Hi = d.Hi, C = d.C, yb = d.tc_yb;
  const uint32_t stage_bytes = tc_stage_bytes(NB);
  uint64_t* full = reinterpret_cast<uint64_t*>(sm + nst * stage_bytes);  // A stores of a stage landed
  uint64_t* empty = full + kTcMaxStages;                                  // MMAs of a stage done
  uint64_t* copied = empty + kTcMaxStages;                                // B copy of a stage landed
  uint64_t* accb = copied + kTcMaxStages;                                 // every MMA done (one phase)
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
      tc::mbar_init(&full[i], kTcStagers / 32);
      tc::mbar_init(&empty[i], 1);
      tc::mbar_init(&copied[i], 1);
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
  bool ok = true;
  int issued = 0;  // DFT-factor chunks whose copies thread 0 has started
  const bool drop = tc::g_drop_arrival != 0;
  if (tid == 0) {  // DFT-factor tiles (constants: the first copies may start before the column kernel ends)
    for (int j = 0; j < nch && ok; ++j) {
      const int b = j % nst;
      if (j >= nst) ok = tc::mbar_wait(&empty[b], ((j / nst) - 1) & 1);  // the MMAs of chunk j - nst are done
      if (!ok) {
        atomicCAS(err, 0, 0x100 | j);
        break;
      }
      tc::mbar_arrive_expect_tx(&copied[b], bbytes);
      tc::bulk_g2s(base + b * stage_bytes + 2 * kTcTileA, bsrc + (size_t)j * 2 * NB * 128, bbytes, &copied[b]);
      issued = j + 1;
    }
  }
  pdl_wait();  // every thread: t2 comes from the column kernel
  pdl_trigger();
  if (tid == 32) {
    const uint32_t idesc = tc::idesc_tf32(kTcRows, nb);
    for (int j = 0; j < nch && ok; ++j) {
      const int b = j % nst;
      ok = tc::mbar_wait(&full[b], (j / nst) & 1) && tc::mbar_wait(&copied[b], (j / nst) & 1);
      if (!ok) {
        atomicCAS(err, 0, 0x200 | j);  // the MMA thread gave up waiting for chunk j's operands
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
  } else if (warp >= 2) {
    // data operand: tile row m = c yb + yl, 16-byte chunk p = sampled columns 16 j + 2p, + 1 (re/im
    // each), split into TF32 hi/lo. Item it = ot + kTcStagers k, yl fastest (consecutive image rows of
    // t2 for consecutive threads); the next chunk's values are loaded before the wait for its stage.
    const int ot = tid - 64;
    const int nit = C * yb * 8;  // items of the C yb tile rows in use (<= 128 x 8); later rows stay unused
    int im[kTcStageItems], ioff[kTcStageItems];
#pragma unroll
    for (int k = 0; k < kTcStageItems; ++k) {
      const int it = ot + kTcStagers * k;
      const int yl = it % yb, rest = it / yb, p = rest & 7, c = rest >> 3;
      const int y = ybase + yl;
      const bool valid = it < nit && y < Hi;
      im[k] = valid ? ((c * yb + yl) << 3 | p) : -1;  // tile row and chunk
      ioff[k] = (c * ns + 2 * p) * Hi + y;             // t2 offset of column 2p of chunk 0
    }
    float2 va[kTcStageItems], vb[kTcStageItems];
    auto load = [&](int j) {
#pragma unroll
      for (int k = 0; k < kTcStageItems; ++k) {
        const int s = 16 * j + 2 * ((im[k] >= 0 ? im[k] : 0) & 7);
        va[k] = vb[k] = c2(0.f, 0.f);
        if (im[k] >= 0 && s < ns) va[k] = t2[(size_t)ioff[k] + (size_t)16 * j * Hi];
        if (im[k] >= 0 && s + 1 < ns) vb[k] = t2[(size_t)ioff[k] + (size_t)(16 * j + 1) * Hi];
      }
    };
    if (nch > 0) load(0);
    for (int j = 0; j < nch && ok; ++j) {
      const int b = j % nst;
      float4 cur[kTcStageItems];
#pragma unroll
      for (int k = 0; k < kTcStageItems; ++k) cur[k] = make_float4(va[k].x, va[k].y, vb[k].x, vb[k].y);
      if (j + 1 < nch) load(j + 1);
      if (j >= nst) {  // one lane polls; the others wait in the warp barrier without taking issue slots
        if (lane == 0) ok = tc::mbar_wait(&empty[b], ((j / nst) - 1) & 1);
        ok = __shfl_sync(0xffffffffu, ok, 0);
      }
      if (!ok) {
        if (lane == 0) atomicCAS(err, 0, 0x400 | j);
        break;
      }
      const uint32_t a_hi = base + b * stage_bytes, a_lo = a_hi + kTcTileA;
#pragma unroll
      for (int k = 0; k < kTcStageItems; ++k) {
        const int it = ot + kTcStagers * k;
        if (it < nit) {  // tile row m = c yb + yl < C yb <= 128 (a D row depends on its own A row only)
          const int yl = it % yb, rest = it / yb, p = rest & 7, m = (rest >> 3) * yb + yl;
          float4 hi, lo;
          tc::split4(cur[k], hi, lo);  // zero for image rows past the last one
          const uint32_t o = tc::sw128(m, p);
          tc::st_shared4(a_hi + o, hi);
          tc::st_shared4(a_lo + o, lo);
        }
      }
      tc::fence_async_smem();
      __syncwarp();
      if (lane == 0 && !(drop && j == 0 && warp == 2)) tc::mbar_arrive(&full[b]);  // one arrival per staging warp
    }
  }
  if (tid == 0) copies_drain(copied, issued, nst, err);

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
// Forward rows: t1[c][s][y] = sum_x (ubar . sens_c)[y][x] w^(q(x) f_s) for the 128 sampled columns of s
// tile blockIdx.z. K = 2 W (x, re/im), split over the KS CTAs of a cluster (grid.y); N = 2 (s, re/im)
// <= 256; M: the adjoint's row tiles (yb image rows of every coil). The DFT factor arrives by bulk copy
// (thread 0); warps 2..15 form the data operand ubar . sens_c on chip, split it into TF32 hi/lo parts
// and arrive on the stage's barrier; thread 32 issues the MMAs. The KS partial accumulators are summed
// through distributed shared memory in rank order (deterministic).
// ------------------------------------------------------------------------------------------------
constexpr int kTcFwdThreads = 512;
constexpr int kTcFwdStagers = kTcFwdThreads - 64;
constexpr int kTcFwdItems = (kTcRows * 8 + kTcFwdStagers - 1) / kTcFwdStagers;  // staging items per thread
constexpr int kTcFwdBatch = 4;  // reduction items per thread whose remote loads are in flight together

template <bool SENS>
__global__ void __launch_bounds__(kTcFwdThreads, 1) tc_rows_fwd(CartDev d, const float2* __restrict__ ubar,
                                                             const unsigned char* __restrict__ btiles,
                                                             float2* __restrict__ t1, int* __restrict__ tick,
                                                             int nst, int* __restrict__ err) {
  namespace cg = cooperative_groups;
  extern __shared__ unsigned char tc_smem_raw[];
  unsigned char* sm = tc_align1024(tc_smem_raw);
  const int W = d.W, ns = d.ns, Hi = d.Hi, C = d.C, yb = d.tc_yb;
  const int s0 = blockIdx.z * 128, nsl = min(128, ns - s0);
  const int nb = (2 * nsl + 15) & ~15;
  const int nbmax = (2 * min(128, ns) + 15) & ~15;  // B tile stride of the precomputed tiles
  const uint32_t stage_bytes = tc_stage_bytes(nb);
  uint64_t* full = reinterpret_cast<uint64_t*>(sm + nst * stage_bytes);  // A stores of a stage landed
  uint64_t* empty = full + kTcMaxStages;                                  // MMAs of a stage done
  uint64_t* copied = empty + kTcMaxStages;                                // B copy of a stage landed
  uint64_t* accb = copied + kTcMaxStages;                                 // every MMA done (one phase)
  uint32_t* tslot = reinterpret_cast<uint32_t*>(accb + 1);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int T = blockIdx.x, ybase = T * yb;
  const int KS = gridDim.y, ks = blockIdx.y;
  const int nchT = (2 * W + 31) >> 5;
  const int jb = ks * nchT / KS, je = (ks + 1) * nchT / KS, nch = je - jb;

  if (tid == 0) {
    for (int i = 0; i < nst; ++i) {
      tc::mbar_init(&full[i], kTcFwdStagers / 32);
      tc::mbar_init(&empty[i], 1);
      tc::mbar_init(&copied[i], 1);
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
  const unsigned char* bsrc = btiles + ((size_t)blockIdx.z * nchT + jb) * 2 * nbmax * 128;

  bool ok = true;
  int issued = 0;  // DFT-factor chunks whose copies thread 0 has started
  const bool drop = tc::g_drop_arrival != 0;
  if (tid == 0) {  // DFT-factor tiles (constants, may start before the previous kernel ends)
    for (int jl = 0; jl < nch && ok; ++jl) {
      const int b = jl % nst;
      if (jl >= nst) ok = tc::mbar_wait(&empty[b], ((jl / nst) - 1) & 1);
      if (!ok) {
        atomicCAS(err, 0, 0x1100 | jl);
        break;
      }
      tc::mbar_arrive_expect_tx(&copied[b], bbytes);
      tc::bulk_g2s(base + b * stage_bytes + 2 * kTcTileA, bsrc + (size_t)jl * 2 * nbmax * 128, bbytes,
                   &copied[b]);
      issued = jl + 1;
    }
  }
  pdl_wait();  // every thread: ubar comes from the previous kernel; t1 may still be read by it
  pdl_trigger();
  if (tick && blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && tid == 0) atomicAdd(tick, 1);
  if (tid == 32) {
    const uint32_t idesc = tc::idesc_tf32(kTcRows, nb);
    for (int jl = 0; jl < nch && ok; ++jl) {
      const int b = jl % nst;
      ok = tc::mbar_wait(&full[b], (jl / nst) & 1) && tc::mbar_wait(&copied[b], (jl / nst) & 1);
      if (!ok) {
        atomicCAS(err, 0, 0x1200 | jl);
        break;
      }
      const uint32_t a_hi = base + b * stage_bytes, a_lo = a_hi + kTcTileA;
      const uint32_t b_hi = a_lo + kTcTileA, b_lo = b_hi + (uint32_t)nb * 128u;
      tc_issue_chunk(tmem, a_hi, a_lo, b_hi, b_lo, min(4, (2 * W - 32 * (jb + jl) + 7) >> 3), idesc, jl == 0,
                     &empty[b]);
    }
    tc::mma_commit(accb);
    if (!tc::mbar_wait(accb, 0)) {
      atomicCAS(err, 0, 0x1300);
      ok = false;
    }
    tc::fence_before_sync();
  } else if (warp >= 2) {
    // data operand: tile row m = c yb + yl, 16-byte chunk p = image columns x0 + 2p, x0 + 2p + 1. Item
    // it = ot + kTcFwdStagers k; the next chunk's ubar and coil-map values are loaded into registers
    // before the wait for its stage, so that their latency overlaps the MMAs.
    const int ot = tid - 64;
    int im[kTcFwdItems];   // tile row of item k (or -1)
    int ioff[kTcFwdItems];  // ubar offset y W + 2 p of item k (add the chunk's first column)
    int isoff[kTcFwdItems];
#pragma unroll
    for (int k = 0; k < kTcFwdItems; ++k) {
      const int it = ot + kTcFwdStagers * k;
      const int p = it & 7, m = it >> 3;
      const int c = m / yb, yl = m - c * yb, y = ybase + yl;
      const bool valid = it < kTcRows * 8 && c < C && y < Hi;
      im[k] = valid ? m : -1;
      ioff[k] = y * W + 2 * p;
      isoff[k] = (c * d.Hf + y + d.y0) * W + 2 * p;
    }
    float4 uv[kTcFwdItems], sv[kTcFwdItems];
    auto load = [&](int jl) {
      const int x0 = 16 * (jb + jl);
#pragma unroll
      for (int k = 0; k < kTcFwdItems; ++k) {
        const int it = ot + kTcFwdStagers * k;
        const int x = x0 + 2 * (it & 7);
        uv[k] = sv[k] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (im[k] >= 0 && x < W) {  // x even and W even: x + 1 < W
          uv[k] = *reinterpret_cast<const float4*>(ubar + (size_t)ioff[k] + x0);
          if (SENS) sv[k] = *reinterpret_cast<const float4*>(d.sens + (size_t)isoff[k] + x0);
        }
      }
    };
    if (nch > 0) load(0);
    for (int jl = 0; jl < nch && ok; ++jl) {
      const int b = jl % nst;
      float4 cur[kTcFwdItems];
#pragma unroll
      for (int k = 0; k < kTcFwdItems; ++k) cur[k] = SENS ? tc_cmul2(uv[k], sv[k]) : uv[k];
      if (jl + 1 < nch) load(jl + 1);
      if (jl >= nst) {  // one lane polls; the others wait in the warp barrier without taking issue slots
        if (lane == 0) ok = tc::mbar_wait(&empty[b], ((jl / nst) - 1) & 1);
        ok = __shfl_sync(0xffffffffu, ok, 0);
      }
      if (!ok) {
        if (lane == 0) atomicCAS(err, 0, 0x1400 | jl);
        break;
      }
      const uint32_t a_hi = base + b * stage_bytes, a_lo = a_hi + kTcTileA;
#pragma unroll
      for (int k = 0; k < kTcFwdItems; ++k) {
        const int it = ot + kTcFwdStagers * k;
        if (it < kTcRows * 8) {
          float4 hi, lo;
          tc::split4(cur[k], hi, lo);
          const uint32_t o = tc::sw128(it >> 3, it & 7);
          tc::st_shared4(a_hi + o, hi);
          tc::st_shared4(a_lo + o, lo);
        }
      }
      tc::fence_async_smem();
      __syncwarp();
      if (lane == 0 && !(drop && jl == 0 && warp == 2)) tc::mbar_arrive(&full[b]);  // one arrival per staging warp
    }
  }
  if (tid == 0) copies_drain(copied, issued, nst, err);
  const bool done = __syncthreads_and(ok);
  tc::fence_after_sync();
  // accumulator -> shared memory as complex values [sl][tile row] (a warp's rows are consecutive); the
  // stage buffers are free
  float2* dt = reinterpret_cast<float2*>(sm);
  if (done) {
    const int q = warp & 3, h = warp >> 2;
    const int G8 = nb >> 3, gb = h * G8 / 4, ge = (h + 1) * G8 / 4;
    const uint32_t taddr = tmem + ((uint32_t)(32 * q) << 16);
    const int row = 32 * q + lane;
    for (int g = gb; g < ge; ++g) {
      float v[8];
      tc::tmem_ld8(taddr + (uint32_t)(8 * g), v);
#pragma unroll
      for (int i = 0; i < 4; ++i) dt[(size_t)(4 * g + i) * kTcRows + row] = c2(v[2 * i], v[2 * i + 1]);
    }
  }
  cg::cluster_group cluster = cg::this_cluster();
  const int anybad = __syncthreads_or(!done);
  cluster.sync();  // every CTA's partial accumulator is in its shared memory (all CTAs reach this)
  if (!anybad) {
    // rank ks writes sampled columns [sb, se) of this s tile: items (c, s, yl), yl fastest, so that a
    // warp's remote loads and t1 stores cover consecutive tile rows / image rows
    const int sb = ks * nsl / KS, se = (ks + 1) * nsl / KS, nsr = se - sb, n = C * nsr * yb;
    for (int i0 = tid; i0 < n; i0 += kTcFwdThreads * kTcFwdBatch) {
      float2 acc[kTcFwdBatch];
      int src[kTcFwdBatch], dst[kTcFwdBatch];
#pragma unroll
      for (int u = 0; u < kTcFwdBatch; ++u) {
        const int i = i0 + u * kTcFwdThreads;
        acc[u] = c2(0.f, 0.f);
        dst[u] = -1;
        src[u] = 0;
        if (i < n) {
          const int yl = i % yb, rest = i / yb, sl = sb + rest % nsr, c = rest / nsr;
          if (ybase + yl < Hi) {
            dst[u] = (c * ns + s0 + sl) * Hi + ybase + yl;
            src[u] = sl * kTcRows + c * yb + yl;
          }
        }
      }
      for (int qq = 0; qq < KS; ++qq) {  // rank order
        const float2* rem = cluster.map_shared_rank(dt, qq);
#pragma unroll
        for (int u = 0; u < kTcFwdBatch; ++u)
          if (dst[u] >= 0) acc[u] += rem[src[u]];
      }
#pragma unroll
      for (int u = 0; u < kTcFwdBatch; ++u)
        if (dst[u] >= 0) t1[(size_t)dst[u]] = acc[u];
    }
  }
  cluster.sync();  // keep this CTA's shared memory alive until the other CTAs have read it
  if (!done && tid == 0) atomicCAS(err, 0, 0x1500);
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, kTcTmemCols);
  }
}

}  // namespace
}  // namespace pdt
