// pdt_tc.cuh -- fifth-generation tensor-core primitives (tcgen05, sm_100 family) as inline PTX:
// tensor-memory allocation, shared-memory matrix descriptors for the 128-byte-swizzled K-major layout,
// the kind::tf32 MMA with an FP32 accumulator in tensor memory, MMA completion through an mbarrier,
// tensor-memory loads for the epilogue, and the TF32 hi/lo split that keeps FP32 accuracy with three
// MMAs per product (a_hi b_hi + a_hi b_lo + a_lo b_hi).
//
// Operand layout (both A and B K-major, 128-byte swizzle): a tile holds rows of 32 FP32 elements along K
// (128 bytes); row m lives at byte m * 128 of the tile, its 16-byte chunk c at chunk position c ^ (m & 7);
// 8-row groups are 1024 bytes apart (the descriptor's stride byte offset). Tiles are 1024-byte aligned.
// One MMA consumes K = 8 (32 bytes of each row); the k-th step of a tile starts 32 k bytes in.
#pragma once

#include <cstdint>

#include "pdt_device.cuh"

namespace pdt {
namespace tc {

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// byte offset of 16-byte chunk `chunk` (0..7) of row `row` in a 128-byte-swizzled tile
__device__ __forceinline__ uint32_t sw128(int row, int chunk) {
  return (uint32_t)(row * 128 + ((chunk ^ (row & 7)) << 4));
}

// Shared-memory matrix descriptor (tcgen05 format): start address >> 4 in bits 0-13, leading byte
// offset >> 4 in 16-29 (unused for swizzled K-major tiles), stride byte offset >> 4 in 32-45, the fixed
// version value 1 in bits 46-47, base offset 0 (1024-aligned tiles), swizzle mode 2 (128 bytes) in 61-63.
__device__ __forceinline__ uint64_t desc_sw128(uint32_t saddr) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

// Shared-memory matrix descriptor, no swizzle, K-major: core matrices of 8 rows x 16 bytes stored
// contiguously (row r at byte 16 r); `kstride` bytes between core matrices adjacent along K (leading byte
// offset), `mnstride` bytes between core matrices adjacent along M / N (stride byte offset).
__device__ __forceinline__ uint64_t desc_interleave(uint32_t saddr, uint32_t kstride, uint32_t mnstride) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((kstride >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((mnstride >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}

// Instruction descriptor of kind::tf32: FP32 accumulator (bits 4-5 = 1), A and B TF32 (bits 7-9 and
// 10-12 = 2), both K-major (bits 15, 16 = 0), N >> 3 in bits 17-22, M >> 4 in bits 24-28.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// D[tmem] (+)= A * B^T for one K = 8 step; issued by a single thread.
__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

// Instruction descriptor of kind::f16 with BF16 A and B (bits 7-9, 10-12 = 1) and an FP32 accumulator.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// D[tmem] (+)= A * B^T for one K = 16 step of BF16 operands; issued by a single thread.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

// The mbarrier receives one arrival once every tcgen05 operation issued so far by this thread is done.
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
               : "memory");
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy shared-memory writes become visible to the tensor core (async proxy)
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// One arrival that also announces `bytes` of asynchronous copies completing on the same phase.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}

// Bulk copy global -> this CTA's shared memory (both 16-byte aligned, size a multiple of 16); the bytes
// complete on the mbarrier's transaction count.
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}
// orders this thread's earlier generic-proxy accesses of global memory before its asynchronous copies
__device__ __forceinline__ void fence_async_global() { asm volatile("fence.proxy.async.global;" ::: "memory"); }

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

constexpr uint64_t kWaitLimitNs = 200000000ull;  // 200 ms

// Waits for the phase with the given parity to complete; gives up (returns false) after about
// `limit_ns` nanoseconds so that a lost arrival ends in an error status instead of a hung kernel. A
// kernel that gives up still waits (with the same limit) for the copies and MMAs it has issued before
// it frees its tensor memory and exits.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint64_t limit_ns = kWaitLimitNs) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  for (uint32_t i = 0;; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 255u) == 255u && global_ns() - t0 > limit_ns) return false;
  }
}

// Test hook for the give-up path: while non-zero, the tensor-core kernels withhold one arrival (the
// Cartesian row kernels: staging warp 2's arrival for operand chunk 0; the convolution: block 0's MMAs
// and commit for its first tile), so that one bounded wait runs out. Nothing else sets it; each
// translation unit including this header has its own copy, set by set_drop_arrival in that unit.
static __device__ int g_drop_arrival = 0;

static inline cudaError_t set_drop_arrival(int on) { return cudaMemcpyToSymbol(g_drop_arrival, &on, sizeof(int)); }

// Tensor memory: one warp allocates `ncols` columns (a power of two >= 32) and writes the address to
// shared memory; the same warp frees them.
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(slot)), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// 16 consecutive FP32 columns of this thread's lane (warp w reads lanes 32 (w % 4) .. + 31; the lane
// offset is in bits 16-31 of the address). Waits for the load before returning.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
// 8 consecutive FP32 columns (same addressing), waited for.
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
  uint32_t r[8];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

// x rounded to TF32 (10 explicit mantissa bits, round to nearest, ties away from zero); the low 13
// bits of the result are zero.
__device__ __forceinline__ float tf32_round(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}
// x = hi + lo + O(2^-22 |x|) with hi and lo TF32 values: three TF32 products then carry FP32 accuracy.
__device__ __forceinline__ void split_tf32(float x, float& hi, float& lo) {
  hi = tf32_round(x);
  lo = tf32_round(x - hi);
}
__device__ __forceinline__ void split4(float4 v, float4& hi, float4& lo) {
  split_tf32(v.x, hi.x, lo.x);
  split_tf32(v.y, hi.y, lo.y);
  split_tf32(v.z, hi.z, lo.z);
  split_tf32(v.w, hi.w, lo.w);
}

__device__ __forceinline__ void st_shared4(uint32_t addr, float4 v) {
  asm volatile("st.shared.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w)
               : "memory");
}

}  // namespace tc
}  // namespace pdt
