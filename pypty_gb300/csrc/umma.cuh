// tcgen05 (5th-generation tensor core) helpers for sm_103a, as inline PTX:
//   * shared-memory matrix descriptors for K-major operands in the 128-byte swizzled layout,
//   * the instruction descriptor of kind::f16 MMAs with BF16 inputs and FP32 accumulation,
//   * single-thread MMA issue, commit to an mbarrier, TMEM allocation and 32-lane loads.
//
// Operand layout (per 8-row group of 128-byte rows, 1024 bytes, the unit of the 128B swizzle):
// element (r, k) of a K-major tile of 16-bit values sits at byte
//   (r / 8) * 1024 + (r % 8) * 128 + (((2k / 16) ^ (r % 8)) * 16) + (2k % 16)
// for k < 64 (one 128-byte row); tiles wider than 64 along K are stored as consecutive
// 64-wide blocks. Tile bases are 1024-byte aligned. An MMA with K = 16 reads 32 bytes of every
// row: the k-th K step of a 64-wide block starts 32 * k bytes after the block's base.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "window_fft.cuh"

namespace pty {
namespace umma {

// byte offset of element (r, k) inside a 128B-swizzled K-major block of 16-bit values, k < 64
__host__ __device__ constexpr uint32_t sw128_offset(uint32_t r, uint32_t k) {
  return (r >> 3) * 1024u + (r & 7u) * 128u + ((((2u * k) >> 4) ^ (r & 7u)) << 4) + ((2u * k) & 15u);
}

// Shared-memory matrix descriptor: start address, leading-dimension offset (unused by the
// swizzled K-major layout), stride between 8-row groups (1024 B), descriptor version 1,
// swizzle mode 2 (128 B).
__device__ __forceinline__ uint64_t desc_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)(16u >> 4) << 16;
  d |= (uint64_t)(1024u >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

// kind::f16 instruction descriptor: D FP32, A and B BF16, both K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// D[tmem] (+)= A * B^T, issued by one thread
__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// arrive once on `bar` when every MMA this thread issued before has completed
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// warp-wide: allocate ncols TMEM columns (power of two >= 32); the address lands in *dst
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// warp-wide: lane l of the warp receives columns [col, col + 32) of TMEM lane (lane_base + l)
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// FP32 -> BF16 bits (round to nearest even) and back
__device__ __forceinline__ uint16_t bf16_bits(float x) { return __bfloat16_as_ushort(__float2bfloat16_rn(x)); }
__device__ __forceinline__ float bf16_value(uint16_t b) { return __uint_as_float((uint32_t)b << 16); }

// FP32 -> BF16 hi/lo split (round to nearest even): x ~= hi + lo with |x - hi - lo| <= 2^-16 |x|
__device__ __forceinline__ void split_bf16(float x, uint16_t& hi, uint16_t& lo) {
  const __nv_bfloat16 h = __float2bfloat16_rn(x);
  const float r = x - __bfloat162float(h);
  const __nv_bfloat16 l = __float2bfloat16_rn(r);
  hi = __bfloat16_as_ushort(h);
  lo = __bfloat16_as_ushort(l);
}

}  // namespace umma
}  // namespace pty
