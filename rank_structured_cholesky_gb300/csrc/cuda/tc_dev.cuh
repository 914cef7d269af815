// Device helpers of the tcgen05 (5th-generation tensor core) paths: the
// 128-byte-swizzled K-major operand layout and its shared-memory descriptor,
// TF32 conversion, mbarriers, and the kind::tf32 MMA with M = 128 (one
// accumulator row per TMEM lane), TMEM allocation and loads.
#pragma once
#include <cuda_bf16.h>

#include <cstdint>

namespace rschol {
namespace tcdev {

constexpr int TC_SPIN_LIMIT = 1 << 22;   // polls before an mbarrier wait gives up

// Byte offset of element (r, k) of a K-major operand tile in the 128-byte
// swizzled layout: row r occupies 128 bytes (32 TF32) of an 8-row, 1024-byte
// atom; its 16-byte chunk c is stored at chunk c ^ (r & 7).
__device__ __forceinline__ uint32_t tc_off(int r, int k) {
  return (uint32_t)(((r >> 3) << 10) + ((r & 7) << 7) + ((((k >> 2) ^ (r & 7)) & 7) << 4) + ((k & 3) << 2));
}

// The same layout for 16-bit elements: a row is 64 BF16, a 16-byte chunk 8.
__device__ __forceinline__ uint32_t tc_off16(int r, int k) {
  return (uint32_t)(((r >> 3) << 10) + ((r & 7) << 7) + ((((k >> 3) ^ (r & 7)) & 7) << 4) + ((k & 7) << 1));
}

__device__ __forceinline__ uint64_t tc_smem_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);            // start address (advances 32 B per K = 8)
  d |= (uint64_t)1 << 16;                             // leading byte offset (unused within a 128 B row)
  d |= (uint64_t)((1024u >> 4) & 0x3FFFu) << 32;      // stride byte offset: next 8-row atom
  d |= (uint64_t)1 << 46;                             // descriptor version (tcgen05)
  d |= (uint64_t)2 << 61;                             // 128-byte swizzle (atoms 1024-byte aligned)
  return d;
}

__device__ __forceinline__ uint32_t to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ void mbar_init(uint32_t addr, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(addr), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t addr, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(addr), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait for the mbarrier phase with the given parity to complete.
__device__ __forceinline__ bool mbar_wait(uint32_t addr, uint32_t parity, int limit = TC_SPIN_LIMIT) {
  for (int it = 0; it < limit; ++it)
    if (mbar_try_wait(addr, parity)) return true;
  return false;
}

__device__ __forceinline__ void tc_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
               : "memory");
}

// One arrival that also expects `bytes` of asynchronous (TMA) transactions.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t addr, uint32_t bytes) {
  asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(addr),
               "r"(bytes)
               : "memory");
}

// The tensor map at tmap (global memory, 64-byte aligned, written before the
// launch) made visible to the tensor-map proxy before its first use.
__device__ __forceinline__ void tmap_acquire(uint64_t tmap) {
  asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(tmap) : "memory");
}

// TMA: the box of the 2D tensor map at element coordinates (x, y) -> shared
// memory at dst, completing `bytes` on the mbarrier at mbar.  x times the
// element size must be a multiple of 16 bytes.
__device__ __forceinline__ void tma_load_2d(uint32_t dst, uint64_t tmap, int x, int y, uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
          "r"(dst),
      "l"(tmap), "r"(x), "r"(y), "r"(mbar)
      : "memory");
}

__device__ __forceinline__ float4 ld_shared_v4(uint32_t addr) {
  float4 v;
  asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "r"(addr)
               : "memory");
  return v;
}

__device__ __forceinline__ void mbar_arrive(uint32_t addr) {
  asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(addr) : "memory");
}

__device__ __forceinline__ void st_shared_v4(uint32_t addr, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
  asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(a), "r"(b), "r"(c), "r"(d) : "memory");
}
__device__ __forceinline__ void st_shared_b32(uint32_t addr, uint32_t a) {
  asm volatile("st.shared.b32 [%0], %1;" ::"r"(addr), "r"(a) : "memory");
}
__device__ __forceinline__ void st_shared_v2(uint32_t addr, uint32_t a, uint32_t b) {
  asm volatile("st.shared.v2.b32 [%0], {%1, %2};" ::"r"(addr), "r"(a), "r"(b) : "memory");
}
__device__ __forceinline__ void st_shared_b16(uint32_t addr, unsigned short a) {
  asm volatile("st.shared.b16 [%0], %1;" ::"r"(addr), "h"(a) : "memory");
}

// Two FP32 values as BF16 (round to nearest even), the first in the low half.
__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<const uint32_t*>(&v);
}
// The same, and the remainders a - bf16(a), b - bf16(b) (exact in FP32) for
// the low part of a split product.
__device__ __forceinline__ uint32_t split_bf16x2(float a, float b, float& ra, float& rb) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
  ra = a - __low2float(v);
  rb = b - __high2float(v);
  return *reinterpret_cast<const uint32_t*>(&v);
}

// Instruction descriptor: D f32, A and B both tf32 (kind::tf32) or both
// bf16 (kind::f16), both K-major, M = 128, N = BN.
template <int BN, bool BF = false>
__host__ __device__ constexpr uint32_t ws_idesc() {
  return (1u << 4) | ((BF ? 1u : 2u) << 7) | ((BF ? 1u : 2u) << 10) | ((uint32_t)(BN >> 3) << 17) |
         ((uint32_t)(128 >> 4) << 24);
}

// One MMA step of 32 bytes along K (8 TF32 or 16 BF16) into the accumulator.
template <int BN, bool BF = false>
__device__ __forceinline__ void ws_mma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  if constexpr (BF)
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(ws_idesc<BN, true>()), "r"(accumulate)
        : "memory");
  else
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(ws_idesc<BN>()), "r"(accumulate)
        : "memory");
}

// TMEM columns for the CTA (one warp, all lanes); the base address lands in
// shared memory at dst.  The CTA then gives up its right to allocate again.
__device__ __forceinline__ void tmem_alloc(uint32_t dst, uint32_t cols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst), "r"(cols) : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t cols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols) : "memory");
}
// 32 consecutive FP32 columns of the warp's 32 TMEM lanes (lane i: row i of
// its quarter), completed before returning.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

}  // namespace tcdev
}  // namespace rschol
