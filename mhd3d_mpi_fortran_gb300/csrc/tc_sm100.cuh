// Fifth-generation tensor-core (tcgen05) building blocks for sm_103a, written
// as inline PTX: tensor-memory (TMEM) allocation, BF16 x BF16 -> FP32 MMA with
// operands in shared memory, completion through an mbarrier, and TMEM -> register
// loads.  Used by the MLP coarse-grid correction (mhd_mlp.cu).
//
// Operand layout ("canonical K-major, no swizzle"): a tile of R rows x K
// columns of BF16 is stored as 8-row x 16-byte core matrices, each 128
// contiguous bytes (row r of the core matrix at byte 16 r).  Core matrix
// (rg, kg) sits at byte 128 (rg (K/8) + kg): neighbours along K are 128 bytes
// apart (the descriptor's leading-dimension offset), neighbours along the rows
// 16 K bytes apart (its stride offset).  One MMA consumes K = 16 (two core
// matrices along K), so the k-th step starts 256 k bytes into the tile.
//
// Every wait is bounded (about a second of clock cycles); a kernel that gives
// up records it in an error word and still releases its TMEM.
#pragma once
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>

namespace mhd {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// byte offset of element (r, k) in a K-major canonical tile with K columns
__host__ __device__ __forceinline__ uint32_t kmaj(int r, int k, int K) {
  return (uint32_t)((((r >> 3) * (K >> 3) + (k >> 3)) << 7) + ((r & 7) << 4) + ((k & 7) << 1));
}

// Shared-memory matrix descriptor: start address, leading- and stride-
// dimension byte offsets, descriptor version 1 (bits 46-47), no swizzle.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Descriptor of a K-major canonical tile with K columns, at MMA step kk.
__device__ __forceinline__ uint64_t tile_desc(uint32_t base, int K, int kk) {
  return sdesc(base + 256u * (uint32_t)kk, 128u, 16u * (uint32_t)K);
}

// Instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), BF16
// A and B (bits 7-9, 10-12 = 1), both K-major, N/8 at bits 17-22, M/16 at 24-28.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy shared-memory writes -> visible to the tensor core's async proxy
__device__ __forceinline__ void fence_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// One warp (all 32 lanes) allocates ncols TMEM columns (power of 2, >= 32);
// the TMEM address lands in *slot.
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_free(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// D (TMEM) [+]= A (smem) * B (smem)^T; issued by one thread.
__device__ __forceinline__ void mma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}

// The mbarrier completes when every MMA this thread issued before has finished.
__device__ __forceinline__ void commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void bar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Wait for phase `parity` of the mbarrier to complete, for at most ~2e9
// cycles; false when it gave up.
__device__ __forceinline__ bool bar_wait(uint64_t* bar, uint32_t parity) {
  const long long t0 = clock64();
  for (;;) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    if (ok) return true;
    if (clock64() - t0 > 2000000000LL) return false;
  }
}

// 16 consecutive FP32 columns of this thread's TMEM lane (32x32b shape).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// TMEM address of lane group q (warp q of a 4-warp group reads lanes 32q..32q+31), column c.
__device__ __forceinline__ uint32_t tmem_at(uint32_t base, int q, int c) {
  return base + ((uint32_t)(32 * q) << 16) + (uint32_t)c;
}

__device__ __forceinline__ void st_bf16(unsigned char* tile, uint32_t off, float x) {
  *reinterpret_cast<__nv_bfloat16*>(tile + off) = __float2bfloat16_rn(x);
}

}  // namespace tc
}  // namespace mhd
