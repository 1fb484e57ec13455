// Thin inline-PTX wrappers for the 5th-generation tensor cores of sm_103a (tcgen05): tensor
// memory (TMEM) allocation, shared-memory matrix descriptors, the single-thread MMA issue,
// its completion through an mbarrier, and the TMEM -> register loads of the epilogue.
//
// Shared-memory operands use the K-major layout without swizzling: the tile is made of core
// matrices of 8 rows x 16 bytes stored as 128 contiguous bytes; for a K step of 32 bytes (8
// tf32 elements) the two core matrices of a row group sit LBO = 128 bytes apart and row
// groups SBO = 256 bytes apart, so element (row r, k) of a step lives at
//   (r / 8) * 256 + (k / 4) * 128 + (r % 8) * 16 + (k % 4) * 4   bytes.
#pragma once
#include <cstdint>

namespace fcg {
namespace tc {

constexpr uint32_t kLbo = 128;  // bytes between the two core matrices of a 32-byte K step
constexpr uint32_t kSbo = 256;  // bytes between groups of 8 rows

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// byte offset of element (row r, q) of one 8-element (32-byte) K step of a K-major operand
__device__ __forceinline__ uint32_t kmajor_off(int r, int q) {
  return uint32_t((r >> 3) * 256 + (q >> 2) * 128 + (r & 7) * 16 + (q & 3) * 4);
}

// Shared-memory matrix descriptor: start address, leading (K) and stride (row-group) byte
// offsets in 16-byte units, the fixed version field of sm_100-class descriptors, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  uint64_t d = 0;
  d |= uint64_t((addr & 0x3FFFFu) >> 4);
  d |= uint64_t((kLbo & 0x3FFFFu) >> 4) << 16;
  d |= uint64_t((kSbo & 0x3FFFFu) >> 4) << 32;
  d |= uint64_t(1) << 46;
  return d;
}

// Instruction descriptor of kind::tf32 with an f32 accumulator, both operands K-major.
__device__ __forceinline__ uint32_t idesc_tf32(int M, int N) {
  return (1u << 4)                        // D format f32
         | (2u << 7) | (2u << 10)         // A, B format tf32
         | (uint32_t(N >> 3) << 17)       // N / 8
         | (uint32_t(M >> 4) << 24);      // M / 16
}

// TMEM allocation of ncols columns (a power of two >= 32) by one whole warp; the address is
// written to shared memory at slot.
__device__ __forceinline__ void tmem_alloc(uint32_t slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// generic-proxy stores to shared memory become visible to the tensor cores' reads
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// D[tmem] (+)= A[smem] * B[smem]^T, issued by one thread
__device__ __forceinline__ void mma_tf32(uint32_t taddr, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(taddr),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// the mbarrier at bar gets one arrival when every MMA this thread issued so far is complete
__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
               : "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ bool mbar_test(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// Waits for phase `parity` of the mbarrier to complete, at most about max_cycles SM cycles;
// false when it gave up.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, long long max_cycles) {
  const long long t0 = clock64();
  while (!mbar_test(bar, parity))
    if (clock64() - t0 > max_cycles) return false;
  return true;
}

// 16 consecutive f32 columns of this thread's TMEM lane (lanes 32w .. 32w+31 for warp w of
// the warpgroup), then the wait for the load
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// x = hi + lo with hi a tf32 value (the low 13 mantissa bits cleared) and lo = x - hi (exact)
__device__ __forceinline__ void split_tf32(float x, float& hi, float& lo) {
  hi = __uint_as_float(__float_as_uint(x) & 0xFFFFE000u);
  lo = x - hi;
}

}  // namespace tc
}  // namespace fcg
