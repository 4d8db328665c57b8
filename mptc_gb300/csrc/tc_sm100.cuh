// sm_100-family (Blackwell, sm_103a) tensor-core and bulk-copy primitives as
// inline PTX: mbarriers, bulk copies and tiled tensor copies (TMA) into shared
// memory, and the fifth-generation tensor core (tcgen05: TMEM allocation, MMA
// issued by one thread with shared-memory operand descriptors, commit to an
// mbarrier, loads of the TMEM accumulator into registers).
//
// Operand layout used throughout: K-major tiles with the 128-byte swizzle.
// A tile of R rows x 64 bf16 (128 bytes per row) is stored as R/8 atoms of
// 1024 bytes; row r of the tile starts at (r/8)*1024 + (r%8)*128 and its
// 16-byte chunk c sits at chunk position c ^ (r%8). Such a tile is what a TMA
// tiled copy with CU_TENSOR_MAP_SWIZZLE_128B and a 64-element inner box
// writes, and what the MMA reads with a descriptor of swizzle mode 128B and a
// stride of 1024 bytes between 8-row groups. Successive K steps of 16 elements
// advance the descriptor's start address by 32 bytes inside the atom.
//
// Every wait is bounded by the global timer: a wait that gives up returns
// false, and the caller records an error status and winds down (it still
// releases its TMEM), so a protocol bug cannot hang the GPU.
#pragma once
#include <cstdint>

namespace mptc {
namespace tc {

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// ---- mbarriers ---------------------------------------------------------------
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// One try_wait that lets the hardware suspend the thread until the phase
// completes or `hint_ns` nanoseconds have passed (no instructions issue while
// it is suspended).
__device__ __forceinline__ bool mbar_test_suspend(uint64_t *bar, uint32_t parity, uint32_t hint_ns) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity), "r"(hint_ns)
      : "memory");
  return ok != 0;
}

// Waits until the phase with the given parity has completed; false after
// about `limit_ns` nanoseconds (or soon after *abort is set by another wait of
// the same CTA that already gave up). The thread sleeps in the try_wait
// between checks; the clock and the abort flag are read every 16 tries.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, const volatile uint32_t *abort,
                                          uint64_t limit_ns = 1000000000ull) {
  if (mbar_test(bar, parity)) return true;
  uint64_t t0 = 0;
  for (uint32_t it = 0;; ++it) {
    if (mbar_test_suspend(bar, parity, 100000u)) return true;
    if ((it & 15u) == 15u) {
      if (*abort) return false;
      const uint64_t t = global_ns();
      if (t0 == 0) t0 = t;
      else if (t - t0 > limit_ns) return false;
    }
  }
}

// ---- bulk copies (TMA) ---------------------------------------------------------
// Contiguous global -> shared copy of `bytes` (a multiple of 16, both addresses
// 16-byte aligned) completing on `bar` as transaction bytes.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

// Tiled 3-D tensor copy global -> shared through a tensor map (coordinates in
// elements, innermost first); elements outside the tensor read as zero.
__device__ __forceinline__ void tma_load_3d(void *dst, const void *tmap, int c0, int c1, int c2, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(smem_addr(dst)),
      "l"(tmap), "r"(c0), "r"(c1), "r"(c2), "r"(smem_addr(bar))
      : "memory");
}

// Orders this thread's generic-proxy shared-memory writes before later
// async-proxy (tensor core, TMA) accesses.
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// ---- tcgen05 -------------------------------------------------------------------
// TMEM allocation by one full warp; the base address is written to *slot.
__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(slot)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_free(uint32_t base, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(base), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart.
__device__ __forceinline__ uint64_t desc_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);  // start address
  d |= (uint64_t)1 << 16;                    // leading byte offset (unused for this layout)
  d |= (uint64_t)(1024 >> 4) << 32;          // stride byte offset: next 8-row group
  d |= (uint64_t)1 << 46;                    // descriptor version of the tcgen05 family
  d |= (uint64_t)2 << 61;                    // swizzle: 128 bytes
  return d;
}

// Instruction descriptor of kind::f16: BF16 A and B (both K-major), FP32
// accumulator, an M x N tile.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// D[tmem] (+)= A[smem] * B[smem]^T, issued by one thread.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// Arrives once on `bar` when every tcgen05 operation this thread issued so far
// has completed.
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_addr(bar))
               : "memory");
}

// 32 consecutive fp32 columns of this thread's TMEM lane (the warp reads its
// 32 lanes: warp w of a CTA reaches lanes 32*(w%4) .. +31). The load and its
// completion wait are one asm statement, so no use of the registers can be
// scheduled before the data has arrived.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,"
      "%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// The first 1024-byte aligned byte of dynamic shared memory at or after p.
// The offset is added to p itself (no round trip through an integer), so
// the compiler still sees a shared-memory pointer and emits shared-memory
// loads, stores and atomics rather than generic ones.
__device__ __forceinline__ uint8_t *align_1024(uint8_t *p) {
  const uint32_t a = smem_addr(p);
  return p + (((a + 1023u) & ~1023u) - a);
}

// One operand tile of 128 rows x 64 bf16 (128 bytes per row).
constexpr uint32_t kTileBytes = 128 * 128;

// Byte offset of (row, 16-byte chunk) in a K-major 128-byte-swizzled tile.
__host__ __device__ __forceinline__ uint32_t sw128_offset(uint32_t row, uint32_t chunk) {
  return (row >> 3) * 1024u + (row & 7u) * 128u + ((chunk ^ (row & 7u)) << 4);
}

}  // namespace tc
}  // namespace mptc
