// Fifth-generation tensor core helpers (sm_103a inline PTX): tensor-memory
// allocation, tcgen05.mma with shared-memory operand descriptors,
// completion through an mbarrier, and tensor-memory loads.
//
// Operand layout used throughout: the canonical K-major layout without
// swizzle. A matrix of R rows x K 16-bit elements is a grid of core
// matrices of 8 rows x 16 bytes (8 elements); a core matrix is 128
// contiguous bytes (row r at +16 r). `lbo` is the byte step between core
// matrices along K, `sbo` between groups of 8 rows.
#pragma once

namespace chfft {
namespace tc {

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

// Byte offset of element (row, k) of a K-major 16-bit tile with K elements
// per row in the canonical layout (lbo = 128, sbo = K * 16).
__host__ __device__ constexpr unsigned kmajor_offset(int row, int k, int K) {
  return (unsigned)((row >> 3) * (K * 16) + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

// Shared-memory matrix descriptor (no swizzle, base offset 0).
__device__ __forceinline__ unsigned long long smem_desc(unsigned addr, unsigned lbo, unsigned sbo) {
  unsigned long long d = 0;
  d |= (unsigned long long)((addr >> 4) & 0x3FFFu);
  d |= (unsigned long long)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (unsigned long long)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (unsigned long long)1 << 46;  // descriptor version of the sm_100 family
  return d;
}

// Instruction descriptor of kind::f16: FP32 accumulator, A and B both FP16
// (or both BF16), both K-major, shape M x N.
__host__ __device__ constexpr unsigned idesc_f16(int M, int N, bool bf16) {
  return (1u << 4) | ((bf16 ? 1u : 0u) << 7) | ((bf16 ? 1u : 0u) << 10) | ((unsigned)(N >> 3) << 17) |
         ((unsigned)(M >> 4) << 24);
}

// D[tmem] (+)= A[smem] * B[smem]^T, one thread issues.
__device__ __forceinline__ void mma_f16(unsigned d_tmem, unsigned long long a, unsigned long long b, unsigned idesc, unsigned accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

// Arrives once on the mbarrier when every MMA this thread issued so far is done.
__device__ __forceinline__ void commit(unsigned long long* mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar))
               : "memory");
}

// Whole warp: allocate ncols (power of two >= 32) tensor-memory columns; the
// address lands in *slot (shared memory).
__device__ __forceinline__ void tmem_alloc(unsigned* slot, unsigned ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(unsigned taddr, unsigned ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// Generic-proxy shared-memory writes become visible to the tensor core.
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_init(unsigned long long* b, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long* b, unsigned phase) {
  unsigned ok;
  asm volatile(
      "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(b)), "r"(phase)
      : "memory");
  return ok != 0;
}

// Bounded wait for phase `phase` of the mbarrier: false after `limit` polls.
__device__ __forceinline__ bool mbar_wait(unsigned long long* b, unsigned phase, int limit) {
  for (int i = 0; i < limit; i++) {
    if (mbar_try_wait(b, phase)) return true;
    __nanosleep(64);
  }
  return false;
}

// This warp's 32 lanes x 32 consecutive FP32 columns starting at taddr
// (lane field = 32 * (warp % 4)); thread i receives lane i.
__device__ __forceinline__ void tmem_ld_32x32(unsigned taddr, float* v) {
  unsigned r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,"
      "%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

}  // namespace tc
}  // namespace chfft
