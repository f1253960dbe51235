// Split-TF32 tensor-core products on sm_103a (tcgen05, TMEM accumulators).
//
// A float32 product X Y is computed as Xh Yh + Xh Yl + Xl Yh, with
// Xh = tf32(X), Xl = tf32(X - Xh) (and the same for Y): three MMAs of
// kind::tf32 accumulating in float32 in tensor memory.  The dropped term
// Xl Yl and the rounding of Xl, Yl leave a relative error near 2^-21 per
// product, float32-like, where a single TF32 MMA would give 2^-11.
//
// Operands live in shared memory in the K-major, unswizzled canonical layout
// of tcgen05: "slabs" of four consecutive k (16 bytes) holding every row,
// element (row, k) of an operand at
//     (k / 4) * slab_bytes + row * 16 + (k % 4) * 4,
// so an 8-row core matrix is 128 contiguous bytes (stride-dimension byte
// offset 128) and the next group of four k is slab_bytes further (leading
// dimension byte offset).  One MMA consumes K = 8, two slabs.  Rows past the
// used ones may hold anything finite or not: they only feed accumulator rows
// or columns that are never read.
//
// One thread issues the MMAs of a product and commits them to an mbarrier;
// every thread waits on the mbarrier with a bounded spin, then reads its
// accumulator row from tensor memory (warp w reads lanes 32 (w % 4) .. + 31).
#pragma once
#include <cstdint>

namespace mpxg {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// tcgen05 shared-memory matrix descriptor, no swizzle, K-major.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo_bytes, uint32_t sbo_bytes) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo_bytes >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo_bytes >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version of tcgen05
  // base offset 0, absolute LBO mode 0, layout type 0 = no swizzle
  return d;
}

// Instruction descriptor of kind::tf32: D float32, A and B TF32, both
// K-major, no negation, dense.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
  return (1u << 4)                      // D format: F32
         | (2u << 7)                    // A format: TF32
         | (2u << 10)                   // B format: TF32
         | ((uint32_t)(N >> 3) << 17)   // N / 8
         | ((uint32_t)(M >> 4) << 24);  // M / 16
}

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// Arrive once on the mbarrier when every MMA this thread issued has completed.
__device__ __forceinline__ void mma_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
               : "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
}

// Bounded wait for the phase with the given parity to complete; false after
// `limit` polls.
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity, int limit) {
  for (int i = 0; i < limit; ++i) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(mbar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// Warp-wide: allocate `ncols` tensor-memory columns (a power of two >= 32);
// the address is written to shared memory at `slot`.
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
__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// Generic-proxy shared-memory writes made visible to the tensor core's reads.
__device__ __forceinline__ void fence_smem_to_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Eight consecutive accumulator columns of this thread's lane (row).
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float* v) {
  uint32_t r[8];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ float tf32_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}
// x = hi + lo, both TF32-representable (up to the rounding of lo).
__device__ __forceinline__ void split(float x, float* hi, float* lo) {
  const float h = tf32_rna(x);
  *hi = h;
  *lo = tf32_rna(x - h);
}

// Byte offset of operand element (row, k) in the slab layout.
__host__ __device__ constexpr uint32_t slab_off(int row, int k, uint32_t slab_bytes) {
  return (uint32_t)(k >> 2) * slab_bytes + (uint32_t)row * 16u + (uint32_t)(k & 3) * 4u;
}

// Issue D (+)= X Y for K = 8 * ksteps from split operands (one thread).
// Xh/Xl: the M-side operand, Yh/Yl: the N-side operand, shared addresses of
// slab 0 of each; slab strides xs, ys bytes.
__device__ __forceinline__ void issue_split_product(uint32_t d_tmem, uint32_t idesc, uint32_t Xh, uint32_t Xl,
                                                    uint32_t xs, uint32_t Yh, uint32_t Yl, uint32_t ys, int ksteps,
                                                    bool accumulate) {
  for (int s = 0; s < ksteps; ++s) {
    const uint32_t xo = 2u * s * xs, yo = 2u * s * ys;
    const uint64_t xh = smem_desc(Xh + xo, xs, 128), xl = smem_desc(Xl + xo, xs, 128);
    const uint64_t yh = smem_desc(Yh + yo, ys, 128), yl = smem_desc(Yl + yo, ys, 128);
    mma_tf32(d_tmem, xh, yh, idesc, (accumulate || s > 0) ? 1u : 0u);
    mma_tf32(d_tmem, xh, yl, idesc, 1u);
    mma_tf32(d_tmem, xl, yh, idesc, 1u);
  }
}

}  // namespace tc
}  // namespace mpxg
