// tc.cuh -- 5th-generation tensor core (tcgen05) building blocks for sm_103a.
//
// Operands are staged by the CTA's threads in shared memory in the canonical
// K-major layout without swizzling: 8-row x 16-byte core matrices, core
// matrices adjacent along M/N 128 bytes apart (SBO), along K (R/8)*128 bytes
// apart (LBO) for an R-row tile.  FP32 data is multiplied as 3xTF32: every
// operand is split into a TF32 high part (round to nearest) and the TF32 of
// the remainder, and A*B ~ Ah*Bh + Ah*Bl + Al*Bh is accumulated in FP32 in
// tensor memory, which keeps about FP32 accuracy.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace pnfam {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// float offset of element (row, k) in a K-major no-swizzle tile of R rows (R % 8 == 0)
__device__ __forceinline__ int cm_off(int row, int k, int R) {
  return ((k >> 2) * (R >> 3) + (row >> 3)) * 32 + (row & 7) * 4 + (k & 3);
}

// shared-memory matrix descriptor: start, LBO (K direction), SBO (M/N direction), no swizzle
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// instruction descriptor: kind::tf32, FP32 accumulator, both operands K-major
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ float tf32_hi(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// x = hi + lo with hi the TF32 rounding of x (lo exact in FP32)
__device__ __forceinline__ void split(float x, float& hi, float& lo) {
  hi = tf32_hi(x);
  lo = x - hi;
}

__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// warp-wide: allocate ncols (power of two >= 32) TMEM columns, address written to *slot
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_free(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// bounded wait for the phase with the given parity; false if the limit was reached
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int limit = 1 << 26) {
  for (int i = 0; i < limit; ++i) {
    uint32_t done;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// arrive on the mbarrier and add `bytes` to the transaction count of its current phase
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// bulk copy global -> shared (both 16-byte aligned, bytes a multiple of 16), completion
// counted on the mbarrier's transaction count
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

// D[tmem] (+)= A[smem] * B[smem]^T, issued by one thread
__device__ __forceinline__ void mma_tf32(uint32_t tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, bool acc) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"((uint32_t)acc)
      : "memory");
}

// arrive on the mbarrier when every MMA issued so far by this thread has completed
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// 8 consecutive FP32 columns of this thread's TMEM lane (warp w reads lanes 32*(w%4)..)
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr)
               : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

// two groups of 8 consecutive FP32 columns, one wait
__device__ __forceinline__ void tmem_ld8x2(uint32_t ta, uint32_t tb, float (&va)[8], float (&vb)[8]) {
  uint32_t r[8], q[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(ta)
               : "memory");
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(q[0]), "=r"(q[1]), "=r"(q[2]), "=r"(q[3]), "=r"(q[4]), "=r"(q[5]), "=r"(q[6]), "=r"(q[7])
               : "r"(tb)
               : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 8; ++i) { va[i] = __uint_as_float(r[i]); vb[i] = __uint_as_float(q[i]); }
}

}  // namespace tc

// operand staging helpers: four consecutive floats of one row (mesh points r..r+3 of
// one state), zero outside the mesh or when !ok
__device__ __forceinline__ float4 ld_row4(const float* __restrict__ src, int r, int nghl, bool ok) {
  float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
  if (!ok) return v;
  if ((nghl & 3) == 0 && r + 3 < nghl) return *reinterpret_cast<const float4*>(src + r);
  if (r < nghl) v.x = src[r];
  if (r + 1 < nghl) v.y = src[r + 1];
  if (r + 2 < nghl) v.z = src[r + 2];
  if (r + 3 < nghl) v.w = src[r + 3];
  return v;
}

__device__ __forceinline__ void st_split4(float* hi, float* lo, float4 v) {
  float4 h, l;
  tc::split(v.x, h.x, l.x); tc::split(v.y, h.y, l.y); tc::split(v.z, h.z, l.z); tc::split(v.w, h.w, l.w);
  *reinterpret_cast<float4*>(hi) = h;
  *reinterpret_cast<float4*>(lo) = l;
}

__device__ __forceinline__ void fma4(float4& acc, float4 m, float4 f) {
  acc.x = fmaf(m.x, f.x, acc.x); acc.y = fmaf(m.y, f.y, acc.y);
  acc.z = fmaf(m.z, f.z, acc.z); acc.w = fmaf(m.w, f.w, acc.w);
}

}  // namespace pnfam
