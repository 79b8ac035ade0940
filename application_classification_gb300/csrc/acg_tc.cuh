// acg_tc.cuh -- tcgen05 / bulk-copy / mbarrier primitives (inline PTX) shared by
// the tensor-core kernels (acg_cdist_tc.cu, acg_edge_tc.cu).
//
// Operands of kind::tf32 MMAs are K-major in the no-swizzle canonical layout:
// core matrices of 8 rows x 16 bytes (4 TF32), stored [k / 4][row / 8][row %
// 8][k % 4].  Adjacent core matrices along K are rows/8 * 128 bytes apart (the
// descriptor's leading byte offset), along M/N 128 bytes apart (its stride
// byte offset).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace acg {
namespace tc {

constexpr long long kSpin = 1LL << 22;  // try_wait rounds before a wait gives up

__host__ __device__ inline uint32_t al128(uint32_t v) { return (v + 127u) & ~127u; }

// Byte offset of element (row, k) of a K-major operand with `rows` rows.
__device__ __forceinline__ uint32_t kmaj_off(int row, int k, int rows) {
  return (uint32_t)(((k >> 2) * (rows >> 3) + (row >> 3)) * 128 + (row & 7) * 16 + (k & 3) * 4);
}

// Shared-memory matrix descriptor: start, leading and stride byte offsets
// (>> 4), descriptor version 1 (bits 46-47), base offset 0, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::tf32: D FP32 (bits 4-5 = 1), A and B TF32
// (bits 7-9, 10-12 = 2), both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ inline uint32_t idesc_tf32(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ float tf32_round(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
// Wait for the phase with the given parity to complete; false if it has not
// after kSpin rounds.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (long long i = 0; i < kSpin; ++i) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}
// Role synchronisation of the warp-specialised kernels: named barriers over a
// role's threads, arrivals, and waits that also give up once another role has
// recorded an abort in shared memory.
__device__ __forceinline__ void named_bar(int id, int n) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory");
}
// Named barrier over n threads that also ANDs a predicate across them.
__device__ __forceinline__ bool named_bar_and(int id, int n, bool pred) {
  uint32_t r;
  asm volatile(
      "{\n .reg .pred p, q;\n setp.ne.u32 q, %1, 0;\n barrier.red.and.pred p, %2, %3, q;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(r)
      : "r"((uint32_t)pred), "r"(id), "r"(n)
      : "memory");
  return r != 0;
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ int ld_volatile(const int* p) { return *reinterpret_cast<const volatile int*>(p); }

// Bounded wait on an mbarrier phase that also gives up when another role has
// recorded an abort.
__device__ __forceinline__ bool wait_bar(uint32_t bar, uint32_t parity, const int* abort) {
  for (long long i = 0; i < kSpin; ++i) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
    if ((i & 63) == 63 && ld_volatile(abort)) return false;
  }
  return false;
}
// Bounded wait until *p >= target (a monotonic count in shared memory).
__device__ __forceinline__ bool wait_count(const int* p, int target, const int* abort) {
  for (long long i = 0; i < kSpin; ++i) {
    if (ld_volatile(p) >= target) {
      __threadfence_block();
      return true;
    }
    if (ld_volatile(abort)) return false;
    __nanosleep(32);
  }
  return false;
}

// Bulk copy global -> shared completing on `bar` (which expects `bytes`).
// dst, src 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_load(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
      "l"(src), "r"(bytes), "r"(bar)
      : "memory");
}
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void mma_tf32(uint32_t tmem, uint64_t ad, uint64_t bd, uint32_t idesc, int acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
      "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
      : "memory");
}
// Arrive on `bar` once every MMA this thread issued before has completed.
__device__ __forceinline__ void commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
               : "memory");
}
// 16 consecutive TMEM columns of this warp's 32 lanes (no wait).
__device__ __forceinline__ void ld16(uint32_t taddr, uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
      "[%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
        "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
        "=r"(v[15])
      : "r"(taddr)
      : "memory");
}
__device__ __forceinline__ void wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// TMEM allocation of `cols` columns (a power of two >= 32) by one whole warp;
// the address lands in shared memory at `slot`.
__device__ __forceinline__ void tmem_alloc(uint32_t slot, uint32_t cols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot), "r"(cols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t tmem, uint32_t cols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(cols) : "memory");
}

// ---- the distance MMA shared by the edge cost matrix (acg_cdist_tc.cu) and
// the edge phase that recomputes it (acg_edge_tc.cu).  With x, y centred on
// the mean pattern feature vector and split into TF32 parts (x0 = tf32(x),
// x1 = tf32(x - x0), likewise y), the operands along K are
//     A' = [x0 | x1 | x0 | nx0 nx1 1 1],  B' = [-2y0 | -2y0 | -2y1 | 1 1 ny0 ny1]
// in blocks of KM (the feature dimension padded to 4), nx = ||x||^2 and
// ny = ||y||^2 in FP32 split the same way, so one accumulator holds
//     d2 = nx + ny - 2 (x0.y0 + x1.y0 + x0.y1)       (x1.y1 ~ 2^-22 relative, dropped)
// and K' = 3 KM + 4 padded to the MMA's K step of 8.
__host__ __device__ constexpr int dist_kp(int KM) { return (3 * KM + 4 + 7) / 8 * 8; }

// Element k of row q of B' from yk, the centred FP32 feature k % KM of pattern
// row q (k < 3 KM), the row's norm ny, and whether the row exists (pad rows:
// zero but for the two 1s, so their d2 is nx).
__device__ __forceinline__ float dist_b_elem(float yk, float ny, bool real, int k, int KM) {
  if (k < 3 * KM) {
    if (!real) return 0.f;
    const float y0 = tf32_round(yk);
    return -2.f * (k >= 2 * KM ? tf32_round(yk - y0) : y0);
  }
  const int e = k - 3 * KM;
  if (e == 0 || e == 1) return 1.f;
  if (!real || e > 3) return 0.f;
  const float n0 = tf32_round(ny);
  return e == 2 ? n0 : tf32_round(ny - n0);
}

// The norm block of a row of A': (nx0, nx1, 1, 1).
__device__ __forceinline__ float4 dist_a_norms(float nx) {
  const float n0 = tf32_round(nx);
  return make_float4(n0, tf32_round(nx - n0), 1.f, 1.f);
}

// d from the accumulator's d2 for a pair with pattern row q < P: a pair whose
// d2 is small against its norms (8 d2 < sn = nx + ny: cancellation) is
// recomputed exactly in the difference form from the FP32 rows xr, yr.
template <int KM>
__device__ __forceinline__ float dist_finish(float d2, float sn, const float* xr, const float* yr) {
  if (8.0f * d2 < sn) {
    float acc = 0.f;
#pragma unroll 1
    for (int k = 0; k < KM; ++k) {
      const float u = xr[k] - yr[k];
      acc = fmaf(u, u, acc);
    }
    d2 = acc;
  }
  d2 = fmaxf(d2, 0.f);
  return d2 > 0.f ? d2 * rsqrtf(d2) : 0.f;
}

}  // namespace tc
}  // namespace acg
