// acg_edge_tc.cu -- the edge phase of an FP32 BP iteration with the edge costs
// recomputed on the tensor cores instead of read from a stored cost matrix.
//
// It computes what edge_max_kernel computes from dE (ac.hxx:115-149 via
// main.cu:207-224, restructured as the segmented maximum over the
// destination-sorted CSR):
//     M[v][q] = max_{e in in(v)} z[s_e][q] - d(e, q),   d(e, q) = ||x_e - y_q||
// but forms d from the FP32 edge features (dst-CSR order, [De][KM]) and the
// pattern's edge features, with exactly the arithmetic of cdist_tc_kernel
// (acg_cdist_tc.cu; operands and rule in acg_tc.cuh): d2 = nx + ny - 2 x.y
// accumulated on tcgen05.mma from centred TF32-split features and norms, the
// exact difference-form recompute of near pairs (8 d2 < nx + ny), d = d2 *
// rsqrt(d2).  So M is the value the stored-matrix path gives, while the
// iteration reads ~72 bytes per in-edge (features and source) instead of
// Pp * 4 + 4.
//
// Work: the in-edges are cut into items (a vertex's in-edges, or 128-position
// chunks of a heavy vertex's, which reduce through partial rows), and the
// items into one contiguous part per CTA of near-equal cost.  A CTA walks its
// part's positions in tiles of 128, each tile through a pipeline of roles
// that run concurrently, each on its own tiles, handing tiles on through
// shared-memory rings:
//   loader (1 thread)   feature rows [128][KM] by cp.async.bulk (TMA) into a
//                       3-slot ring
//   split (8 warps)     TF32 split of a tile's rows into A' (a row's two halves
//                       by two threads), the row norms; one thread issues the
//                       tile's MMAs into one of two TMEM accumulators and
//                       commits them to an mbarrier
//   gather (2 warps)    the gathered z rows of a tile, z[s_e][0 .. Pp), by
//                       cp.async (two rows per instruction, 16 bytes a lane)
//                       into a 4-slot ring, completing on an mbarrier; the
//                       sources are loaded two tiles ahead
//   epilogue (8 warps)  tcgen05.ld the accumulator (lane quarter w % 4, 16-column
//                       chunks), form d, overwrite the gathered row with
//                       z - d, publish the tile (a monotonic count)
//   consumers (8 warps) claim items in order; the max over an item's rows of
//                       z - d (lanes: rows x 16-byte columns, four rows in
//                       flight) into M or the item's partial row; the warp
//                       completing a heavy vertex's last chunk combines its
//                       partial rows (after a fence and a per-vertex count,
//                       left at zero); rows consumed are counted per ring slot
//                       (monotonic), which frees the slot for the gather four
//                       tiles on.
// The in-order hand-offs (loader -> split -> MMA -> epilogue, gather ->
// epilogue, epilogue -> split for the accumulator) are mbarriers; the
// consumers, which finish items out of order, use the monotonic counts.  Every
// wait is bounded: on expiry the CTA records an error flag, every role leaves
// its loop (the threads of a role together), the copies and MMAs in flight are
// waited for (bounded) and TMEM is freed.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "acg_device.cuh"
#include "acg_iter.cuh"
#include "acg_tc.cuh"

namespace acg {

namespace {

using namespace tc;

constexpr int kTM = 128;  // positions per tile (the MMA's M)
constexpr int kLoaderWarp = 0;
constexpr int kSplitWarp0 = 1, kSplitWarps = 8;
constexpr int kGatherWarp0 = 9, kGatherWarps = 2;
constexpr int kEpiWarp0 = 11, kEpiWarps = 8;
constexpr int kConsWarp0 = 19, kConsWarps = 8;
constexpr int kWarps = kConsWarp0 + kConsWarps;  // 27
constexpr int kET = kWarps * 32;                 // 864 threads
constexpr int kRing = 4;                         // gathered-row ring slots
constexpr int kMaxCols = 64;

inline __host__ __device__ int zstride_of(int Pp) { return Pp % 8 == 0 ? Pp + 4 : Pp; }

struct EtLayout {
  uint32_t a, b, f, z, nx, y, ny, mean, misc, bar, tslot, total;
  int zstride;
  uint32_t zslot, fslot;
};
__host__ __device__ inline EtLayout et_layout(int KM, int N, int Pp) {
  EtLayout L;
  const uint32_t kp = (uint32_t)dist_kp(KM);
  L.zstride = zstride_of(Pp);
  L.zslot = (uint32_t)kTM * (uint32_t)L.zstride * 4;
  L.fslot = (uint32_t)kTM * (uint32_t)KM * 4;
  uint32_t o = 0;
  L.a = o;     o = al128(o + (uint32_t)kTM * kp * 4);
  L.b = o;     o = al128(o + (uint32_t)N * kp * 4);
  L.f = o;     o = al128(o + 3 * L.fslot);
  L.z = o;     o = al128(o + kRing * L.zslot);
  L.nx = o;    o = al128(o + 2 * kTM * 4);
  L.y = o;     o = al128(o + (uint32_t)N * KM * 4);
  L.ny = o;    o = al128(o + (uint32_t)N * 4);
  L.mean = o;  o = al128(o + 32 * 4);
  L.misc = o;  o = al128(o + 16 * 4);
  L.bar = o;   o = al128(o + 16 * 8);
  L.tslot = o; o = al128(o + 4);
  L.total = o;
  return L;
}

// mbarriers (8 bytes each, in order)
enum { B_FFULL = 0, B_FEMPTY = 3, B_MMA = 6, B_NX = 8, B_ACCFREE = 10, B_ZFULL = 12, B_COUNT = 16 };
// ints in the misc area
enum { M_ABORT = 0, M_VREADY = 1, M_CLAIM = 2, M_FWAITED = 3, M_FISSUED = 4, M_MISSUED = 5,
       M_NYMAX = 6 /* float */, M_CONSUMED = 8 /* .. +kRing */ };

__device__ __forceinline__ void cp16(uint32_t sdst, const void* gsrc) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sdst), "l"(gsrc) : "memory");
}
// arrive on `bar` once this thread's earlier cp.async copies have landed
__device__ __forceinline__ void cp_arrive(uint32_t bar) {
  asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void cp_wait0() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

template <int KM>
__global__ void __launch_bounds__(kET, 1) edge_tc_kernel(const EdgeTcArgs a) {
  constexpr int KP = dist_kp(KM);  // K' padded to the MMA's K step
  constexpr int KB = KM / 4;       // core columns per block
  extern __shared__ __align__(1024) unsigned char sm[];
  const int N = a.N, Pp = a.Pp, P = a.P, K = a.K;
  const EtLayout L = et_layout(KM, N, Pp);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t sb = (uint32_t)__cvta_generic_to_shared(sm);
  float* sA = reinterpret_cast<float*>(sm + L.a);
  float* sB = reinterpret_cast<float*>(sm + L.b);
  float* sZ = reinterpret_cast<float*>(sm + L.z);
  float* snx = reinterpret_cast<float*>(sm + L.nx);
  float* sY = reinterpret_cast<float*>(sm + L.y);
  float* sny = reinterpret_cast<float*>(sm + L.ny);
  float* smean = reinterpret_cast<float*>(sm + L.mean);
  int* smisc = reinterpret_cast<int*>(sm + L.misc);
  int* abort = smisc + M_ABORT;
  auto bar = [&](int i) { return sb + L.bar + 8u * (uint32_t)i; };
  const int zs = L.zstride;
  const int tcols = a.tcols;

  // ---- this CTA's part: items [i0, i1), positions [R0, R1)
  const int i0 = __ldg(a.wsplit + blockIdx.x), i1 = __ldg(a.wsplit + blockIdx.x + 1);
  if (i0 >= i1) return;  // the whole CTA leaves: no barrier or TMEM touched yet
  const int R0 = __ldg(a.items + i0).y, R1 = __ldg(a.items + i1 - 1).z;
  const int T = (R1 - R0 + kTM - 1) / kTM;
  auto rows_of = [&](int t) { return min(kTM, R1 - (R0 + t * kTM)); };

  if (tid == 0) {
    for (int i = 0; i < 3; ++i) {
      mbar_init(bar(B_FFULL + i), 1);
      mbar_init(bar(B_FEMPTY + i), kSplitWarps);  // one arrival per split warp
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(bar(B_MMA + i), 1);
      mbar_init(bar(B_NX + i), kSplitWarps);
      mbar_init(bar(B_ACCFREE + i), kEpiWarps);  // one arrival per epilogue warp
    }
    for (int i = 0; i < kRing; ++i) mbar_init(bar(B_ZFULL + i), kGatherWarps * 32);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    for (int i = 0; i < 16; ++i) smisc[i] = 0;
  }
  if (warp == 0) {
    tmem_alloc(sb + L.tslot, (uint32_t)tcols);
    fence_before();
  }
  // the centre m, the FP32 pattern rows, the centred pattern norms and B' (as
  // cdist_tc_kernel); A' zeroed (its padding columns stay zero)
  for (int k = tid; k < KM; k += kET) {
    float s = 0.f;
    if (k < K)
      for (int q = 0; q < P; ++q) s += (float)a.y[(size_t)q * K + k];
    smean[k] = k < K ? s / (float)P : 0.f;
  }
  for (int i = tid; i < N * KM; i += kET) {
    const int q = i / KM, k = i - q * KM;
    sY[i] = (q < P && k < K) ? (float)a.y[(size_t)q * K + k] : 0.f;
  }
  __syncthreads();
  for (int q = tid; q < N; q += kET) {
    float s = 0.f;
    if (q < P)
      for (int k = 0; k < KM; ++k) {
        const float yc = sY[(size_t)q * KM + k] - smean[k];
        s = fmaf(yc, yc, s);
      }
    sny[q] = s;
  }
  __syncthreads();
  if (tid == 0) {
    float m = 0.f;
    for (int q = 0; q < P; ++q) m = fmaxf(m, sny[q]);
    reinterpret_cast<float*>(smisc)[M_NYMAX] = m;
  }
  for (int i = tid; i < N * KP; i += kET) {
    const int q = i / KP, k = i - q * KP, kk = k % KM;
    const float yk = (q < P && k < 3 * KM) ? sY[(size_t)q * KM + kk] - smean[kk] : 0.f;
    *reinterpret_cast<float*>(reinterpret_cast<unsigned char*>(sB) + kmaj_off(q, k, N)) =
        dist_b_elem(yk, q < P ? sny[q] : 0.f, q < P, k, KM);
  }
  for (int i = tid; i < kTM * KP; i += kET) sA[i] = 0.f;
  fence_proxy_async();  // B' and the zeroed A' before any MMA reads them
  __syncthreads();
  fence_after();
  const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(sm + L.tslot);
  auto give_up = [&]() {
    if (atomicExch(abort, 1) == 0) atomicExch(a.err, 1);
  };

  if (warp == kLoaderWarp) {
    // ---------------- loader: feature tiles, three ahead of the split
    if (lane == 0) {
      for (int t = 0; t < T; ++t) {
        if (t >= 3 && !wait_bar(bar(B_FEMPTY + t % 3), (uint32_t)((t / 3 - 1) & 1), abort)) {
          give_up();
          break;
        }
        fence_proxy_async();  // the split's reads of the slot before the copy rewrites it
        bulk_load(sb + L.f + (uint32_t)(t % 3) * L.fslot, a.x + (size_t)(R0 + t * kTM) * KM,
                  (uint32_t)rows_of(t) * (uint32_t)KM * 4u, bar(B_FFULL + t % 3));
        smisc[M_FISSUED] = t + 1;
      }
    }
  } else if (warp < kSplitWarp0 + kSplitWarps) {
    // ---------------- split: A' and the row norms, then the tile's MMAs
    const int st = tid - kSplitWarp0 * 32, r = st & (kTM - 1), h = st >> 7;
    const uint32_t lboA = (kTM / 8) * 128, lboB = (uint32_t)(N / 8) * 128, sbo = 128;
    const uint32_t idesc = idesc_tf32(kTM, N);
    for (int t = 0; t < T; ++t) {
      bool ok = wait_bar(bar(B_FFULL + t % 3), (uint32_t)((t / 3) & 1), abort);
      if (ok && t >= 1) ok = wait_bar(bar(B_MMA + ((t - 1) & 1)), (uint32_t)(((t - 1) >> 1) & 1), abort);
      if (ok && t >= 2) ok = wait_bar(bar(B_ACCFREE + (t & 1)), (uint32_t)(((t >> 1) - 1) & 1), abort);
      ok = named_bar_and(1, kSplitWarps * 32, ok);  // the split threads leave together or not at all
      if (!ok) {
        give_up();
        break;
      }
      if (st == 0) smisc[M_FWAITED] = t + 1;
      const int nr = rows_of(t);
      if (r < nr) {
        // half 0: the x0 blocks and the norms; half 1: the x1 block
        const float4* xr = reinterpret_cast<const float4*>(sm + L.f + (uint32_t)(t % 3) * L.fslot +
                                                           (uint32_t)r * (uint32_t)KM * 4u);
        unsigned char* A = reinterpret_cast<unsigned char*>(sA);
        const uint32_t rb = (uint32_t)((r >> 3) * 128 + (r & 7) * 16);
        float s = 0.f;
#pragma unroll
        for (int jj = 0; jj < KB; ++jj) {
          const float4 xv = xr[jj];
          const float4 mv = reinterpret_cast<const float4*>(smean)[jj];
          const float c[4] = {xv.x - mv.x, xv.y - mv.y, xv.z - mv.z, xv.w - mv.w};
          float h0[4];
#pragma unroll
          for (int w = 0; w < 4; ++w) h0[w] = tf32_round(c[w]);
          if (h == 0) {
#pragma unroll
            for (int w = 0; w < 4; ++w) s = fmaf(c[w], c[w], s);
            const float4 v0 = make_float4(h0[0], h0[1], h0[2], h0[3]);
            *reinterpret_cast<float4*>(A + (uint32_t)jj * lboA + rb) = v0;
            *reinterpret_cast<float4*>(A + (uint32_t)(2 * KB + jj) * lboA + rb) = v0;
          } else {
            *reinterpret_cast<float4*>(A + (uint32_t)(KB + jj) * lboA + rb) =
                make_float4(tf32_round(c[0] - h0[0]), tf32_round(c[1] - h0[1]), tf32_round(c[2] - h0[2]),
                            tf32_round(c[3] - h0[3]));
          }
        }
        if (h == 0) {
          snx[(t & 1) * kTM + r] = s;
          *reinterpret_cast<float4*>(A + (uint32_t)(3 * KB) * lboA + rb) = dist_a_norms(s);
        }
      } else if (h == 0) {
        snx[(t & 1) * kTM + r] = 0.f;
      }
      __syncwarp();
      if (lane == 0) {  // the warp's reads of the feature slot and writes of the norms are done
        mbar_arrive(bar(B_FEMPTY + t % 3));
        mbar_arrive(bar(B_NX + (t & 1)));
      }
      fence_proxy_async();  // the generic-proxy writes of A' before the MMA reads them
      fence_before();
      named_bar(1, kSplitWarps * 32);
      if (st == 0) {
        fence_after();
        const uint32_t acc = tmem + (uint32_t)(t & 1) * (uint32_t)N;
#pragma unroll
        for (int k8 = 0; k8 < KP / 8; ++k8)
          mma_tf32(acc, smem_desc(sb + L.a + (uint32_t)k8 * 2 * lboA, lboA, sbo),
                   smem_desc(sb + L.b + (uint32_t)k8 * 2 * lboB, lboB, sbo), idesc, k8 > 0);
        commit(bar(B_MMA + (t & 1)));
        smisc[M_MISSUED] = t + 1;
      }
    }
  } else if (warp < kGatherWarp0 + kGatherWarps) {
    // ---------------- gather: z rows of each tile into the ring
    const int gw = warp - kGatherWarp0;
    const int nvec = Pp / 4;  // 16-byte chunks per row
    const int half = lane >> 4, ch = lane & 15;
    // sources of this warp's 64 rows of a tile, two per lane (rows lane and
    // 32 + lane), loaded two tiles ahead of their copies
    auto load_src = [&](int t, int& s0, int& s1) {
      s0 = s1 = 0;
      if (t >= T) return;
      const int nr = rows_of(t), r0 = R0 + t * kTM, ra = gw * 64 + lane;
      if (ra < nr) s0 = __ldg(a.src_of + r0 + ra);
      if (ra + 32 < nr) s1 = __ldg(a.src_of + r0 + ra + 32);
    };
    int sa0, sb0, sa1, sb1;
    load_src(0, sa0, sb0);
    load_src(1, sa1, sb1);
    for (int t = 0; t < T; ++t) {
      const int slot = t % kRing;
      // the slot's previous tile (t - kRing) fully consumed
      if (t >= kRing && !wait_count(smisc + M_CONSUMED + slot, (t / kRing) * kTM, abort)) {
        give_up();
        break;
      }
      const int sa = sa0, sbv = sb0;
      sa0 = sa1;
      sb0 = sb1;
      load_src(t + 2, sa1, sb1);
      const int nr = rows_of(t);
      const uint32_t base = sb + L.z + (uint32_t)slot * L.zslot;
      // two rows per instruction (lanes 0-15 the first, 16-31 the second)
#pragma unroll 4
      for (int i = 0; i < 32; ++i) {
        const int row = gw * 64 + 2 * i + half;
        const int src = i < 16 ? __shfl_sync(0xffffffffu, sa, 2 * i + half)
                               : __shfl_sync(0xffffffffu, sbv, 2 * i + half - 32);
        if (row < nr && ch < nvec)
          cp16(base + (uint32_t)(row * zs + 4 * ch) * 4u, a.z + (size_t)src * Pp + 4 * ch);
      }
      cp_arrive(bar(B_ZFULL + slot));
    }
    cp_wait0();
  } else if (warp < kEpiWarp0 + kEpiWarps) {
    // ---------------- epilogue: z - d in place, the tile published
    const int e = warp - kEpiWarp0;
    const int q4 = warp & 3, half = e >> 2, r = q4 * 32 + lane;
    for (int t = 0; t < T; ++t) {
      const int slot = t % kRing;
      bool ok = wait_bar(bar(B_MMA + (t & 1)), (uint32_t)((t >> 1) & 1), abort);
      if (ok) ok = wait_bar(bar(B_NX + (t & 1)), (uint32_t)((t >> 1) & 1), abort);
      if (ok) ok = wait_bar(bar(B_ZFULL + slot), (uint32_t)((t / kRing) & 1), abort);
      ok = named_bar_and(3, kEpiWarps * 32, ok);  // the epilogue threads leave together
      if (!ok) {
        give_up();
        break;
      }
      fence_after();
      const int nr = rows_of(t);
      const float nx = snx[(t & 1) * kTM + r];
      const float thr = 0.125f * (nx + reinterpret_cast<const float*>(smisc)[M_NYMAX]);
      float* zrow = sZ + (size_t)slot * (L.zslot / 4) + (size_t)r * zs;
      const long long erow = (long long)(R0 + t * kTM) + r;
      for (int c = half; c < N / 16; c += 2) {
        uint32_t v[16];
        ld16(tmem + ((uint32_t)(q4 * 32) << 16) + (uint32_t)(t & 1) * (uint32_t)N + (uint32_t)c * 16, v);
        wait_ld();
        if (r >= nr || c * 16 >= Pp) continue;
        // every pair of the chunk far (8 d2 > nx + ny for all of them, which
        // 8 min d2 > nx + max ny implies; d2 > 0 then): d2 * rsqrt(d2);
        // otherwise the rule pair by pair (acg_tc.cuh dist_finish)
        float mn = __uint_as_float(v[0]);
#pragma unroll
        for (int jj = 1; jj < 16; ++jj) mn = fminf(mn, __uint_as_float(v[jj]));
        float d[16];
        if (mn > thr) {
#pragma unroll
          for (int jj = 0; jj < 16; ++jj) {
            const float d2 = __uint_as_float(v[jj]);
            d[jj] = d2 * rsqrtf(d2);
          }
        } else {
          const float* xr = a.x + (size_t)erow * KM;
#pragma unroll
          for (int jj = 0; jj < 16; ++jj) {
            const int q = c * 16 + jj;
            d[jj] = q < P ? dist_finish<KM>(__uint_as_float(v[jj]), nx + sny[q], xr, sY + (size_t)q * KM) : 0.f;
          }
        }
#pragma unroll
        for (int j4 = 0; j4 < 4; ++j4) {
          if (c * 16 + 4 * j4 < Pp) {
            float4* zp = reinterpret_cast<float4*>(zrow + c * 16 + 4 * j4);
            float4 zv = *zp;
            zv.x -= d[4 * j4];
            zv.y -= d[4 * j4 + 1];
            zv.z -= d[4 * j4 + 2];
            zv.w -= d[4 * j4 + 3];
            *zp = zv;
          }
        }
      }
      fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(bar(B_ACCFREE + (t & 1)));  // the accumulator and the tile's norms are free
      named_bar(2, kEpiWarps * 32);
      if (e == 0 && lane == 0) {
        __threadfence_block();
        *reinterpret_cast<volatile int*>(smisc + M_VREADY) = t + 1;  // the tile's rows hold z - d
      }
    }
  } else {
    // ---------------- consumers: the maximum over each item's rows
    const int nvec = Pp / 4;
    int npow = 1;
    while (npow < nvec) npow <<= 1;
    const int S = 32 / npow;  // rows per instruction
    const int rs = lane / npow, cv = lane % npow;
    const bool con = cv < nvec;
    for (;;) {
      int c = 0;
      if (lane == 0) c = atomicAdd(smisc + M_CLAIM, 1);
      const int it = i0 + __shfl_sync(0xffffffffu, c, 0);
      if (it >= i1 || ld_volatile(abort)) break;
      const int4 item = __ldg(a.items + it);
      const int ta = (item.y - R0) / kTM, tb = (item.z - 1 - R0) / kTM;
      if (!__all_sync(0xffffffffu, wait_count(smisc + M_VREADY, tb + 1, abort))) {
        if (lane == 0) give_up();
        break;
      }
      // four rows per lane in flight (independent maxima), merged at the end
      float4 acc[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) acc[u] = make_float4(-CUDART_INF_F, -CUDART_INF_F, -CUDART_INF_F, -CUDART_INF_F);
      if (con) {
        for (int p0 = item.y + rs; p0 < item.z; p0 += 4 * S) {
          float4 x[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const int p = p0 + u * S;
            if (p < item.z) {
              const int rel = p - R0, tt = rel >> 7;
              x[u] = *reinterpret_cast<const float4*>(sZ + (size_t)(tt % kRing) * (L.zslot / 4) +
                                                      (size_t)(rel & (kTM - 1)) * zs + 4 * cv);
            } else {
              x[u] = acc[u];
            }
          }
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            acc[u].x = fmaxf(acc[u].x, x[u].x);
            acc[u].y = fmaxf(acc[u].y, x[u].y);
            acc[u].z = fmaxf(acc[u].z, x[u].z);
            acc[u].w = fmaxf(acc[u].w, x[u].w);
          }
        }
      }
#pragma unroll
      for (int u = 1; u < 4; ++u) {
        acc[0].x = fmaxf(acc[0].x, acc[u].x);
        acc[0].y = fmaxf(acc[0].y, acc[u].y);
        acc[0].z = fmaxf(acc[0].z, acc[u].z);
        acc[0].w = fmaxf(acc[0].w, acc[u].w);
      }
      float4 m = acc[0];
      for (int o = npow; o < 32; o <<= 1) {
        m.x = fmaxf(m.x, __shfl_xor_sync(0xffffffffu, m.x, o));
        m.y = fmaxf(m.y, __shfl_xor_sync(0xffffffffu, m.y, o));
        m.z = fmaxf(m.z, __shfl_xor_sync(0xffffffffu, m.z, o));
        m.w = fmaxf(m.w, __shfl_xor_sync(0xffffffffu, m.w, o));
      }
      // the rows are read: count them consumed (the gather may rewrite the slot)
      if (lane == 0) {
        __threadfence_block();
        const int split = min(item.z, R0 + (ta + 1) * kTM);
        atomicAdd(smisc + M_CONSUMED + ta % kRing, split - item.y);
        if (tb != ta) atomicAdd(smisc + M_CONSUMED + tb % kRing, item.z - split);
      }
      float* out = item.w >= 0 ? a.partial + (size_t)item.w * Pp : a.M + (size_t)item.x * Pp;
      if (rs == 0 && con) reinterpret_cast<float4*>(out)[cv] = m;
      if (item.w >= 0) {
        // a chunk of a heavy vertex: the warp completing its last chunk
        // combines the partial rows (written by this and other CTAs)
        __threadfence();
        __syncwarp();
        const int hv = __ldg(a.pheavy + item.w);
        const int cnt = __ldg(a.hcount + hv);
        int last = 0;
        if (lane == 0) last = atomicAdd(a.hcnt + hv, 1) == cnt - 1;
        if (__shfl_sync(0xffffffffu, last, 0)) {
          __threadfence();
          const size_t b0 = (size_t)__ldg(a.hbase + hv) * Pp, ov = (size_t)__ldg(a.hvert + hv) * Pp;
          for (int q = lane; q < Pp; q += 32) {
            float mq = -CUDART_INF_F;
            for (int k = 0; k < cnt; ++k) mq = fmaxf(mq, __ldcg(a.partial + b0 + (size_t)k * Pp + q));
            a.M[ov + q] = mq;
          }
          if (lane == 0) a.hcnt[hv] = 0;  // ready for the next launch
        }
      }
    }
  }
  __syncthreads();
  if (ld_volatile(abort)) {
    // copies and MMAs issued and not waited for land before the CTA leaves
    // (at most three feature copies and two MMA commits; bounded waits; the
    // gather threads waited for their row copies themselves)
    if (tid == 0)
      for (int t = smisc[M_FWAITED]; t < smisc[M_FISSUED]; ++t)
        mbar_wait(bar(B_FFULL + t % 3), (uint32_t)((t / 3) & 1));
    if (tid == kSplitWarp0 * 32)
      for (int t = max(0, smisc[M_MISSUED] - 2); t < smisc[M_MISSUED]; ++t)
        mbar_wait(bar(B_MMA + (t & 1)), (uint32_t)((t >> 1) & 1));
    fence_before();
    __syncthreads();
  }
  if (warp == 0) {
    fence_after();
    tmem_dealloc(tmem, (uint32_t)tcols);
  }
}

template <int KM>
acg_status launch_km(const EdgeTcArgs& a, int grid, cudaStream_t s) {
  const EtLayout L = et_layout(KM, a.N, a.Pp);
  ACG_CUDA_TRY(cudaFuncSetAttribute(edge_tc_kernel<KM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)L.total));
  edge_tc_kernel<KM><<<grid, kET, L.total, s>>>(a);
  ACG_LAUNCH_CHECK();
  return ACG_OK;
}

}  // namespace

size_t edge_tc_smem(int kstride, int Pp) {
  const int N = (Pp + 15) / 16 * 16;
  return et_layout(kstride, N, Pp).total;
}

bool edge_tc_eligible(int K, int kstride, int P, int Pp) {
  if (P <= 0 || K < 1 || kstride != (K + 3) / 4 * 4 || kstride > 24 || Pp > kMaxCols || Pp % 4) return false;
  int dev = 0, optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return false;
  return edge_tc_smem(kstride, Pp) <= (size_t)optin;
}

acg_status launch_edge_tc(const EdgeTcArgs& a0, int parts, cudaStream_t s) {
  if (a0.De == 0 || a0.P == 0) return ACG_OK;
  EdgeTcArgs a = a0;
  a.N = (a.Pp + 15) / 16 * 16;
  a.tcols = 2 * a.N <= 32 ? 32 : (2 * a.N <= 64 ? 64 : 128);
  switch (a.KM) {
    case 4: return launch_km<4>(a, parts, s);
    case 8: return launch_km<8>(a, parts, s);
    case 12: return launch_km<12>(a, parts, s);
    case 16: return launch_km<16>(a, parts, s);
    case 20: return launch_km<20>(a, parts, s);
    case 24: return launch_km<24>(a, parts, s);
    default: return set_error(ACG_ERR_UNSUPPORTED, "fused edge phase: feature stride %d", a.KM);
  }
}

}  // namespace acg
