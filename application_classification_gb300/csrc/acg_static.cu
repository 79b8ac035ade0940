// acg_static.cu -- the static per-vertex reductions of a match.
//
// The reference builds, once per match, the quirk buffers and their edge
// maxima (main.cu:113-114, 135-146: RowSoftmax2 + EdgeMaxReduce2_t over the
// negated cost matrix); the restructured iteration also needs, per data vertex
// v and pattern edge q, dEmin = min over v's out-edges of dE and
// B = log sum over v's out-edges of exp(-dE).  Both sides are segmented
// reductions over a CSR and use the edge phase's structure (acg_iter.cu):
// one warp per work item, lanes = (edge slot, 16-byte column), kU loads per
// slot issued back to back with the next step's row indices in flight,
// static cost-balanced warp ranges, hubs split into chunks whose partial rows
// are combined in chunk order.
//   src_stats_kernel  out-edges (source-sorted CSR, dE rows gathered from
//                     their destination-sorted position): dEmin, B, and the
//                     quirk maximum of the columns q < qcov
//   dst_quirk_kernel  in-edges (consecutive destination-sorted rows): the
//                     quirk maximum of the columns q < qcov only; the other
//                     columns of the quirk buffer are all zero
#include <cuda_runtime.h>

#include <cstdint>

#include "acg_bp.cuh"
#include "acg_device.cuh"
#include "acg_static.cuh"

namespace acg {

namespace {

constexpr int kST = 256;  // threads per block (the edge phase's warp work uses 8 warps per block)
#ifndef ACG_SRC_KU
#define ACG_SRC_KU 4
#endif
// An explicit minimum of one block per SM (the compiler then keeps more of the
// pipelined loads in registers): static passes 14.3 -> 10.3 ms at RMAT-22.
#ifndef ACG_SRC_MINB
#define ACG_SRC_MINB 1
#endif
constexpr int kSU = ACG_SRC_KU;  // load steps issued back to back

template <typename T>
struct SV;
template <>
struct SV<double> {
  using type = double2;
  static constexpr int W = 2;
};
template <>
struct SV<float> {
  using type = float4;
  static constexpr int W = 4;
};
template <typename T>
__device__ __forceinline__ T sg(const typename SV<T>::type& v, int w) {
  return reinterpret_cast<const T*>(&v)[w];
}
template <typename T>
__device__ __forceinline__ typename SV<T>::type sfill(T x) {
  typename SV<T>::type r;
#pragma unroll
  for (int w = 0; w < SV<T>::W; ++w) reinterpret_cast<T*>(&r)[w] = x;
  return r;
}

__device__ __forceinline__ float exp_fast(float x) { return __expf(x); }
__device__ __forceinline__ double exp_fast(double x) { return exp(x); }
template <typename T>
__device__ __forceinline__ void kahan_add(T& s, T& c, T x) {
  const T y = x - c;
  const T t = s + y;
  c = (t - s) - y;
  s = t;
}

// Largest dEmin for which exp(-dE) of the nearest out-edge is still a normal
// number; above it a column's sum is redone relative to its minimum.
template <typename T>
__device__ __forceinline__ T exp_ref_limit() { return sizeof(T) == 4 ? T(60) : T(600); }

// The FP32 one-vector-per-lane shapes stage the gathered dE rows through a
// per-warp ring in shared memory with cp.async: a stage is one step's positions
// (S * kSU rows, 2 KB), issued kSrcAhead stages ahead of the step that reads
// it, so the rows in flight no longer cost registers.
constexpr int kSrcAhead = 3;
constexpr int kSrcSlots = kSrcAhead + 2;  // a step spans at most two stages
constexpr int kSrcStageBytes = 32 * kSU * 16;
template <typename T, int NQV>
__host__ __device__ constexpr bool src_staged() { return sizeof(T) == 4 && NQV == 1; }
template <typename T, int NQV>
__host__ __device__ constexpr size_t src_stage_smem() {
  return src_staged<T, NQV>() ? (size_t)(kST / 32) * kSrcSlots * kSrcStageBytes : 0;
}
__device__ __forceinline__ void src_cp16(void* sdst, const void* gsrc) {
  const uint32_t d = (uint32_t)__cvta_generic_to_shared(sdst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void src_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
// wait until at most n of this thread's copy groups are pending (n <= kSrcAhead)
__device__ __forceinline__ void src_wait(int n) {
  switch (n) {
    case 0: asm volatile("cp.async.wait_group 0;\n" ::: "memory"); break;
    case 1: asm volatile("cp.async.wait_group 1;\n" ::: "memory"); break;
    case 2: asm volatile("cp.async.wait_group 2;\n" ::: "memory"); break;
    default: asm volatile("cp.async.wait_group 3;\n" ::: "memory"); break;
  }
}

#if ACG_SRC_MINB > 0
#define ACG_SRC_BOUNDS __launch_bounds__(kST, ACG_SRC_MINB)
#else
#define ACG_SRC_BOUNDS __launch_bounds__(kST)
#endif
// One range of a warp's items, [it, it_end).
template <typename T, int NPOW, int NQV>
__device__ __forceinline__ void src_stats_range(const SrcStatsArgs<T>& a, int it, const int it_end,
                                                const int slot, const int qc) {
  using VT = typename SV<T>::type;
  constexpr int W = SV<T>::W;
  constexpr int S = 32 / NPOW;
  constexpr int NQ = NQV * W;
  constexpr int STEP = S * kSU;
  const int Pp = a.Pp, Pqc = a.Pqc, qcov = a.qcov;
  if (it >= it_end) return;

  int4 item = __ldg(a.items + it);
  int4 item_next = it + 1 < it_end ? __ldg(a.items + it + 1) : make_int4(0, 0, 0, -1);
  int base = item.y;
  int ridx[kSU], eidx[kSU];
#pragma unroll
  for (int u = 0; u < kSU; ++u) {
    const int e = base + slot + S * u;
    const bool ok = e < item.z;
    ridx[u] = ok && !src_staged<T, NQV>() ? __ldg(a.row_of + e) : 0;
    eidx[u] = ok ? __ldg(a.eid + e) : 0;
  }
  // staged: the warp's positions [P0, P1) in stages of STEP rows, stage j in
  // ring slot j % kSrcSlots
  const int lane = threadIdx.x & 31;
  const int P0 = item.y;
  const int P1 = src_staged<T, NQV>() ? __ldg(a.items + it_end - 1).z : 0;
  const int nst = (P1 - P0 + STEP - 1) / STEP;
  VT* ring = nullptr;
  int issued = 0;
  // dE rows of the next stage to issue, loaded one stage ahead of their copies
  int nrow[kSU];
  auto load_rows = [&](int j) {
#pragma unroll
    for (int i = 0; i < kSU; ++i) {
      const int e = P0 + j * STEP + (lane + 32 * i) / NPOW;
      nrow[i] = j < nst && e < P1 ? __ldg(a.row_of + e) : 0;
    }
  };
  auto issue_stage = [&]() {  // stage `issued`: STEP rows x NPOW chunks, kSU 16-byte chunks a lane
    if (issued < nst) {
      VT* dst = ring + (size_t)(issued % kSrcSlots) * (kSrcStageBytes / 16);
#pragma unroll
      for (int i = 0; i < kSU; ++i) {
        const int c = lane + 32 * i, row = c / NPOW, qv = c % NPOW;
        const int e = P0 + issued * STEP + row;
        if (e < P1 && qv * W < Pp)
          src_cp16(dst + c, reinterpret_cast<const VT*>(a.dE + (size_t)nrow[i] * Pp) + qv);
      }
    }
    src_commit();  // one group per stage (empty past the range)
    ++issued;
    load_rows(issued);
  };
  if constexpr (src_staged<T, NQV>()) {
    extern __shared__ __align__(16) unsigned char src_ring[];
    ring = reinterpret_cast<VT*>(src_ring) + (size_t)(threadIdx.x >> 5) * kSrcSlots * (kSrcStageBytes / 16);
    load_rows(0);
    for (int j = 0; j < kSrcAhead; ++j) issue_stage();
  }
  // Per column: the minimum mn of dE and sum_i exp(-dE_i) (with a compensation
  // term; -dE <= 0, so the sum cannot overflow): one exponential and no branch
  // per element.  A column whose nearest edge is so far (mn above
  // exp_ref_limit) that the terms leave the normal range is summed again
  // relative to its minimum, which is rare and uniform across the warp.
  T mn[NQ], qx[NQ], sm[NQ], sc[NQ];
  // quirk coverage of column q: original edge id < lim - q * De (no edge for
  // the columns q >= qcov, whose quirk value is never read)
  long long qlim[NQ];
#pragma unroll
  for (int k = 0; k < NQ; ++k) {
    mn[k] = pos_inf<T>();
    qx[k] = neg_inf<T>();
    sm[k] = T(0);
    sc[k] = T(0);
    const int q = (qc + NPOW * (k / W)) * W + k % W;
    qlim[k] = q < qcov ? __ldg(a.qlim_col + q) : 0;
  }
  for (;;) {
    VT x[kSU][NQV];
    bool okv[kSU];
    int ecur[kSU];
    if constexpr (src_staged<T, NQV>()) {
      // the stages this step reads (its first and last position's) in place,
      // kSrcAhead more in flight
      const int jlo = (base - P0) / STEP, jhi = min(nst - 1, (base + STEP - 1 - P0) / STEP);
      __syncwarp();  // every lane is done with the slot the next issue rewrites
      while (issued < jhi + 1 + kSrcAhead) issue_stage();
      src_wait(issued - 1 - jhi);
      __syncwarp();  // the other lanes' copies are visible
#pragma unroll
      for (int u = 0; u < kSU; ++u) {
        const int e = base + slot + S * u;
        okv[u] = e < item.z;
        ecur[u] = eidx[u];
        const int rel = e - P0, j = rel / STEP;
        (void)jlo;
        x[u][0] = (okv[u] && qc * W < Pp)
                      ? ring[(size_t)(j % kSrcSlots) * (kSrcStageBytes / 16) + (rel - j * STEP) * NPOW + qc]
                      : sfill<T>(pos_inf<T>());
      }
    } else {
#pragma unroll
      for (int u = 0; u < kSU; ++u) {
        const int e = base + slot + S * u;
        okv[u] = e < item.z;
        ecur[u] = eidx[u];
#pragma unroll
        for (int k = 0; k < NQV; ++k) {
          const int qv = qc + NPOW * k;
          x[u][k] = (okv[u] && qv * W < Pp)
                        ? __ldg(reinterpret_cast<const VT*>(a.dE + (size_t)ridx[u] * Pp) + qv)
                        : sfill<T>(pos_inf<T>());
        }
      }
    }
    const bool item_done = base + STEP >= item.z;
    int nbase = base + STEP, nend = item.z;
    bool more = true;
    if (item_done) {
      more = it + 1 < it_end;
      nbase = item_next.y;
      nend = item_next.z;
    }
#pragma unroll
    for (int u = 0; u < kSU; ++u) {
      const int e = nbase + slot + S * u;
      const bool ok = more && e < nend;
      ridx[u] = ok && !src_staged<T, NQV>() ? __ldg(a.row_of + e) : 0;
      eidx[u] = ok ? __ldg(a.eid + e) : 0;
    }
    // branch-free: a missing edge reads +inf, which changes no minimum, adds
    // exp(-inf) = 0 and gives a quirk value of -inf
#pragma unroll
    for (int u = 0; u < kSU; ++u)
#pragma unroll
      for (int k = 0; k < NQV; ++k)
#pragma unroll
        for (int w = 0; w < W; ++w) {
          const T d = sg<T>(x[u][k], w);
          const int j = k * W + w;
          mn[j] = fmin(mn[j], d);
          kahan_add(sm[j], sc[j], exp_fast(-d));
          qx[j] = fmax(qx[j], (long long)ecur[u] < qlim[j] ? -d : T(0));
        }
    if (item_done) {
      T lm[NQ], lsum[NQ];  // the column's (reference, sum of exp(-dE - reference))
#pragma unroll
      for (int k = 0; k < NQ; ++k) lsum[k] = sm[k] - sc[k];
#pragma unroll
      for (int o = NPOW; o < 32; o <<= 1)
#pragma unroll
        for (int k = 0; k < NQ; ++k) {
          mn[k] = fmin(mn[k], __shfl_xor_sync(0xffffffffu, mn[k], o));
          qx[k] = fmax(qx[k], __shfl_xor_sync(0xffffffffu, qx[k], o));
          lsum[k] += __shfl_xor_sync(0xffffffffu, lsum[k], o);
        }
      bool far = false;
#pragma unroll
      for (int k = 0; k < NQ; ++k) {
        lm[k] = T(0);
        far |= mn[k] > exp_ref_limit<T>() && mn[k] < pos_inf<T>();
      }
      if (__any_sync(0xffffffffu, far)) {
        // sum exp(mn - dE) again over this item's edges, for every column
#pragma unroll
        for (int k = 0; k < NQ; ++k) {
          sm[k] = T(0);
          sc[k] = T(0);
        }
        for (int e = item.y + slot; e < item.z; e += S) {
          const T* row = a.dE + (size_t)__ldg(a.row_of + e) * Pp;
#pragma unroll
          for (int k = 0; k < NQV; ++k) {
            const int qv = qc + NPOW * k;
            if (qv * W >= Pp) continue;
            const VT xv = __ldg(reinterpret_cast<const VT*>(row) + qv);
#pragma unroll
            for (int w = 0; w < W; ++w)
              kahan_add(sm[k * W + w], sc[k * W + w], exp_fast(mn[k * W + w] - sg<T>(xv, w)));
          }
        }
#pragma unroll
        for (int k = 0; k < NQ; ++k) {
          lsum[k] = sm[k] - sc[k];
          lm[k] = -mn[k];
        }
#pragma unroll
        for (int o = NPOW; o < 32; o <<= 1)
#pragma unroll
          for (int k = 0; k < NQ; ++k) lsum[k] += __shfl_xor_sync(0xffffffffu, lsum[k], o);
      }
      if (slot == 0) {
        const int v = item.x;
#pragma unroll
        for (int k = 0; k < NQV; ++k)
#pragma unroll
          for (int w = 0; w < W; ++w) {
            const int q = (qc + NPOW * k) * W + w;
            if (q >= Pp) continue;
            const int j = k * W + w;
            if (item.w >= 0) {
              T* pr = a.partial + (size_t)item.w * (3 * Pp + Pqc);
              pr[q] = mn[j];
              pr[Pp + q] = lm[j];
              pr[2 * Pp + q] = lsum[j];
              if (q < Pqc) pr[3 * Pp + q] = qx[j];
            } else {
              a.dEmin[(size_t)v * Pp + q] = mn[j];
              a.B[(size_t)v * Pp + q] =
                  (lm[j] > neg_inf<T>() && lsum[j] > T(0)) ? lm[j] + dev_log(lsum[j]) : neg_inf<T>();
              if (q < Pqc) a.Rq[(size_t)v * Pqc + q] = qx[j];
            }
          }
      }
#pragma unroll
      for (int k = 0; k < NQ; ++k) {
        mn[k] = pos_inf<T>();
        qx[k] = neg_inf<T>();
        sm[k] = T(0);
        sc[k] = T(0);
      }
      if (!more) break;
      ++it;
      item = item_next;
      item_next = it + 1 < it_end ? __ldg(a.items + it + 1) : make_int4(0, 0, 0, -1);
    }
    base = nbase;
  }
  if constexpr (src_staged<T, NQV>()) {
    src_wait(0);  // nothing of this range in flight when the ring is reused
    __syncwarp();
  }
}

// The warp's own range first, then claimed ones (as edge_max_kernel).
// The staged shapes keep two blocks (16 warps) per SM: their rows in flight sit
// in shared memory, not in registers.
template <typename T, int NPOW, int NQV>
__global__ void __launch_bounds__(kST, src_staged<T, NQV>() ? 2 : (ACG_SRC_MINB > 0 ? ACG_SRC_MINB : 1))
src_stats_kernel(const SrcStatsArgs<T> a) {
  const int lane = threadIdx.x & 31;
  const int slot = lane / NPOW, qc = lane % NPOW;
  const int nw = (int)gridDim.x * (kST / 32);
  const int gw = (blockIdx.x * kST + threadIdx.x) >> 5;
  for (int r = gw; r < a.nranges;) {
    int rn = a.nranges;
    if (a.ctr && lane == 0) rn = nw + atomicAdd(a.ctr, 1);
    src_stats_range<T, NPOW, NQV>(a, __ldg(a.wsplit + r), __ldg(a.wsplit + r + 1), slot, qc);
    r = __shfl_sync(0xffffffffu, rn, 0);
  }
  if (a.ctr && lane == 0) {
    __threadfence();  // this warp's claims come before its finish count
    if (atomicAdd(a.ctr + 1, 1) == nw - 1) {  // every warp has made its last claim
      a.ctr[0] = 0;
      a.ctr[1] = 0;
    }
  }
}

// One warp per heavy vertex: its chunk rows merged in chunk order (FP64).
template <typename T>
__global__ void __launch_bounds__(256)
src_stats_combine_kernel(const SrcStatsArgs<T> a, const int* __restrict__ hbase,
                         const int* __restrict__ hcount, const int* __restrict__ hvert,
                         int nheavy) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= nheavy) return;
  const int Pp = a.Pp, Pqc = a.Pqc;
  const size_t rs = (size_t)3 * Pp + Pqc;
  const T* p0 = a.partial + (size_t)hbase[warp] * rs;
  const int cnt = hcount[warp];
  const size_t v = (size_t)hvert[warp];
  for (int q = lane; q < Pp; q += 32) {
    T mn = pos_inf<T>(), qx = neg_inf<T>();
    double m = -CUDART_INF, s = 0.0;
    for (int r = 0; r < cnt; ++r) {
      const T* pr = p0 + (size_t)r * rs;
      mn = fmin(mn, pr[q]);
      lse_merge(m, s, (double)pr[Pp + q], (double)pr[2 * Pp + q]);
      if (q < Pqc) qx = fmax(qx, pr[3 * Pp + q]);
    }
    a.dEmin[v * Pp + q] = mn;
    a.B[v * Pp + q] = (m > -CUDART_INF && s > 0.0) ? (T)(m + log(s)) : neg_inf<T>();
    if (q < Pqc) a.Rq[v * Pqc + q] = qx;
  }
}

template <typename T, int NPOW, int NQV>
__global__ void __launch_bounds__(kST)
dst_quirk_kernel(const DstQuirkArgs<T> a) {
  using VT = typename SV<T>::type;
  constexpr int W = SV<T>::W;
  constexpr int S = 32 / NPOW;
  constexpr int NQ = NQV * W;
  constexpr int STEP = S * kSU;
  extern __shared__ __align__(16) unsigned char smem_q[];
  const int Pp = a.Pp, Pqc = a.Pqc, qcov = a.qcov;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int slot = lane / NPOW, qc = lane % NPOW;
  const int gw = (blockIdx.x * kST + threadIdx.x) >> 5;
  const int nw = (int)gridDim.x * (kST / 32);
  T qx[NQ];
  long long qlim[NQ];
  // LSE of -dE over the covered elements of each column (the reference's
  // first softmax of its RE/FE buffers, main.cu:113-114, 135-146)
  OnlineLse<T> ls[NQ];
#pragma unroll
  for (int k = 0; k < NQ; ++k) {
    qx[k] = neg_inf<T>();
    ls[k].init();
    const int q = (qc + NPOW * (k / W)) * W + k % W;
    qlim[k] = q < qcov ? __ldg(a.qlim_col + q) : 0;
  }
  for (int r = gw; r < a.nranges; r += nw) {
    const int it_end = __ldg(a.wsplit + r + 1);
    int it = __ldg(a.wsplit + r);
    if (it >= it_end) continue;
    int4 item = __ldg(a.items + it);
    int base = item.y;
    for (;;) {
      VT x[kSU][NQV];
      int ev[kSU];
#pragma unroll
      for (int u = 0; u < kSU; ++u) {
        const int e = base + slot + S * u;
        const bool ok = e < item.z;
        ev[u] = ok ? __ldg(a.eid + e) : 0;
#pragma unroll
        for (int k = 0; k < NQV; ++k) {
          const int qv = qc + NPOW * k;
          x[u][k] = (ok && qv * W < Pqc)
                        ? __ldcs(reinterpret_cast<const VT*>(a.dE + (size_t)e * (a.dstride ? a.dstride : Pp)) + qv)
                        : sfill<T>(pos_inf<T>());
        }
      }
      // a missing edge reads +inf: quirk value -inf, nothing added
#pragma unroll
      for (int u = 0; u < kSU; ++u)
#pragma unroll
        for (int k = 0; k < NQV; ++k)
#pragma unroll
          for (int w = 0; w < W; ++w) {
            const int j = k * W + w;
            const T d = sg<T>(x[u][k], w);
            const bool covered = (long long)ev[u] < qlim[j];
            qx[j] = fmax(qx[j], covered ? -d : T(0));
            if (covered) ls[j].add(-d);
          }
      if (base + STEP >= item.z) {
#pragma unroll
        for (int o = NPOW; o < 32; o <<= 1)
#pragma unroll
          for (int k = 0; k < NQ; ++k) qx[k] = fmax(qx[k], __shfl_xor_sync(0xffffffffu, qx[k], o));
        if (slot == 0) {
          T* row = item.w >= 0 ? a.partial + (size_t)item.w * Pqc : a.Fq + (size_t)item.x * Pqc;
#pragma unroll
          for (int k = 0; k < NQV; ++k)
#pragma unroll
            for (int w = 0; w < W; ++w) {
              const int q = (qc + NPOW * k) * W + w;
              if (q < Pqc) row[q] = qx[k * W + w];
            }
        }
#pragma unroll
        for (int k = 0; k < NQ; ++k) qx[k] = neg_inf<T>();
        if (++it >= it_end) break;
        item = __ldg(a.items + it);
        base = item.y;
      } else {
        base += STEP;
      }
    }
  }
  // column log-sum-exps: slots merged across the warp, warps in order
  double* red = reinterpret_cast<double*>(smem_q);  // [warp][2 Pqc]
#pragma unroll
  for (int k = 0; k < NQ; ++k) {
    double m = ls[k].mval(), sv = ls[k].sval();
#pragma unroll
    for (int o = NPOW; o < 32; o <<= 1) {
      const double m2 = __shfl_xor_sync(0xffffffffu, m, o);
      const double s2 = __shfl_xor_sync(0xffffffffu, sv, o);
      lse_merge(m, sv, m2, s2);
    }
    const int q = (qc + NPOW * (k / W)) * W + k % W;
    if (slot == 0 && q < Pqc) {
      red[(size_t)wib * 2 * Pqc + 2 * q] = m;
      red[(size_t)wib * 2 * Pqc + 2 * q + 1] = sv;
    }
  }
  __syncthreads();
  write_block_partials(red, kST / 32, 0, Pqc, a.bpart, gridDim.x, blockIdx.x);
}

// ------------------------------------------------------------ init, warp form
// The first VF, VR of the iteration loop and their statistics (main.cu:112-133,
// 135-146, 165-176): CV = dV - LSE_v(dV), MU0 = -dV - LSE_v(-dV), RMax0 / FMax0
// from the quirk-buffer maxima, Y = VF' - dEmin and Z = VR' (shift 0).  Lanes
// own fixed columns as in the vertex phase's warp form (QPL edge columns,
// PPL pattern vertices); each warp walks a contiguous vertex range with the
// next vertex's rows loaded while the current one is computed.  In FP32 the
// FP64 constants enter as hi/lo pairs and CV, MU0 are formed with TwoSum, so
// that no per-element arithmetic runs at the FP64 rate.
template <typename T>
__device__ __forceinline__ void two_sum(T a, T b, T& s, T& e) {
  s = a + b;
  const T bp = s - a;
  e = (a - (s - bp)) + (b - bp);
}

template <typename T, int QPL, int PPL>
struct InitRow {
  T b[QPL], em[QPL], rq[QPL], fq[QPL], cv[PPL];
};

template <typename T, int QPL, int PPL>
__global__ void __launch_bounds__(kST)
init_warp_kernel(const InitArgs<T> a) {
  constexpr int kW = kST / 32;
  extern __shared__ __align__(16) unsigned char smem[];
  const int Pe = a.Pe, Pn = a.Pn, Pp = a.Pp, Pnp = a.Pnp, Pqc = a.Pqc, qcov = a.qcov, Dn = a.Dn;
  const int tid = threadIdx.x, lane = tid & 31, wib = tid >> 5;
  int* s_pat = reinterpret_cast<int*>(smem);
  const int npat = 4 * Pe + 2 * (Pn + 1);
  T* s_mu = reinterpret_cast<T*>(smem + ((sizeof(int) * (size_t)npat + 15) & ~size_t(15)));
  T* smu = s_mu + (size_t)wib * 64 * PPL;  // hi | lo
  for (int t = tid; t < npat; t += kST) s_pat[t] = a.pat[t];
  __syncthreads();
  const int* s_psrc = s_pat;
  const int* s_pdst = s_pat + Pe;
  const double* gv = a.gv;  // [maxneg(Pn) | lse_pos(Pn) | lse_neg(Pn)]

  const int qo = lane * QPL;
  const bool qon = qo < Pp;
  T vfm[QPL], vrm[QPL], lbh[QPL], lbl[QPL];
  int qd[QPL], qs[QPL];
#pragma unroll
  for (int k = 0; k < QPL; ++k) {
    const int q = qo + k;
    vfm[k] = vrm[k] = lbh[k] = lbl[k] = T(0);
    qd[k] = qs[k] = 0;
    if (q < Pe) {
      qd[k] = s_pdst[q];
      qs[k] = s_psrc[q];
      vfm[k] = (T)(gv[qd[k]] - gv[2 * Pn + qd[k]]);  // max_v MU0[dst_q]
      vrm[k] = (T)(gv[qs[k]] - gv[2 * Pn + qs[k]]);
      // LSE of the whole quirk row q: its covered part, plus exp(0) per zero
      long long covered = a.qlim_col[q];
      covered = covered < 0 ? 0 : (covered > a.De ? a.De : covered);
      LseD r;
      r.init();
      if (a.ge[q] > -CUDART_INF) r.merge(a.ge[q], 1.0);
      const long long zeros = a.De - covered;
      if (zeros > 0) r.merge(0.0, (double)zeros);
      const double lb = r.value();
      lbh[k] = (T)lb;
      lbl[k] = (T)(lb - (double)lbh[k]);
    }
  }
  T l1h[PPL], l1l[PPL], l2h[PPL], l2l[PPL];
#pragma unroll
  for (int j = 0; j < PPL; ++j) {
    const int p = lane + 32 * j;
    const double l1 = p < Pn ? gv[Pn + p] : 0.0, l2 = p < Pn ? gv[2 * Pn + p] : 0.0;
    l1h[j] = (T)l1;
    l1l[j] = (T)(l1 - (double)l1h[j]);
    l2h[j] = (T)l2;
    l2l[j] = (T)(l2 - (double)l2h[j]);
  }
  T mxF[QPL], mxR[QPL];
  OnlineLse<T> lr[QPL], lf[QPL];
#pragma unroll
  for (int k = 0; k < QPL; ++k) {
    mxF[k] = mxR[k] = neg_inf<T>();
    lr[k].init();
    lf[k].init();
  }

  auto load = [&](int v, InitRow<T, QPL, PPL>& r) {
#pragma unroll
    for (int k = 0; k < QPL; ++k) {
      const int q = qo + k;
      const bool on = q < Pp;
      r.b[k] = on ? __ldcs(a.B + (size_t)v * Pp + q) : T(0);
      r.em[k] = on ? __ldcs(a.dEmin + (size_t)v * Pp + q) : T(0);
      r.rq[k] = q < qcov ? __ldcs(a.Rq + (size_t)v * Pqc + q) : T(0);
      r.fq[k] = q < qcov ? __ldcs(a.Fq + (size_t)v * Pqc + q) : T(0);
    }
#pragma unroll
    for (int j = 0; j < PPL; ++j) {
      const int p = lane + 32 * j;
      r.cv[j] = p < Pn ? __ldcs(a.CV + (size_t)v * Pnp + p) : T(0);
    }
  };

  const long long nw = (long long)gridDim.x * kW;
  const long long gw = (long long)blockIdx.x * kW + wib;
  const int vb = (int)(gw * Dn / nw), ve = (int)((gw + 1) * Dn / nw);
  InitRow<T, QPL, PPL> cur, nxt;
  if (vb < ve) load(vb, cur);
  for (int v0 = vb; v0 < ve; v0 += 32) {
    const int nv = min(32, ve - v0);
    bool hi = false, ho = false;
    if (lane < nv) {
      const int v = v0 + lane;
      hi = __ldg(a.d_off + v + 1) > __ldg(a.d_off + v);
      ho = __ldg(a.s_off + v + 1) > __ldg(a.s_off + v);
    }
    const unsigned inmask = __ballot_sync(0xffffffffu, hi);
    const unsigned outmask = __ballot_sync(0xffffffffu, ho);
    for (int jv = 0; jv < nv; ++jv) {
      const int v = v0 + jv;
      if (v + 1 < ve) load(v + 1, nxt);
      // p side: CV = dV - lse1 (hi/lo, written back), MU0 = -dV - lse2 (hi/lo)
#pragma unroll
      for (int j = 0; j < PPL; ++j) {
        const int p = lane + 32 * j;
        T s1, e1, s2, e2;
        two_sum(cur.cv[j], -l1h[j], s1, e1);
        e1 -= l1l[j];
        const T ch = s1 + e1, cl = e1 - (ch - s1);
        two_sum(-cur.cv[j], -l2h[j], s2, e2);
        e2 -= l2l[j];
        const T mh = s2 + e2, ml = e2 - (mh - s2);
        if (p < Pn) {
          a.CV[(size_t)v * Pnp + p] = ch;
          if constexpr (sizeof(T) == 4) a.CVlo[(size_t)v * Pnp + p] = cl;
        }
        smu[p] = mh;
        smu[32 * PPL + p] = ml;
        if (a.rec_mh && p < Pn) {
          a.rec_mh[(size_t)v * Pn + p] = mh;
          a.rec_ml[(size_t)v * Pn + p] = ml;
        }
      }
      __syncwarp();
      if (qon) {
        const bool hin = (inmask >> jv) & 1u, hout = (outmask >> jv) & 1u;
#pragma unroll
        for (int k = 0; k < QPL; ++k) {
          const int q = qo + k;
          T yo = T(0), zo = T(0), fo = T(0);
          if (q < Pe) {
            T R0 = vfm[k], F0 = vrm[k];
            if (hout) R0 = fmax(R0, ((q < qcov ? cur.rq[k] : T(0)) - lbh[k]) - lbl[k]);
            if (hin) F0 = fmax(F0, ((q < qcov ? cur.fq[k] : T(0)) - lbh[k]) - lbl[k]);
            const T f = (smu[qd[k]] - F0) + smu[32 * PPL + qd[k]];
            const T r = (smu[qs[k]] - R0) + smu[32 * PPL + qs[k]];
            mxF[k] = fmax(mxF[k], f);
            mxR[k] = fmax(mxR[k], r);
            lr[k].add_fast(f + cur.b[k]);
            lf[k].add_fast(r + cur.b[k]);
            yo = f - cur.em[k];  // no out-edges: dEmin = +inf, Y = -inf
            zo = r;
            fo = f;
          }
          if (q < Pp) {
            a.vf[(size_t)v * Pp + q] = yo;
            a.vr[(size_t)v * Pp + q] = zo;
            if (a.rec_f) a.rec_f[(size_t)v * Pp + q] = fo;
          }
        }
      }
      __syncwarp();
      cur = nxt;
    }
  }

  // block partials: mVF, mVR (max), lR, lF (lse); warps combined in order
  __syncthreads();
  const int nmax = 2 * Pe, nlse = 2 * Pe, slots = nmax + 2 * nlse;
  double* red = reinterpret_cast<double*>(s_mu);  // the MU rows are free now
  double* r = red + (size_t)wib * slots;
#pragma unroll
  for (int k = 0; k < QPL; ++k) {
    const int q = qo + k;
    if (q < Pe) {
      r[q] = (double)mxF[k];
      r[Pe + q] = (double)mxR[k];
      r[nmax + 2 * q] = lr[k].mval();
      r[nmax + 2 * q + 1] = lr[k].sval();
      r[nmax + 2 * (Pe + q)] = lf[k].mval();
      r[nmax + 2 * (Pe + q) + 1] = lf[k].sval();
    }
  }
  __syncthreads();
  write_block_partials(red, kW, nmax, nlse, a.bpart, gridDim.x, blockIdx.x);
}

template <typename T, int QPL, int PPL>
size_t init_warp_smem(int pn, int pe) {
  const size_t pat = (sizeof(int) * (size_t)(4 * pe + 2 * (pn + 1)) + 15) & ~size_t(15);
  const size_t mu = sizeof(T) * (size_t)(kST / 32) * 64 * PPL;
  const size_t red = sizeof(double) * (size_t)(kST / 32) * 6 * pe;
  return pat + (mu > red ? mu : red);
}

// Resident blocks per SM of the init kernel's shape (sets its shared-memory
// attribute); the shape is chosen as for the vertex phase.
template <typename T, int QPL, int PPL>
int init_warp_fit(int pn, int pe, size_t* sm) {
  *sm = init_warp_smem<T, QPL, PPL>(pn, pe);
  if (*sm > 48 * 1024)
    cudaFuncSetAttribute(init_warp_kernel<T, QPL, PPL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)*sm);
  int nb = 1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, init_warp_kernel<T, QPL, PPL>, kST, *sm) !=
      cudaSuccess)
    nb = 1;
  return nb < 1 ? 1 : nb;
}

template <typename T, typename F>
bool init_warp_shape(int pn, int pp, F&& f) {
  if (pp > 64 || pn > 64) return false;
  if (pp <= 32 && pn <= 32) f.template operator()<1, 1>();
  else if (pp <= 32) f.template operator()<1, 2>();
  else if (pn <= 32) f.template operator()<2, 1>();
  else f.template operator()<2, 2>();
  return true;
}

#define ACG_STATIC_SHAPES(X) \
  X(1, 1) X(2, 1) X(4, 1) X(8, 1) X(16, 1) X(32, 1) X(32, 2) X(32, 4)

}  // namespace

#define ACG_SRC_LAUNCH(NP_, NQ_)                                                            \
  if (ws.npow == NP_ && ws.nqv == NQ_) {                                                    \
    constexpr size_t sm = src_stage_smem<T, NQ_>();                                         \
    if (sm > 48 * 1024)                                                                     \
      ACG_CUDA_TRY(cudaFuncSetAttribute(src_stats_kernel<T, NP_, NQ_>,                      \
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm)); \
    src_stats_kernel<T, NP_, NQ_><<<blocks, kST, sm, s>>>(a);                               \
    ACG_LAUNCH_CHECK();                                                                     \
    return ACG_OK;                                                                          \
  }

template <typename T>
acg_status launch_src_stats(const SrcStatsArgs<T>& a, WarpShape ws, int blocks, cudaStream_t s) {
  if (a.nitems == 0) return ACG_OK;
  ACG_STATIC_SHAPES(ACG_SRC_LAUNCH)
  return set_error(ACG_ERR_UNSUPPORTED, "no source-side kernel for npow=%d nqv=%d", ws.npow, ws.nqv);
}

template <typename T>
acg_status launch_src_stats_combine(const SrcStatsArgs<T>& a, const WarpWork& w, cudaStream_t s) {
  if (w.nheavy == 0) return ACG_OK;
  src_stats_combine_kernel<T><<<ceil_div(w.nheavy, 8), 256, 0, s>>>(a, w.hbase, w.hcount, w.hvert,
                                                                    w.nheavy);
  ACG_LAUNCH_CHECK();
  return ACG_OK;
}

#define ACG_DST_LAUNCH(NP_, NQ_)                                                  \
  if (ws.npow == NP_ && ws.nqv == NQ_) {                                          \
    const size_t sm = sizeof(double) * (size_t)(kST / 32) * 2 * a.Pqc;            \
    if (sm > 48 * 1024)                                                           \
      ACG_CUDA_TRY(cudaFuncSetAttribute(dst_quirk_kernel<T, NP_, NQ_>,            \
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm)); \
    dst_quirk_kernel<T, NP_, NQ_><<<blocks, kST, sm, s>>>(a);                     \
    ACG_LAUNCH_CHECK();                                                           \
    return ACG_OK;                                                                \
  }

template <typename T>
acg_status launch_dst_quirk(const DstQuirkArgs<T>& a, WarpShape ws, int blocks, cudaStream_t s) {
  if (a.nitems == 0 || a.qcov == 0) return ACG_OK;
  ACG_STATIC_SHAPES(ACG_DST_LAUNCH)
  return set_error(ACG_ERR_UNSUPPORTED, "no quirk kernel for npow=%d nqv=%d", ws.npow, ws.nqv);
}

#define ACG_SRC_OCC(NP_, NQ_)                                                           \
  if (ws.npow == NP_ && ws.nqv == NQ_) {                                                \
    constexpr size_t sm = src_stage_smem<T, NQ_>();                                     \
    if (sm > 48 * 1024)                                                                 \
      cudaFuncSetAttribute(src_stats_kernel<T, NP_, NQ_>,                               \
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);       \
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, src_stats_kernel<T, NP_, NQ_>, \
                                                      kST, sm) != cudaSuccess)          \
      nb = 1;                                                                           \
  }

template <typename T>
int src_stats_blocks_per_sm(WarpShape ws) {
  int nb = 1;
  ACG_STATIC_SHAPES(ACG_SRC_OCC)
  return nb < 1 ? 1 : nb;
}

template <typename T>
int init_warp_blocks(int pn, int pe, int pp, int num_sms) {
  int nb = 0;
  const bool ok = init_warp_shape<T>(pn, pp, [&]<int QPL, int PPL>() {
    size_t sm = 0;
    nb = init_warp_fit<T, QPL, PPL>(pn, pe, &sm);
  });
  return ok ? num_sms * nb : 0;
}

template <typename T>
acg_status launch_init_warp(const InitArgs<T>& a, int blocks, cudaStream_t s) {
  cudaError_t le = cudaSuccess;
  const bool ok = init_warp_shape<T>(a.Pn, a.Pp, [&]<int QPL, int PPL>() {
    size_t sm = 0;
    init_warp_fit<T, QPL, PPL>(a.Pn, a.Pe, &sm);
    init_warp_kernel<T, QPL, PPL><<<blocks, kST, sm, s>>>(a);
    le = cudaGetLastError();
  });
  if (!ok) return set_error(ACG_ERR_UNSUPPORTED, "init warp form: pattern too large");
  if (le != cudaSuccess) return set_error(ACG_ERR_CUDA, "init_warp_kernel launch: %s", cudaGetErrorString(le));
  return ACG_OK;
}

template int init_warp_blocks<double>(int, int, int, int);
template int init_warp_blocks<float>(int, int, int, int);
template acg_status launch_init_warp<double>(const InitArgs<double>&, int, cudaStream_t);
template acg_status launch_init_warp<float>(const InitArgs<float>&, int, cudaStream_t);

template acg_status launch_src_stats<double>(const SrcStatsArgs<double>&, WarpShape, int, cudaStream_t);
template acg_status launch_src_stats<float>(const SrcStatsArgs<float>&, WarpShape, int, cudaStream_t);
template acg_status launch_src_stats_combine<double>(const SrcStatsArgs<double>&, const WarpWork&, cudaStream_t);
template acg_status launch_src_stats_combine<float>(const SrcStatsArgs<float>&, const WarpWork&, cudaStream_t);
template acg_status launch_dst_quirk<double>(const DstQuirkArgs<double>&, WarpShape, int, cudaStream_t);
template acg_status launch_dst_quirk<float>(const DstQuirkArgs<float>&, WarpShape, int, cudaStream_t);
template int src_stats_blocks_per_sm<double>(WarpShape);
template int src_stats_blocks_per_sm<float>(WarpShape);

}  // namespace acg
