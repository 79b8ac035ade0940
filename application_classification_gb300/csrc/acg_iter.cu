// acg_iter.cu -- one BP iteration as two kernels (see acg_bp.cu's header for
// the algebra).
//
// Phase A, edge_max_kernel -- the segmented (max, -) reduction over the
// destination-sorted CSR:  M'[v][q] = max_{e in in(v)} VR'[s_e][q] - dE[e][q].
//   One warp per work item (a light vertex's in-edges, or one chunk of a heavy
//   vertex's).  The 32 lanes are (edge slot, 16-byte column) pairs: NPOW lanes
//   cover one [Pp] row, S = 32 / NPOW in-edges are loaded per instruction and
//   kU instructions are issued back to back, so each warp keeps S * kU pairs of
//   (streamed dE row, gathered VR' row) in flight.  The items are cut into
//   contiguous ranges of near-equal cost (load steps plus a per-item
//   overhead; built on the device once per data graph), up to 32 per launched
//   warp: a warp walks its own range, then claims further ranges from a
//   counter as it finishes, so the SMs stay full until the last ranges.  Every
//   item is written by exactly one warp, whichever it is, so the result does
//   not depend on the order of the claims.  A chunk writes a partial row;
//   heavy_combine_kernel takes the max of a heavy vertex's partial rows.
//
// Phase B, vertex_warp_kernel (patterns up to 64 x 64) -- one warp per
//   contiguous vertex range, rows staged per warp with cp.async; see its own
//   comment.  The block-tile form below it serves larger patterns.
//
// Phase B, vertex_update_kernel -- everything per vertex, streamed with
//   coalesced 16-byte accesses: FMax, RMax, MU_raw (compensated sum), the next
//   VF', VR', and per-column statistics.  One thread per (vertex, 16-byte
//   column) for the q-side and per (vertex, pattern vertex) for MU; a block
//   walks fixed tiles of consecutive vertices and every thread owns fixed
//   columns, so statistics are accumulated in registers in a fixed order and
//   results are bit-reproducible.  No kernel waits on another block.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <limits>
#include <vector>

#include "acg_device.cuh"
#include "acg_iter.cuh"
#include "acg_vschedule.h"

namespace acg {

namespace {

constexpr int kAT = 256;       // threads per block, phase A
// 3 steps in flight measured fastest at RMAT-22 (4.07 ms per edge phase; 2: 4.44,
// 4: 4.47, 5: 4.36, 6: 5.37, 8: 5.21 ms)
#ifndef ACG_EDGE_KU
#define ACG_EDGE_KU 3
#endif
constexpr int kU = ACG_EDGE_KU;  // edge steps issued back to back
constexpr int kBT = 256;       // threads per block, phase B

template <typename T>
struct VecT;
template <>
struct VecT<double> {
  using type = double2;
  static constexpr int W = 2;
};
template <>
struct VecT<float> {
  using type = float4;
  static constexpr int W = 4;
};
template <typename T>
__device__ __forceinline__ T vg(const typename VecT<T>::type& v, int w) {
  return reinterpret_cast<const T*>(&v)[w];
}
template <typename T>
__device__ __forceinline__ void vs(typename VecT<T>::type& v, int w, T x) {
  reinterpret_cast<T*>(&v)[w] = x;
}
template <typename T>
__device__ __forceinline__ typename VecT<T>::type vfill(T x) {
  typename VecT<T>::type r;
#pragma unroll
  for (int w = 0; w < VecT<T>::W; ++w) vs<T>(r, w, x);
  return r;
}

__host__ __device__ inline size_t a16(size_t b) { return (b + 15) & ~size_t(15); }

// ------------------------------------------------------------------ phase A
// (An explicit minimum of one block per SM lets the compiler keep more of the
// pipelined loads in registers: 72 registers and 3 blocks/SM measured faster
// than 56 registers and 4 blocks/SM at RMAT-22, 4.47 ms against 5.30 ms.)
#ifndef ACG_EDGE_MINB
#define ACG_EDGE_MINB 1
#endif
// ARG: also the first maximal dst-CSR position of each maximum (adjoint
// recording): ties go to the smaller position.
// The max of heavy vertex h's cnt partial rows into its M row; one warp, lanes
// over columns.  The rows were written by other warps of this launch: read
// through L2.
template <typename T>
__device__ __forceinline__ void heavy_finish(const T* partial, T* M, size_t b0, size_t out, int cnt,
                                             int Pp) {
  const int lane = threadIdx.x & 31;
  for (int q = lane; q < Pp; q += 32) {
    T m = neg_inf<T>();
    for (int r = 0; r < cnt; ++r) m = fmax(m, __ldcg(partial + b0 + (size_t)r * Pp + q));
    M[out + q] = m;
  }
}

// One range of a warp's items, [it, it_end).
template <typename T, int NPOW, int NQV, bool ARG>
__device__ __forceinline__ void edge_max_range(const EdgeMaxArgs<T>& a, int it, const int it_end,
                                               const int slot, const int qc) {
  using VT = typename VecT<T>::type;
  constexpr int W = VecT<T>::W;
  constexpr int S = 32 / NPOW;
  constexpr int NQ = NQV * W;
  constexpr int STEP = S * kU;
  const int Pp = a.Pp;
  if (it >= it_end) return;

  // Software pipeline over the warp's steps (kU in-edges per slot per step,
  // crossing item boundaries): the source indices of step k+1 are loaded while
  // the gathered rows of step k are in flight.
  int4 item = __ldg(a.items + it);
  int4 item_next = it + 1 < it_end ? __ldg(a.items + it + 1) : make_int4(0, 0, 0, -1);
  int base = item.y;
  int sidx[kU];
#pragma unroll
  for (int u = 0; u < kU; ++u) {
    const int e = base + slot + S * u;
    sidx[u] = e < item.z ? __ldg(a.src_of + e) : 0;
  }
  T acc[NQ];
  int pos[ARG ? NQ : 1];
#pragma unroll
  for (int k = 0; k < NQ; ++k) acc[k] = neg_inf<T>();
  if constexpr (ARG) {
#pragma unroll
    for (int k = 0; k < NQ; ++k) pos[k] = -1;
  }
  for (;;) {
    // rows of this step
    VT x[kU][NQV], y[kU][NQV];
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const int e = base + slot + S * u;
      const bool ok = e < item.z;
#pragma unroll
      for (int k = 0; k < NQV; ++k) {
        const int qv = qc + NPOW * k;
        if (ok && qv * W < Pp) {
          x[u][k] = __ldg(reinterpret_cast<const VT*>(a.vr_in + (size_t)sidx[u] * Pp) + qv);
          y[u][k] = __ldcs(reinterpret_cast<const VT*>(a.dE + (size_t)e * Pp) + qv);
        } else {
          x[u][k] = vfill<T>(neg_inf<T>());
          y[u][k] = vfill<T>(T(0));
        }
      }
    }
    // next step's position, and its source indices (in flight with the rows)
    const bool item_done = base + STEP >= item.z;
    int nbase = base + STEP, nend = item.z;
    bool more = true;
    if (item_done) {
      more = it + 1 < it_end;
      nbase = item_next.y;
      nend = item_next.z;
    }
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const int e = nbase + slot + S * u;
      sidx[u] = (more && e < nend) ? __ldg(a.src_of + e) : 0;
    }
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      if constexpr (ARG) {
        const int e = base + slot + S * u;
        if (e < item.z) {
#pragma unroll
          for (int k = 0; k < NQV; ++k)
#pragma unroll
            for (int w = 0; w < W; ++w) {
              const T v = vg<T>(x[u][k], w) - vg<T>(y[u][k], w);
              if (pos[k * W + w] < 0 || v > acc[k * W + w]) {
                acc[k * W + w] = v;
                pos[k * W + w] = e;
              }
            }
        }
      } else {
#pragma unroll
        for (int k = 0; k < NQV; ++k)
#pragma unroll
          for (int w = 0; w < W; ++w)
            acc[k * W + w] = fmax(acc[k * W + w], vg<T>(x[u][k], w) - vg<T>(y[u][k], w));
      }
    }
    if (item_done) {
      if constexpr (ARG) {
#pragma unroll
        for (int o = NPOW; o < 32; o <<= 1)
#pragma unroll
          for (int k = 0; k < NQ; ++k) {
            const T ob = __shfl_xor_sync(0xffffffffu, acc[k], o);
            const int op = __shfl_xor_sync(0xffffffffu, pos[k], o);
            if (op >= 0 && (pos[k] < 0 || ob > acc[k] || (ob == acc[k] && op < pos[k]))) {
              acc[k] = ob;
              pos[k] = op;
            }
          }
      } else {
#pragma unroll
        for (int o = NPOW; o < 32; o <<= 1)
#pragma unroll
          for (int k = 0; k < NQ; ++k) acc[k] = fmax(acc[k], __shfl_xor_sync(0xffffffffu, acc[k], o));
      }
      if (slot == 0) {
        T* row = item.w >= 0 ? a.partial + (size_t)item.w * Pp : a.M + (size_t)item.x * Pp;
#pragma unroll
        for (int k = 0; k < NQV; ++k) {
          const int qv = qc + NPOW * k;
          if (qv * W < Pp) {
            VT o;
#pragma unroll
            for (int w = 0; w < W; ++w) vs<T>(o, w, acc[k * W + w]);
            reinterpret_cast<VT*>(row)[qv] = o;
            if constexpr (ARG) {
              int* prow = item.w >= 0 ? a.ppos + (size_t)item.w * Pp : a.argpos + (size_t)item.x * Pp;
#pragma unroll
              for (int w = 0; w < W; ++w) prow[qv * W + w] = pos[k * W + w];
            }
          }
        }
      }
      // (FP32 without argmax only: in the other forms the finisher would cost
      // the edge loop registers, 64 -> 72..94; they keep heavy_combine)
      if (sizeof(T) == 4 && !ARG && item.w >= 0 && a.hcnt) {
        // a chunk: its rows are fenced before the count; the warp that
        // completes the heavy vertex's last chunk fences again and combines
        __threadfence();
        __syncwarp();
        const int h = __ldg(a.pheavy + item.w);
        const int cnt = __ldg(a.hcount + h);
        int last = 0;
        if ((threadIdx.x & 31) == 0) last = atomicAdd(a.hcnt + h, 1) == cnt - 1;
        if (__shfl_sync(0xffffffffu, last, 0)) {
          __threadfence();
          heavy_finish<T>(a.partial, a.M, (size_t)__ldg(a.hbase + h) * Pp,
                          (size_t)__ldg(a.hvert + h) * Pp, cnt, Pp);
          if ((threadIdx.x & 31) == 0) a.hcnt[h] = 0;  // ready for the next launch
        }
      }
#pragma unroll
      for (int k = 0; k < NQ; ++k) acc[k] = neg_inf<T>();
      if constexpr (ARG) {
#pragma unroll
        for (int k = 0; k < NQ; ++k) pos[k] = -1;
      }
      if (!more) break;
      ++it;
      item = item_next;
      item_next = it + 1 < it_end ? __ldg(a.items + it + 1) : make_int4(0, 0, 0, -1);
    }
    base = nbase;
  }
}

template <typename T, int NPOW, int NQV, bool ARG>
__global__ void __launch_bounds__(kAT, ACG_EDGE_MINB)
edge_max_kernel(const EdgeMaxArgs<T> a) {
  const int lane = threadIdx.x & 31;
  const int slot = lane / NPOW, qc = lane % NPOW;
  const int nw = (int)gridDim.x * (kAT / 32);
  const int gw = (blockIdx.x * kAT + threadIdx.x) >> 5;
  // The warp's own range first, then claimed ones (the claim of the next is in
  // flight while this one runs): warps that finish early keep taking work, so
  // the SMs stay full until the last ranges instead of waiting on the slowest
  // warp of a static split.
  for (int r = gw; r < a.nranges;) {
    int rn = a.nranges;
    if (a.ctr && lane == 0) rn = nw + atomicAdd(a.ctr, 1);
    edge_max_range<T, NPOW, NQV, ARG>(a, __ldg(a.wsplit + r), __ldg(a.wsplit + r + 1), slot, qc);
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

// Max over each heavy vertex's partial rows: one warp per heavy vertex.
template <typename T>
__global__ void __launch_bounds__(256)
heavy_combine_kernel(const T* __restrict__ partial, const int* __restrict__ hbase,
                     const int* __restrict__ hcount, const int* __restrict__ hvert, int nheavy,
                     int Pp, T* __restrict__ M) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= nheavy) return;
  const T* p0 = partial + (size_t)hbase[warp] * Pp;
  const int cnt = hcount[warp];
  T* row = M + (size_t)hvert[warp] * Pp;
  for (int q = lane; q < Pp; q += 32) {
    T m = neg_inf<T>();
    int r = 0;
    for (; r + 4 <= cnt; r += 4) {
      const T a0 = p0[(size_t)r * Pp + q], a1 = p0[(size_t)(r + 1) * Pp + q];
      const T a2 = p0[(size_t)(r + 2) * Pp + q], a3 = p0[(size_t)(r + 3) * Pp + q];
      m = fmax(m, fmax(fmax(a0, a1), fmax(a2, a3)));
    }
    for (; r < cnt; ++r) m = fmax(m, p0[(size_t)r * Pp + q]);
    row[q] = m;
  }
}

// The same with the chunks' argmax positions (chunks in order: an earlier
// chunk keeps a tie).
template <typename T>
__global__ void __launch_bounds__(256)
heavy_combine_arg_kernel(const T* __restrict__ partial, const int* __restrict__ ppos,
                         const int* __restrict__ hbase, const int* __restrict__ hcount,
                         const int* __restrict__ hvert, int nheavy, int Pp, T* __restrict__ M,
                         int* __restrict__ A) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= nheavy) return;
  const size_t b0 = (size_t)hbase[warp] * Pp, out = (size_t)hvert[warp] * Pp;
  const int cnt = hcount[warp];
  for (int q = lane; q < Pp; q += 32) {
    T m = neg_inf<T>();
    int bi = -1;
    auto take = [&](T x, int px) {
      if (px >= 0 && (bi < 0 || x > m)) {
        m = x;
        bi = px;
      }
    };
    int c = 0;
    for (; c + 4 <= cnt; c += 4) {  // four rows in flight, applied in order
      const size_t r = b0 + (size_t)c * Pp + q;
      const T x0 = partial[r], x1 = partial[r + Pp], x2 = partial[r + 2 * (size_t)Pp],
              x3 = partial[r + 3 * (size_t)Pp];
      const int p0 = ppos[r], p1 = ppos[r + Pp], p2 = ppos[r + 2 * (size_t)Pp],
                p3 = ppos[r + 3 * (size_t)Pp];
      take(x0, p0);
      take(x1, p1);
      take(x2, p2);
      take(x3, p3);
    }
    for (; c < cnt; ++c) {
      const size_t r = b0 + (size_t)c * Pp + q;
      take(partial[r], ppos[r]);
    }
    M[out + q] = m;
    A[out + q] = bi;
  }
}

// ------------------------------------------------------------------ phase B
struct UpdSmem {
  size_t pat, fill, lq, F, R, MU, red, stage, sM, sVF, sEM, sB, sCV, sCVl, sOff, stage_bytes, total;
  __host__ __device__ UpdSmem(int V, int Pn, int Pe, int Pp, int Pnp, int sz) {
    size_t o = 0;
    pat = o; o += a16(sizeof(int) * (size_t)(4 * Pe + 2 * (Pn + 1)));
    fill = o; o += a16((size_t)2 * Pp * sz);  // fillF, fillR (padded to Pp)
    lq = o; o += a16((size_t)8 * Pp * sz);    // dF, dR, cR', cF' as hi/lo pairs (padded to Pp)
    F = o; o += a16((size_t)V * Pp * sz);
    R = o; o += a16((size_t)V * Pp * sz);
    MU = o; o += a16((size_t)V * 2 * Pn * sz);  // hi, lo
    red = o; o += a16(sizeof(double) * (size_t)kBT * 6);
    // one stage: the tile's M, Y, dEmin, B rows, CV (hi, lo) rows, in-degree offsets
    size_t so = 0;
    sM = so; so += a16((size_t)V * Pp * sz);
    sVF = so; so += a16((size_t)V * Pp * sz);
    sEM = so; so += a16((size_t)V * Pp * sz);
    sB = so; so += a16((size_t)V * Pp * sz);
    sCV = so; so += a16((size_t)V * Pnp * sz);
    sCVl = so; so += sz == 4 ? a16((size_t)V * Pnp * sz) : 0;
    sOff = so; so += a16(sizeof(int) * (size_t)(V + 1));
    stage_bytes = so;
    stage = o; o += 2 * so;
    total = o;
  }
};

__device__ __forceinline__ unsigned sm_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void cp16(void* sdst, const void* gsrc) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sm_u32(sdst)), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp4(void* sdst, const void* gsrc) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sm_u32(sdst)), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_wait1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }
__device__ __forceinline__ void cp_wait0() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

template <typename T>
__global__ void __launch_bounds__(kBT, 2)
vertex_update_kernel(const VertexUpdArgs<T> a) {
  using VT = typename VecT<T>::type;
  constexpr int W = VecT<T>::W;
  extern __shared__ __align__(16) unsigned char smem[];
  const int Pe = a.Pe, Pn = a.Pn, Pp = a.Pp, Pnp = a.Pnp, Dn = a.Dn;
  const int nvec = Pp / W;
  const int V = kBT / nvec;  // vertices per tile
  const UpdSmem L(V, Pn, Pe, Pp, Pnp, sizeof(T));
  int* s_pat = reinterpret_cast<int*>(smem + L.pat);
  T* s_fillF = reinterpret_cast<T*>(smem + L.fill);
  T* s_fillR = s_fillF + Pp;
  T* s_dF = reinterpret_cast<T*>(smem + L.lq);  // hi, lo of each constant
  T* s_dFlo = s_dF + Pp;
  T* s_dR = s_dFlo + Pp;
  T* s_dRlo = s_dR + Pp;
  T* s_cR = s_dRlo + Pp;
  T* s_cRlo = s_cR + Pp;
  T* s_cF = s_cRlo + Pp;
  T* s_cFlo = s_cF + Pp;
  T* s_F = reinterpret_cast<T*>(smem + L.F);
  T* s_R = reinterpret_cast<T*>(smem + L.R);
  T* s_MU = reinterpret_cast<T*>(smem + L.MU);  // [V][Pn] hi then [V][Pn] lo
  T* s_MUlo = s_MU + (size_t)V * Pn;
  double* s_red = reinterpret_cast<double*>(smem + L.red);
  const int* s_psrc = s_pat;
  const int* s_pdst = s_pat + Pe;
  const int* s_inoff = s_pat + 2 * Pe;
  const int* s_inq = s_inoff + Pn + 1;
  const int* s_outoff = s_inq + Pe;
  const int* s_outq = s_outoff + Pn + 1;
  const int tid = threadIdx.x;

  for (int t = tid; t < 4 * Pe + 2 * (Pn + 1); t += kBT) s_pat[t] = a.pat[t];
  __syncthreads();
  {
    // Shifted storage: Y = VF' - dEmin - cR and Z = VR' - cF with per-q FP64
    // shifts, so that the entries that can win a max are small numbers and an
    // FP32 store keeps their low bits.  With dR = lR - cR, dF = lF - cF
    // (statistics of the previous pass, in that pass's shifts):
    //   RMax = max(fillR, Y - dR)       FMax = max(fillF, max_e(Z[s_e] - dE) - dF)
    // New shifts for this pass's stores: lR, lF of the pass before the previous
    // one (the iteration has period two, so that value tracks lR, lF closely);
    // the first pass uses the previous pass's own.  Any finite shift is exact.
    const double* g = a.glob_in;
    const int x0 = 4 * Pe + Pn;
    auto split = [](double x, T* hi, T* lo, int q) {
      const T h = (T)x;
      hi[q] = h;
      lo[q] = (T)(x - (double)h);
    };
    for (int q = tid; q < Pp; q += kBT) {
      if (q >= Pe) {
        s_fillF[q] = s_fillR[q] = T(0);
        s_dF[q] = s_dFlo[q] = s_dR[q] = s_dRlo[q] = T(0);
        s_cR[q] = s_cRlo[q] = s_cF[q] = s_cFlo[q] = T(0);
        continue;
      }
      const double cRu = g[x0 + q], cFu = g[x0 + Pe + q];
      const double dR = g[2 * Pe + q], dF = g[3 * Pe + q];
      double fr = g[q] + cRu - g[4 * Pe + s_pdst[q]];
      double ff = g[Pe + q] + cFu - g[4 * Pe + s_psrc[q]];
      if (a.cnull) {
        fr -= a.cnull[q];
        ff -= a.cnull[q];
      }
      s_fillR[q] = (T)fr;
      s_fillF[q] = (T)ff;
      split(dR, s_dR, s_dRlo, q);
      split(dF, s_dF, s_dFlo, q);
      const double lRp = cRu + dR, lFp = cFu + dF;
      double cRn = a.first ? lRp : g[x0 + 2 * Pe + q];
      double cFn = a.first ? lFp : g[x0 + 3 * Pe + q];
      if (!isfinite(cRn)) cRn = 0.0;
      if (!isfinite(cFn)) cFn = 0.0;
      split(cRn, s_cR, s_cRlo, q);
      split(cFn, s_cF, s_cFlo, q);
      if (blockIdx.x == 0) {
        double* o = a.glob_out;
        o[x0 + q] = (double)s_cR[q] + (double)s_cRlo[q];
        o[x0 + Pe + q] = (double)s_cF[q] + (double)s_cFlo[q];
        o[x0 + 2 * Pe + q] = lRp;
        o[x0 + 3 * Pe + q] = lFp;
      }
    }
  }
  __syncthreads();

  // fixed columns: q-vector qv (vertex j0 of the tile), pattern vertex pc.
  // Everything a thread indexes in shared memory is fixed across tiles, so the
  // pointers and the pattern endpoints of its columns are set up once.
  const int qv = tid % nvec, j0 = tid / nvec;
  const bool qact = j0 < V;
  const int pc = tid % Pn, jp0 = tid / Pn, prows = kBT / Pn;
  T* const myF = s_F + j0 * Pp + qv * W;
  T* const myR = s_R + j0 * Pp + qv * W;
  const T* const myMU = s_MU + j0 * Pn;
  const T* const myMUlo = s_MUlo + j0 * Pn;
  const int qoff = j0 * Pp + qv * W;  // offset in a [V][Pp] stage block
  int pdst[W], psrc[W];
#pragma unroll
  for (int w = 0; w < W; ++w) {
    const int q = qv * W + w;
    pdst[w] = q < Pe ? s_pdst[q] : 0;
    psrc[w] = q < Pe ? s_psrc[q] : 0;
  }
  const int in0 = s_inoff[pc], in1 = s_inoff[pc + 1];
  const int out0 = s_outoff[pc], out1 = s_outoff[pc + 1];
  const bool my_last = __ldg(a.iters_p + pc) == a.t;
  T mxF[W], mxR[W];
  OnlineLse<T> lr[W], lf[W], lmu;
#pragma unroll
  for (int w = 0; w < W; ++w) {
    mxF[w] = neg_inf<T>();
    mxR[w] = neg_inf<T>();
    lr[w].init();
    lf[w].init();
  }
  lmu.init();

  const int ntiles = (Dn + V - 1) / V;
  const int cvec = Pnp / W;
  // Stage a tile's rows into shared memory with asynchronous 16-byte copies
  // (its vertices are consecutive, so every row block is contiguous).
  auto issue = [&](int tile, int k) {
    if (tile >= ntiles) return;
    unsigned char* st = smem + L.stage + (size_t)(k & 1) * L.stage_bytes;
    const int v0 = tile * V;
    const int nv = min(V, Dn - v0);
    const T* gM = a.M + (size_t)v0 * Pp;
    const T* gVF = a.vf + (size_t)v0 * Pp;
    const T* gEM = a.dEmin + (size_t)v0 * Pp;
    const T* gB = a.B + (size_t)v0 * Pp;
    T* sM = reinterpret_cast<T*>(st + L.sM);
    T* sVF = reinterpret_cast<T*>(st + L.sVF);
    T* sEM = reinterpret_cast<T*>(st + L.sEM);
    T* sB = reinterpret_cast<T*>(st + L.sB);
    for (int c = tid * W; c < nv * Pp; c += kBT * W) {
      cp16(sM + c, gM + c);
      cp16(sVF + c, gVF + c);
      cp16(sEM + c, gEM + c);
      cp16(sB + c, gB + c);
    }
    const T* gCV = a.CV + (size_t)v0 * Pnp;
    T* sCV = reinterpret_cast<T*>(st + L.sCV);
    for (int c = tid * W; c < nv * Pnp; c += kBT * W) cp16(sCV + c, gCV + c);
    if constexpr (sizeof(T) == 4) {
      const T* gCVl = a.CVlo + (size_t)v0 * Pnp;
      T* sCVl = reinterpret_cast<T*>(st + L.sCVl);
      for (int c = tid * W; c < nv * Pnp; c += kBT * W) cp16(sCVl + c, gCVl + c);
    }
    int* sOff = reinterpret_cast<int*>(st + L.sOff);
    for (int j = tid; j <= nv; j += kBT) cp4(sOff + j, a.d_off + v0 + j);
  };
  (void)cvec;
  issue(blockIdx.x, 0);
  cp_commit();
  int k = 0;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++k) {
    issue(tile + gridDim.x, k + 1);  // next tile's copies fly while this one computes
    cp_commit();
    cp_wait1();
    __syncthreads();
    const unsigned char* st = smem + L.stage + (size_t)(k & 1) * L.stage_bytes;
    const T* sCV = reinterpret_cast<const T*>(st + L.sCV);
    const int* sOff = reinterpret_cast<const int*>(st + L.sOff);
    const int v0 = tile * V;
    const int v = v0 + j0;
    const bool vok = qact && v < Dn;
    VT bv = vfill<T>(T(0)), emv = vfill<T>(T(0));
    if (vok) {
      const bool has_in = sOff[j0 + 1] > sOff[j0];
      const VT mv = has_in ? *reinterpret_cast<const VT*>(reinterpret_cast<const T*>(st + L.sM) + qoff)
                           : vfill<T>(neg_inf<T>());
      const VT yv = *reinterpret_cast<const VT*>(reinterpret_cast<const T*>(st + L.sVF) + qoff);
      emv = *reinterpret_cast<const VT*>(reinterpret_cast<const T*>(st + L.sEM) + qoff);
      bv = *reinterpret_cast<const VT*>(reinterpret_cast<const T*>(st + L.sB) + qoff);
      // per-q constants of the thread's columns (16-byte shared loads)
      const VT fF = *reinterpret_cast<const VT*>(s_fillF + qv * W);
      const VT fR = *reinterpret_cast<const VT*>(s_fillR + qv * W);
      const VT dF = *reinterpret_cast<const VT*>(s_dF + qv * W);
      const VT dFl = *reinterpret_cast<const VT*>(s_dFlo + qv * W);
      const VT dR = *reinterpret_cast<const VT*>(s_dR + qv * W);
      const VT dRl = *reinterpret_cast<const VT*>(s_dRlo + qv * W);
      VT fo, ro;
#pragma unroll
      for (int w = 0; w < W; ++w) {
        // no in-edges: M = -inf; no out-edges: Y = -inf; the fill wins
        vs<T>(fo, w, fmax(vg<T>(fF, w), (vg<T>(mv, w) - vg<T>(dF, w)) - vg<T>(dFl, w)));
        vs<T>(ro, w, fmax(vg<T>(fR, w), (vg<T>(yv, w) - vg<T>(dR, w)) - vg<T>(dRl, w)));
      }
      *reinterpret_cast<VT*>(myF) = fo;
      *reinterpret_cast<VT*>(myR) = ro;
    }
    __syncthreads();
    // MU_raw = -CV + sum F + sum R, compensated (CV carries a low part)
    for (int j = jp0; j < V && jp0 < prows; j += prows) {
      const int vv = v0 + j;
      if (vv >= Dn) break;
      const T* rowF = s_F + j * Pp;
      const T* rowR = s_R + j * Pp;
      CSum<T> mu;
      mu.init(-sCV[j * Pnp + pc]);
      if constexpr (sizeof(T) == 4)
        mu.lo = -reinterpret_cast<const T*>(st + L.sCVl)[j * Pnp + pc];
      for (int t = in0; t < in1; ++t) mu.add(rowF[s_inq[t]]);
      for (int t = out0; t < out1; ++t) mu.add(rowR[s_outq[t]]);
      s_MU[j * Pn + pc] = mu.hi;
      if constexpr (sizeof(T) == 4) s_MUlo[j * Pn + pc] = mu.lo;
      lmu.add2(mu.hi, mu.lo);
      if (my_last) a.mu_raw[(size_t)vv * Pn + pc] = mu.dvalue();
    }
    __syncthreads();
    if (!a.last && vok) {
      const VT fo = *reinterpret_cast<const VT*>(myF);
      const VT ro = *reinterpret_cast<const VT*>(myR);
      const VT cR = *reinterpret_cast<const VT*>(s_cR + qv * W);
      const VT cF = *reinterpret_cast<const VT*>(s_cF + qv * W);
      VT nf, nr;
#pragma unroll
      for (int w = 0; w < W; ++w) {
        // f = VF' - cR, r = VR' - cF; the shift is taken off the compensated
        // MU_raw first (for the entries that matter the two are close, so the
        // difference is exact) and the small message after
        T f, r;
        if constexpr (sizeof(T) == 4) {
          const VT cRl = *reinterpret_cast<const VT*>(s_cRlo + qv * W);
          const VT cFl = *reinterpret_cast<const VT*>(s_cFlo + qv * W);
          f = ((myMU[pdst[w]] - vg<T>(cR, w)) - vg<T>(fo, w)) + (myMUlo[pdst[w]] - vg<T>(cRl, w));
          r = ((myMU[psrc[w]] - vg<T>(cF, w)) - vg<T>(ro, w)) + (myMUlo[psrc[w]] - vg<T>(cFl, w));
        } else {
          f = (myMU[pdst[w]] - vg<T>(cR, w)) - vg<T>(fo, w);
          r = (myMU[psrc[w]] - vg<T>(cF, w)) - vg<T>(ro, w);
        }
        T y;
        if (qv * W + w < Pe) {
          mxF[w] = fmax(mxF[w], f);
          mxR[w] = fmax(mxR[w], r);
          const T b = vg<T>(bv, w);
          lr[w].add_fast(f + b);
          lf[w].add_fast(r + b);
          y = f - vg<T>(emv, w);  // no out-edges: dEmin = +inf, Y = -inf
        } else {
          y = T(0);
          r = T(0);
        }
        vs<T>(nf, w, y);
        vs<T>(nr, w, r);
      }
      const size_t go = (size_t)v * Pp + (size_t)qv * W;
      *reinterpret_cast<VT*>(a.vf + go) = nf;
      *reinterpret_cast<VT*>(a.vr_out + go) = nr;
    }
    __syncthreads();  // the tile's smem rows and this stage are free
  }
  cp_wait0();

  // ---- block partials: mVF, mVR (max), lR, lF, S (lse); rows combined in order
  const int nmax = 2 * Pe;
  const int ncols = gridDim.x, col = blockIdx.x;
#pragma unroll
  for (int w = 0; w < W; ++w) {
    __syncthreads();
    double* e = s_red + (size_t)tid * 6;
    e[0] = (double)mxF[w];
    e[1] = (double)mxR[w];
    e[2] = lr[w].mval();
    e[3] = lr[w].sval();
    e[4] = lf[w].mval();
    e[5] = lf[w].sval();
    __syncthreads();
    for (int c = tid; c < nvec; c += kBT) {
      const int q = c * W + w;
      if (q >= Pe) continue;
      double f = -CUDART_INF, r = -CUDART_INF, m1 = -CUDART_INF, s1 = 0, m2 = -CUDART_INF, s2 = 0;
      for (int row = 0; row < V; ++row) {
        const double* x = s_red + (size_t)(row * nvec + c) * 6;
        f = fmax(f, x[0]);
        r = fmax(r, x[1]);
        lse_merge(m1, s1, x[2], x[3]);
        lse_merge(m2, s2, x[4], x[5]);
      }
      a.bpart[(size_t)q * ncols + col] = f;
      a.bpart[(size_t)(Pe + q) * ncols + col] = r;
      a.bpart[(size_t)(nmax + 2 * q) * ncols + col] = m1;
      a.bpart[(size_t)(nmax + 2 * q + 1) * ncols + col] = s1;
      a.bpart[(size_t)(nmax + 2 * (Pe + q)) * ncols + col] = m2;
      a.bpart[(size_t)(nmax + 2 * (Pe + q) + 1) * ncols + col] = s2;
    }
  }
  __syncthreads();
  s_red[tid * 2] = lmu.mval();
  s_red[tid * 2 + 1] = lmu.sval();
  __syncthreads();
  for (int p = tid; p < Pn; p += kBT) {
    double m = -CUDART_INF, s = 0;
    for (int row = 0; row < prows; ++row)
      lse_merge(m, s, s_red[(row * Pn + p) * 2], s_red[(row * Pn + p) * 2 + 1]);
    a.bpart[(size_t)(nmax + 2 * (2 * Pe + p)) * ncols + col] = m;
    a.bpart[(size_t)(nmax + 2 * (2 * Pe + p) + 1) * ncols + col] = s;
  }
}


// ------------------------------------------------------ phase B, warp form
// Patterns with Pp <= 64 and Pn <= 64.  Lane l owns the QPL contiguous edge
// columns q = l * QPL + k and the pattern vertices p = l + 32 j (j < PPL); the
// per-q constants and statistics of its columns live in registers.  Each warp
// walks a contiguous range of vertices; their rows are staged into a per-warp
// double-buffered ring (kVps vertices per stage) with cp.async, so a warp never
// waits on another.  Per stage:
//   1. F, R of each staged vertex from its M, Y rows, written over them in the
//      stage (the CV rows are negated in place);
//   2. the compensated sums MU_raw[v][p] = -CV[v][p] + sum F + sum R of all
//      staged vertices through a per-lane schedule built on the host
//      (vertex_warp_schedule): each (vertex, p) sum is one job whose terms are
//      -CV, then F[q] of the in-edges q of p ascending, then R[q] of its
//      out-edges ascending -- the order of the tile form -- and the jobs are
//      spread over the lanes longest first, so a lane runs ~1/32 of the
//      stage's terms instead of the largest pattern degree for every vertex;
//   3. per staged vertex: the MU_raw statistics and outputs of the lane's p,
//      and the new Y, Z of its columns from MU_raw[dst_q], MU_raw[src_q].
// Every sum keeps its terms and their order, so the results do not depend on
// how the jobs are spread.  Vertices without in-edges have M rows of -inf (set
// once, never written by phase A).
#ifndef ACG_VTX_VPS
#define ACG_VTX_VPS 4
#endif
constexpr int kVps = ACG_VTX_VPS;  // vertices per stage
constexpr int kVw = kBT / 32;
template <typename T, int QPL, int PPL>
struct VwSmem {
  size_t pat, sched, ring, mu, total, stage, warp_ring, mu_n;
  __host__ __device__ VwSmem(int Pn, int Pe, int Pp, int Pnp, int nterms) {
    const size_t sz = sizeof(T);
    size_t o = 0;
    pat = o; o += a16(sizeof(int) * (size_t)(4 * Pe + 2 * (Pn + 1)));
    sched = o; o += a16(sizeof(uint32_t) * (size_t)nterms * 32);
    stage = (size_t)VwStage(Pp, Pnp, sz == 4, kVps).n * sz;  // row sizes are 16-byte multiples
    warp_ring = 2 * stage;
    const size_t red = sizeof(double) * (size_t)kVw * (6 * Pe + 2 * Pn);  // aliases the rings
    ring = o; o += a16(red > kVw * warp_ring ? red : kVw * warp_ring);
    mu_n = 2 * kVps * (32 * PPL + 1);  // MU_raw hi | lo rows of the staged vertices
    mu = o; o += a16((size_t)kVw * mu_n * sz);
    total = o;
  }
};

template <typename T, int N>
__device__ __forceinline__ void lds_n(const T* p, T (&x)[N]) {
  if constexpr (N == 2 && sizeof(T) == 4) {
    const float2 v = *reinterpret_cast<const float2*>(p);
    x[0] = v.x;
    x[1] = v.y;
  } else if constexpr (N == 2 && sizeof(T) == 8) {
    const double2 v = *reinterpret_cast<const double2*>(p);
    x[0] = v.x;
    x[1] = v.y;
  } else {
#pragma unroll
    for (int k = 0; k < N; ++k) x[k] = p[k];
  }
}
template <typename T, int N>
__device__ __forceinline__ void st_n(T* p, const T (&x)[N]) {
  if constexpr (N == 2 && sizeof(T) == 4) {
    *reinterpret_cast<float2*>(p) = make_float2(x[0], x[1]);
  } else if constexpr (N == 2 && sizeof(T) == 8) {
    *reinterpret_cast<double2*>(p) = make_double2(x[0], x[1]);
  } else {
#pragma unroll
    for (int k = 0; k < N; ++k) p[k] = x[k];
  }
}

// Two blocks per SM bounds the registers at 128
#ifndef ACG_VTX_MINB
#define ACG_VTX_MINB 2
#endif
template <typename T, int QPL, int PPL>
__global__ void __launch_bounds__(kBT, ACG_VTX_MINB)
vertex_warp_kernel(const VertexUpdArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int Pe = a.Pe, Pn = a.Pn, Pp = a.Pp, Pnp = a.Pnp, Dn = a.Dn, nterms = a.vterms;
  const VwSmem<T, QPL, PPL> L(Pn, Pe, Pp, Pnp, nterms);
  const VwStage G(Pp, Pnp, sizeof(T) == 4, kVps);
  const int tid = threadIdx.x, lane = tid & 31, wib = tid >> 5;
  int* s_pat = reinterpret_cast<int*>(smem + L.pat);
  uint32_t* s_sched = reinterpret_cast<uint32_t*>(smem + L.sched);
  for (int t = tid; t < 4 * Pe + 2 * (Pn + 1); t += kBT) s_pat[t] = a.pat[t];
  for (int t = tid; t < nterms * 32; t += kBT) s_sched[t] = a.vsched[t];
  __syncthreads();
  const int* s_psrc = s_pat;
  const int* s_pdst = s_pat + Pe;

  // per-q constants of the lane's columns (see the tile form for the algebra)
  const double* g = a.glob_in;
  const int x0 = 4 * Pe + Pn;
  const int qo = lane * QPL;
  const bool qon = qo < Pp;
  T fF[QPL], fR[QPL], dFh[QPL], dFl[QPL], dRh[QPL], dRl[QPL], cRh[QPL], cRl[QPL], cFh[QPL], cFl[QPL];
  int qd[QPL], qs[QPL];
#pragma unroll
  for (int k = 0; k < QPL; ++k) {
    const int q = qo + k;
    fF[k] = fR[k] = dFh[k] = dFl[k] = dRh[k] = dRl[k] = cRh[k] = cRl[k] = cFh[k] = cFl[k] = T(0);
    qd[k] = qs[k] = 0;
    if (q < Pe) {
      qd[k] = s_pdst[q];
      qs[k] = s_psrc[q];
      const double cRu = g[x0 + q], cFu = g[x0 + Pe + q];
      const double dR = g[2 * Pe + q], dF = g[3 * Pe + q];
      double fr = g[q] + cRu - g[4 * Pe + qd[k]];
      double ff = g[Pe + q] + cFu - g[4 * Pe + qs[k]];
      if (a.cnull) {
        fr -= a.cnull[q];
        ff -= a.cnull[q];
      }
      fR[k] = (T)fr;
      fF[k] = (T)ff;
      dRh[k] = (T)dR;
      dRl[k] = (T)(dR - (double)dRh[k]);
      dFh[k] = (T)dF;
      dFl[k] = (T)(dF - (double)dFh[k]);
      const double lRp = cRu + dR, lFp = cFu + dF;
      double cRn = a.first ? lRp : g[x0 + 2 * Pe + q];
      double cFn = a.first ? lFp : g[x0 + 3 * Pe + q];
      if (!isfinite(cRn)) cRn = 0.0;
      if (!isfinite(cFn)) cFn = 0.0;
      cRh[k] = (T)cRn;
      cRl[k] = (T)(cRn - (double)cRh[k]);
      cFh[k] = (T)cFn;
      cFl[k] = (T)(cFn - (double)cFh[k]);
      if (blockIdx.x == 0 && wib == 0) {
        double* o = a.glob_out;
        o[x0 + q] = (double)cRh[k] + (double)cRl[k];
        o[x0 + Pe + q] = (double)cFh[k] + (double)cFl[k];
        o[x0 + 2 * Pe + q] = lRp;
        o[x0 + 3 * Pe + q] = lFp;
      }
    }
  }
  T mxF[QPL], mxR[QPL];
  OnlineLse<T> lr[QPL], lf[QPL], lmu[PPL];
  bool plast[PPL];  // this iteration is the last of pattern vertex p's pattern
#pragma unroll
  for (int k = 0; k < QPL; ++k) {
    mxF[k] = mxR[k] = neg_inf<T>();
    lr[k].init();
    lf[k].init();
  }
#pragma unroll
  for (int j = 0; j < PPL; ++j) {
    lmu[j].init();
    const int p = lane + 32 * j;
    plast[j] = p < Pn && __ldg(a.iters_p + p) == a.t;
  }

  const long long nw = (long long)gridDim.x * kVw;
  const long long gw = (long long)blockIdx.x * kVw + wib;
  const int vb = (int)(gw * Dn / nw), ve = (int)((gw + 1) * Dn / nw);
  unsigned char* ring = smem + L.ring + (size_t)wib * L.warp_ring;
  T* smu = reinterpret_cast<T*>(smem + L.mu) + (size_t)wib * L.mu_n;
  // MU_raw rows of the staged vertices, one word apart in bank order so that
  // the lanes ending jobs of one p for different vertices do not collide
  constexpr int kMuRow = 32 * PPL + 1;
  constexpr int kMuLo = kVps * kMuRow;  // the low parts after the high parts
  const size_t rowb = (size_t)Pp * sizeof(T), crow = (size_t)Pnp * sizeof(T);
  auto issue = [&](int v0, int buf) {
    const int nv = min(kVps, ve - v0);
    if (nv <= 0) return;
    unsigned char* st = ring + (size_t)buf * L.stage;
    const int n16 = (int)((size_t)nv * rowb / 16);
    const size_t go = (size_t)v0 * rowb;
    for (int c = lane; c < n16; c += 32) {
      cp16(st + G.oM * sizeof(T) + c * 16, reinterpret_cast<const unsigned char*>(a.M) + go + c * 16);
      cp16(st + G.oY * sizeof(T) + c * 16, reinterpret_cast<const unsigned char*>(a.vf) + go + c * 16);
      cp16(st + G.oE * sizeof(T) + c * 16, reinterpret_cast<const unsigned char*>(a.dEmin) + go + c * 16);
      cp16(st + G.oB * sizeof(T) + c * 16, reinterpret_cast<const unsigned char*>(a.B) + go + c * 16);
    }
    const int c16 = (int)((size_t)nv * crow / 16);
    const size_t co = (size_t)v0 * crow;
    for (int c = lane; c < c16; c += 32) {
      cp16(st + G.oC * sizeof(T) + c * 16, reinterpret_cast<const unsigned char*>(a.CV) + co + c * 16);
      if constexpr (sizeof(T) == 4)
        cp16(st + G.oCl * sizeof(T) + c * 16, reinterpret_cast<const unsigned char*>(a.CVlo) + co + c * 16);
    }
  };
  issue(vb, 0);
  cp_commit();
  int buf = 0;
  for (int v0 = vb; v0 < ve; v0 += kVps, buf ^= 1) {
    issue(v0 + kVps, buf ^ 1);  // the next stage flies while this one computes
    cp_commit();
    cp_wait1();
    __syncwarp();
    T* st = reinterpret_cast<T*>(ring + (size_t)buf * L.stage);
    const int nv = min(kVps, ve - v0);
    // ---- 1. F over M, R over Y; -CV (and its low part) in place
#pragma unroll
    for (int jv = 0; jv < kVps; ++jv) {
      if (jv >= nv) break;
      if (qon) {
        T m[QPL], y[QPL], F[QPL], R[QPL];
        T* sm_ = st + G.oM + jv * Pp + qo;
        T* sy_ = st + G.oY + jv * Pp + qo;
        lds_n<T, QPL>(sm_, m);
        lds_n<T, QPL>(sy_, y);
#pragma unroll
        for (int k = 0; k < QPL; ++k) {
          // no in-edges: M = -inf; no out-edges: Y = -inf; the fill wins
          F[k] = fmax(fF[k], (m[k] - dFh[k]) - dFl[k]);
          R[k] = fmax(fR[k], (y[k] - dRh[k]) - dRl[k]);
        }
        st_n<T, QPL>(sm_, F);
        st_n<T, QPL>(sy_, R);
      }
#pragma unroll
      for (int j = 0; j < PPL; ++j) {
        const int p = lane + 32 * j;
        if (p < Pn) {
          T* c = st + G.oC + jv * Pnp + p;
          *c = -*c;
          if constexpr (sizeof(T) == 4) c[G.oCl - G.oC] = -c[G.oCl - G.oC];
        }
      }
    }
    __syncwarp();
    // ---- 2. the compensated sums of the stage's (vertex, p) jobs, four terms
    // per step: their schedule words in one 16-byte load, their values loaded
    // before the dependent additions
    {
      T hi = T(0), lo = T(0);
      const uint4* sch = reinterpret_cast<const uint4*>(s_sched) + lane;
      for (int t4 = 0; t4 < nterms / 4; ++t4) {
        const uint4 w4 = sch[t4 * 32];
        const uint32_t w[4] = {w4.x, w4.y, w4.z, w4.w};
        T x[4], xl[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const T* xp = st + (w[u] & 0xfffu);
          x[u] = *xp;
          if constexpr (sizeof(T) == 4) xl[u] = (w[u] & kSchedStart) ? xp[G.oCl - G.oC] : T(0);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const bool first = (w[u] & kSchedStart) != 0;
          const T h0 = first ? T(0) : hi;
          if constexpr (sizeof(T) == 4) {
            // a job starts from (0, -CV_lo) and adds -CV_hi: exactly (-CV_hi, -CV_lo)
            const T l0 = first ? xl[u] : lo;
            const T sm = h0 + x[u];
            const T bp = sm - h0;
            lo = l0 + ((h0 - (sm - bp)) + (x[u] - bp));
            hi = sm;
          } else {
            hi = h0 + x[u];
          }
          if (w[u] & kSchedEnd) {
            const int slot = (int)((w[u] >> 16) & 0x1ffu);
            smu[slot] = hi;
            if constexpr (sizeof(T) == 4) smu[kMuLo + slot] = lo;
          }
        }
      }
    }
    __syncwarp();
    // ---- 3. per staged vertex: MU_raw outputs, new Y and Z; the FP32 column
    // log-sum-exps take the stage's values four at a time
    constexpr bool kBatch = sizeof(T) == 4 && kVps == 4;
    T lrv[QPL][kVps], lfv[QPL][kVps], muh[PPL][kVps], mul[PPL][kVps];
#pragma unroll
    for (int jv = 0; jv < kVps; ++jv) {
#pragma unroll
      for (int k = 0; k < QPL; ++k) lrv[k][jv] = lfv[k][jv] = neg_inf<T>();
#pragma unroll
      for (int j = 0; j < PPL; ++j) {
        muh[j][jv] = neg_inf<T>();
        mul[j][jv] = T(0);
      }
    }
#pragma unroll
    for (int jv = 0; jv < kVps; ++jv) {
      if (jv >= nv) break;
      const int v = v0 + jv;
      const T* mu_hi = smu + jv * kMuRow;
#pragma unroll
      for (int j = 0; j < PPL; ++j) {
        const int p = lane + 32 * j;
        if (p < Pn) {
          const T h = mu_hi[p];
          const T l = sizeof(T) == 4 ? mu_hi[kMuLo + p] : T(0);
          if constexpr (kBatch) {
            muh[j][jv] = h;
            mul[j][jv] = l;
          } else {
            lmu[j].add2_fast(h, l);
          }
          if (plast[j]) a.mu_raw[(size_t)v * Pn + p] = (double)h + (double)l;
          if (a.rec_mh) {
            a.rec_mh[(size_t)v * Pn + p] = h;
            a.rec_ml[(size_t)v * Pn + p] = l;
          }
        }
      }
      if (!a.last && qon) {
        T F[QPL], R[QPL], em[QPL], b[QPL], yo[QPL], zo[QPL], fo[QPL];
        lds_n<T, QPL>(st + G.oM + jv * Pp + qo, F);
        lds_n<T, QPL>(st + G.oY + jv * Pp + qo, R);
        lds_n<T, QPL>(st + G.oE + jv * Pp + qo, em);
        lds_n<T, QPL>(st + G.oB + jv * Pp + qo, b);
#pragma unroll
        for (int k = 0; k < QPL; ++k) {
          // f = VF' - cR, r = VR' - cF: the shift comes off the compensated
          // MU_raw first, the small message after
          T f, r;
          if constexpr (sizeof(T) == 4) {
            f = ((mu_hi[qd[k]] - cRh[k]) - F[k]) + (mu_hi[kMuLo + qd[k]] - cRl[k]);
            r = ((mu_hi[qs[k]] - cFh[k]) - R[k]) + (mu_hi[kMuLo + qs[k]] - cFl[k]);
          } else {
            f = (mu_hi[qd[k]] - cRh[k]) - F[k];
            r = (mu_hi[qs[k]] - cFh[k]) - R[k];
          }
          if (qo + k < Pe) {
            mxF[k] = fmax(mxF[k], f);
            mxR[k] = fmax(mxR[k], r);
            if constexpr (kBatch) {
              lrv[k][jv] = f + b[k];
              lfv[k][jv] = r + b[k];
            } else {
              lr[k].add_fast(f + b[k]);
              lf[k].add_fast(r + b[k]);
            }
            yo[k] = f - em[k];  // no out-edges: dEmin = +inf, Y = -inf
            zo[k] = r;
            fo[k] = f;
          } else {
            yo[k] = zo[k] = fo[k] = T(0);
          }
        }
        st_n<T, QPL>(a.vf + (size_t)v * Pp + qo, yo);
        st_n<T, QPL>(a.vr_out + (size_t)v * Pp + qo, zo);
        if (a.rec_f) {
          st_n<T, QPL>(a.rec_f + (size_t)v * Pp + qo, fo);
          st_n<T, QPL>(a.rec_r + (size_t)v * Pp + qo, zo);
        }
      }
    }
    if constexpr (kBatch) {
#pragma unroll
      for (int k = 0; k < QPL; ++k) {
        lr[k].add4_fast(lrv[k][0], lrv[k][1], lrv[k][2], lrv[k][3]);
        lf[k].add4_fast(lfv[k][0], lfv[k][1], lfv[k][2], lfv[k][3]);
      }
#pragma unroll
      for (int j = 0; j < PPL; ++j) lmu[j].add2x4_fast(muh[j], mul[j]);
    }
    __syncwarp();  // this stage's buffer is free for the stage after next
  }
  cp_wait0();
  __syncthreads();  // the rings become the reduction area

  const int nmax = 2 * Pe, nlse = 2 * Pe + Pn, slots = nmax + 2 * nlse;
  double* red = reinterpret_cast<double*>(smem + L.ring);
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
#pragma unroll
  for (int j = 0; j < PPL; ++j) {
    const int p = lane + 32 * j;
    if (p < Pn) {
      r[nmax + 2 * (2 * Pe + p)] = lmu[j].mval();
      r[nmax + 2 * (2 * Pe + p) + 1] = lmu[j].sval();
    }
  }
  __syncthreads();
  write_block_partials(red, kVw, nmax, nlse, a.bpart, gridDim.x, blockIdx.x, sizeof(T) == 4);
}

__global__ void capture_s_kernel(const double* __restrict__ S, const int* __restrict__ iters_p,
                                 int t, double* __restrict__ S_final, int Pn) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < Pn && iters_p[p] == t) S_final[p] = S[p];
}

template <typename T>
__global__ void fill_kernel(T* __restrict__ p, size_t n, T v) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    p[i] = v;
}

#define ACG_EDGE_SHAPES(X) \
  X(1, 1) X(2, 1) X(4, 1) X(8, 1) X(16, 1) X(32, 1) X(32, 2) X(32, 4)

}  // namespace

int edge_step(WarpShape ws) { return (32 / ws.npow) * kU; }

WarpShape choose_warp_shape(int elem_bytes, int pp) {
  const int W = 16 / elem_bytes;
  const int nvec = (pp + W - 1) / W;
  WarpShape ws{32, 1};
  if (nvec <= 32) {
    int np = 1;
    while (np < nvec) np <<= 1;
    ws.npow = np;
    ws.nqv = 1;
  } else {
    ws.npow = 32;
    ws.nqv = nvec <= 64 ? 2 : 4;
  }
  return ws;
}

#define ACG_EDGE_LAUNCH(NP_, NQ_)                                           \
  if (ws.npow == NP_ && ws.nqv == NQ_) {                                    \
    if (a.argpos)                                                           \
      edge_max_kernel<T, NP_, NQ_, true><<<blocks, kAT, 0, s>>>(a);         \
    else                                                                    \
      edge_max_kernel<T, NP_, NQ_, false><<<blocks, kAT, 0, s>>>(a);        \
    ACG_LAUNCH_CHECK();                                                     \
    return ACG_OK;                                                          \
  }

template <typename T>
acg_status launch_edge_max(const EdgeMaxArgs<T>& a, WarpShape ws, int blocks, cudaStream_t s) {
  if (a.nitems == 0) return ACG_OK;
  ACG_EDGE_SHAPES(ACG_EDGE_LAUNCH)
  return set_error(ACG_ERR_UNSUPPORTED, "no edge kernel for npow=%d nqv=%d", ws.npow, ws.nqv);
}

#define ACG_EDGE_OCC(NP_, NQ_)                                                        \
  if (ws.npow == NP_ && ws.nqv == NQ_) {                                             \
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, edge_max_kernel<T, NP_, NQ_, false>, \
                                                      kAT, 0) != cudaSuccess)        \
      nb = 1;                                                                        \
  }

template <typename T>
int edge_max_blocks_per_sm(WarpShape ws) {
  int nb = 1;
  ACG_EDGE_SHAPES(ACG_EDGE_OCC)
  return nb < 1 ? 1 : nb;
}


template <typename T>
acg_status launch_heavy_combine_arg(const T* partial, const int* ppos, const int* hbase,
                                    const int* hcount, const int* hvert, int nheavy, int Pp, T* M,
                                    int* A, cudaStream_t s) {
  if (nheavy == 0) return ACG_OK;
  heavy_combine_arg_kernel<T><<<ceil_div(nheavy, 8), 256, 0, s>>>(partial, ppos, hbase, hcount, hvert,
                                                                   nheavy, Pp, M, A);
  ACG_LAUNCH_CHECK();
  return ACG_OK;
}
template <typename T>
acg_status launch_heavy_combine(const T* partial, const int* hbase, const int* hcount,
                                const int* hvert, int nheavy, int Pp, T* M, cudaStream_t s) {
  if (nheavy == 0) return ACG_OK;
  heavy_combine_kernel<T><<<ceil_div(nheavy, 8), 256, 0, s>>>(partial, hbase, hcount, hvert,
                                                               nheavy, Pp, M);
  ACG_LAUNCH_CHECK();
  return ACG_OK;
}

template <typename T>
size_t vertex_update_smem(int pn, int pe, int pp) {
  const int nvec = pp / VecT<T>::W;
  const int pnp = (pn + VecT<T>::W - 1) / VecT<T>::W * VecT<T>::W;
  return UpdSmem(kBT / nvec, pn, pe, pp, pnp, sizeof(T)).total;
}

template <typename T, int QPL, int PPL>
size_t vertex_warp_setup(int pn, int pe, int pp, int pnp, int nterms) {
  const size_t sm = VwSmem<T, QPL, PPL>(pn, pe, pp, pnp, nterms).total;
  if (sm > 48 * 1024)
    cudaFuncSetAttribute(vertex_warp_kernel<T, QPL, PPL>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  return sm;
}

// Calls f.template operator()<QPL, PPL>() for the warp form's shape; false if
// the pattern is too large for it.
template <typename F>
bool warp_form(int pn, int pp, F&& f) {
  if (pp > 64 || pn > 64) return false;
  if (pp <= 32 && pn <= 32) f.template operator()<1, 1>();
  else if (pp <= 32) f.template operator()<1, 2>();
  else if (pn <= 32) f.template operator()<2, 1>();
  else f.template operator()<2, 2>();
  return true;
}

template <typename T>
acg_status launch_vertex_update(const VertexUpdArgs<T>& a, int blocks, cudaStream_t s) {
  cudaError_t le = cudaSuccess;
  if (a.vsched == nullptr && a.Pn > 0 && a.Pn <= 64 && a.Pp <= 64)
    return set_error(ACG_ERR_INVALID_ARGUMENT, "vertex phase: no schedule for the warp form");
  const bool warp = warp_form(a.Pn, a.Pp, [&]<int QPL, int PPL>() {
    const size_t sm = vertex_warp_setup<T, QPL, PPL>(a.Pn, a.Pe, a.Pp, a.Pnp, a.vterms);
    vertex_warp_kernel<T, QPL, PPL><<<blocks, kBT, sm, s>>>(a);
    le = cudaGetLastError();
  });
  if (warp) {
    if (le != cudaSuccess)
      return set_error(ACG_ERR_CUDA, "vertex_warp_kernel launch: %s", cudaGetErrorString(le));
    return ACG_OK;
  }
  const size_t sm = vertex_update_smem<T>(a.Pn, a.Pe, a.Pp);
  if (sm > 48 * 1024)
    ACG_CUDA_TRY(cudaFuncSetAttribute(vertex_update_kernel<T>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  vertex_update_kernel<T><<<blocks, kBT, sm, s>>>(a);
  ACG_LAUNCH_CHECK();
  return ACG_OK;
}

template <typename T>
int vertex_update_blocks(int pn, int pe, int pp, int pnp, int nterms, int num_sms, int dn) {
  int nb = 0;
  const bool warp = warp_form(pn, pp, [&]<int QPL, int PPL>() {
    const size_t sm = vertex_warp_setup<T, QPL, PPL>(pn, pe, pp, pnp, nterms);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, vertex_warp_kernel<T, QPL, PPL>, kBT,
                                                      sm) != cudaSuccess)
      nb = 1;
  });
  if (warp) return num_sms * (nb < 1 ? 1 : nb);
  const int V = kBT / (pp / VecT<T>::W);
  const long long tiles = (dn + V - 1) / V;
  const long long b = (long long)num_sms * vertex_update_blocks_per_sm<T>(pn, pe, pp);
  return (int)(tiles < 1 ? 1 : (tiles < b ? tiles : b));
}

int vertex_warp_schedule(const int* pat, int pn, int pe, int pp, int pnp, std::vector<uint32_t>* out) {
  return vertex_warp_schedule(pat, pn, pe, pp, pnp, kVps, out);
}

acg_status launch_capture_s(const double* S, const int* iters_p, int t, double* S_final, int Pn,
                            cudaStream_t s) {
  if (Pn == 0) return ACG_OK;
  capture_s_kernel<<<ceil_div(Pn, 128), 128, 0, s>>>(S, iters_p, t, S_final, Pn);
  ACG_LAUNCH_CHECK();
  return ACG_OK;
}

template <typename T>
acg_status launch_fill(T* p, size_t n, T v, cudaStream_t s) {
  if (n == 0) return ACG_OK;
  fill_kernel<T><<<(unsigned)std::min<size_t>((n + 255) / 256, 4096), 256, 0, s>>>(p, n, v);
  ACG_LAUNCH_CHECK();
  return ACG_OK;
}

template <typename T>
int vertex_update_blocks_per_sm(int pn, int pe, int pp) {
  const size_t sm = vertex_update_smem<T>(pn, pe, pp);
  if (sm > 48 * 1024)
    cudaFuncSetAttribute(vertex_update_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  int nb = 1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, vertex_update_kernel<T>, kBT, sm) !=
      cudaSuccess)
    nb = 1;
  return nb < 1 ? 1 : nb;
}

template acg_status launch_edge_max<double>(const EdgeMaxArgs<double>&, WarpShape, int, cudaStream_t);
template acg_status launch_edge_max<float>(const EdgeMaxArgs<float>&, WarpShape, int, cudaStream_t);
template acg_status launch_heavy_combine_arg<double>(const double*, const int*, const int*, const int*, const int*, int, int, double*, int*, cudaStream_t);
template acg_status launch_heavy_combine_arg<float>(const float*, const int*, const int*, const int*, const int*, int, int, float*, int*, cudaStream_t);
template acg_status launch_heavy_combine<double>(const double*, const int*, const int*, const int*, int, int, double*, cudaStream_t);
template acg_status launch_heavy_combine<float>(const float*, const int*, const int*, const int*, int, int, float*, cudaStream_t);
template acg_status launch_vertex_update<double>(const VertexUpdArgs<double>&, int, cudaStream_t);
template acg_status launch_vertex_update<float>(const VertexUpdArgs<float>&, int, cudaStream_t);
template int edge_max_blocks_per_sm<double>(WarpShape);
template int edge_max_blocks_per_sm<float>(WarpShape);
template int vertex_update_blocks<double>(int, int, int, int, int, int, int);
template int vertex_update_blocks<float>(int, int, int, int, int, int, int);
template acg_status launch_fill<double>(double*, size_t, double, cudaStream_t);
template acg_status launch_fill<float>(float*, size_t, float, cudaStream_t);
template int vertex_update_blocks_per_sm<double>(int, int, int);
template int vertex_update_blocks_per_sm<float>(int, int, int);

}  // namespace acg
