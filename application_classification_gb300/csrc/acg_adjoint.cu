// acg_adjoint.cu -- the hand-written adjoint of a match (acg_match_record,
// acg_backward): gradients of sum(grad_mu * mu) with respect to the data and
// pattern vertex and edge features, through cdist, the row log-softmaxes,
// the edge maxima and every BP iteration.
//
// The forward is the production path (acg_api.cu), run with state records:
// acg_match_record keeps the state of every checkpoint iteration (every k-th,
// plus the last).  acg_backward walks the segments between checkpoints from
// the last: it restores the segment's first state, recomputes its iterations
// with the same kernels (bit-identical: every reduction order is fixed), and
// runs the adjoint steps of the segment backwards.  The edge maxima of each
// state and their first maximal in-edge are recorded by the edge phase that
// computes them (the argmax form of edge_max_kernel): in the recorded match for
// the state before each checkpoint, in the recompute for the others.  The
// algebra is that of the
// restructured iteration (the header of acg_bp.cu), unshifted; the numpy model
// tests/adjoint_model.py states every step and is checked against torch
// autograd.  Conventions, matching the forward kernels' arithmetic:
//   * max(fill, b) sends the gradient to b when b > fill, else to the fill;
//   * a column maximum over data vertices sends it to the smallest maximal
//     vertex; a segmented maximum (minimum) over a vertex's edges to its first
//     maximal (minimal) edge in CSR order, i.e. the smallest original edge id;
//   * log-sum-exps send it through their softmax weights.
// Every sum has a fixed order (per-lane sequences, fixed shuffle trees,
// blocks in order): the gradients are bit-reproducible.  The one atomic is an
// integer OR (the per-edge column masks of the maxima), the same in any order.
//
// Limits: single-pattern plans of at most 64 padded edge columns and 64
// pattern vertices (the warp forms), feature dimensions up to 32.  With the
// C-null option, the term's gradient goes to the pattern edge features
// (adj_cnull_*).
#include <cuda_runtime.h>

#include <algorithm>
#include <limits>
#include <memory>
#include <vector>

#include "acg.h"
#include "acg_plan.h"
#include "acg_static.cuh"

using namespace acg;

namespace acg {

struct AdjWork {
  int every = 0, T = 0, nck = 0;
  std::vector<int> ck_t;         // checkpointed states
  StateRec ck;                   // the checkpoints (indexed by state)
  std::vector<void*> sf, sr, smh, sml;  // segment slots (states between checkpoints)
  std::vector<double*> sglob;
  bool recorded = false;
  int vblocks = 0;                 // grid of the per-vertex adjoint kernels
  // work buffers (element type per precision)
  void *gMU = nullptr, *gMU2 = nullptr;            // [Dn][Pn]
  void *gFd = nullptr, *gRd = nullptr;             // [Dn][Pp]
  void *gbR = nullptr, *gM = nullptr, *gVRe = nullptr;  // [Dn][Pp]
  std::vector<void*> sm;                           // segment slots: edge maxima of states t0 ..
  std::vector<int*> sa;                            //   and their argmax positions ([Dn][Pp])
  int seg_t0 = 0;                                  // first state of the segment being processed
  unsigned long long* emask = nullptr;             // [De] columns each edge is the maximum of
  void *gdEmin = nullptr, *gB = nullptr;           // [Dn][Pp]
  void* gCV = nullptr;                             // [Dn][Pn]
  void* gdE = nullptr;                             // [De][Pp]
  void *gRb = nullptr, *gFb = nullptr;             // [Dn][Pqc]
  int* ppos = nullptr;                             // [edge-side partial rows][Pp]: hub chunk positions
  void* pscat = nullptr;                           // [src partial rows][Pp]
  void* pstat = nullptr;                           // [src partial rows][4 Pp]
  int* pstati = nullptr;                           // [src partial rows][2 Pp]
  void* pq = nullptr;                              // [dst partial rows][Pqc]
  int* pqi = nullptr;                              // [dst partial rows][2 Pqc]
  double* part = nullptr;                          // column partials
  int* parti = nullptr;
  double* cols = nullptr;                          // [8 Pe + 2 Pn + 8]
  int* colsi = nullptr;                            // [2 Pe + Pn]
  double* ypart = nullptr;                         // pattern-gradient partials
  double* gcn = nullptr;                           // [Pe] gradient into the C-null term (option cnull)
  std::vector<DevBuf> owned;
  // the backward as one CUDA graph (its launches are the same on every call
  // with the same gradient pointers), captured on a stream of its own
  cudaGraphExec_t gexec = nullptr;
  cudaStream_t gstream = nullptr;
  const void* gkey[5] = {};
  bool gfailed = false;  // capture refused once: launch directly from then on
  void drop_graph() {
    if (gexec) cudaGraphExecDestroy(gexec);
    gexec = nullptr;
  }
};

void adj_free(acg_plan* P) {
  if (!P || !P->adj) return;
  dev_free_all(&P->adj->owned);
  P->adj->drop_graph();
  if (P->adj->gstream) cudaStreamDestroy(P->adj->gstream);
  delete P->adj;
  P->adj = nullptr;
}

}  // namespace acg

namespace {

constexpr int kT = 256;
constexpr int kW = kT / 32;
#ifndef ACG_ADJ_KU
#define ACG_ADJ_KU 4
#endif
#ifndef ACG_ADJ_MINB
#define ACG_ADJ_MINB 0
#endif
constexpr int kU = ACG_ADJ_KU;  // gather steps in flight (edge-max argmax, max-gradient scatter)
#if ACG_ADJ_MINB > 0
#define ACG_ADJ_BOUNDS __launch_bounds__(kT, ACG_ADJ_MINB)
#else
#define ACG_ADJ_BOUNDS __launch_bounds__(kT)
#endif

template <typename T>
struct AV;
template <>
struct AV<double> {
  using type = double2;
  static constexpr int W = 2;
};
template <>
struct AV<float> {
  using type = float4;
  static constexpr int W = 4;
};
template <typename T>
__device__ __forceinline__ T ag(const typename AV<T>::type& v, int w) {
  return reinterpret_cast<const T*>(&v)[w];
}
__device__ __forceinline__ float ex(float x) { return expf(x); }
__device__ __forceinline__ double ex(double x) { return exp(x); }

// ------------------------------------------------------------ column helpers
// Block partials of per-lane column values: red[warp][col] in shared memory is
// combined over the warps in order and written to part[col][block].
__device__ void block_sums_out(double* red, int ncol, double* part) {
  __syncthreads();
  for (int c = threadIdx.x; c < ncol; c += kT) {
    double s = 0;
    for (int w = 0; w < kW; ++w) s += red[w * ncol + c];
    part[(size_t)c * gridDim.x + blockIdx.x] = s;
  }
}
// Argmax partials: (value, index) per warp, combined in warp order (strict >:
// earlier warps cover smaller indices).
__device__ void block_argmax_out(const double* rv, const int* ri, int ncol, double* pv, int* pi) {
  __syncthreads();
  for (int c = threadIdx.x; c < ncol; c += kT) {
    double b = -CUDART_INF;
    int bi = -1;
    for (int w = 0; w < kW; ++w)
      if (ri[w * ncol + c] >= 0 && (bi < 0 || rv[w * ncol + c] > b)) {
        b = rv[w * ncol + c];
        bi = ri[w * ncol + c];
      }
    pv[(size_t)c * gridDim.x + blockIdx.x] = b;
    pi[(size_t)c * gridDim.x + blockIdx.x] = bi;
  }
}

// One warp per column: out[c] = the sum of part[c][0, nblk) (lane-strided
// partial sums, then a fixed shuffle tree: deterministic); argmax columns: the
// first maximal index (the blocks cover increasing vertex ranges, and ties go
// to the smaller index).
__global__ void col_final_kernel(const double* __restrict__ part, int nsum, const double* __restrict__ pv,
                                 const int* __restrict__ pi, int narg, int nblk, double* __restrict__ out,
                                 int* __restrict__ outi) {
  const int c = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
  if (c < nsum) {
    double s = 0;
    for (int b = lane; b < nblk; b += 32) s += part[(size_t)c * nblk + b];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) out[c] = s;
  } else if (c < nsum + narg) {
    const int j = c - nsum;
    double bv = -CUDART_INF;
    int bi = -1;
    for (int b = lane; b < nblk; b += 32) {
      const int i = pi[(size_t)j * nblk + b];
      if (i >= 0 && (bi < 0 || pv[(size_t)j * nblk + b] > bv)) {
        bv = pv[(size_t)j * nblk + b];
        bi = i;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double ov = __shfl_down_sync(0xffffffffu, bv, o);
      const int oi = __shfl_down_sync(0xffffffffu, bi, o);
      if (oi >= 0 && (bi < 0 || ov > bv || (ov == bv && oi < bi))) {
        bv = ov;
        bi = oi;
      }
    }
    if (lane == 0) outi[j] = bi;
  }
}

// part[c][block] = sum over the block's rows of x[row][c] (c < ncol), rows in order.
template <typename S>
__global__ void col_sum_kernel(const S* __restrict__ x, int ld, int ncol, long long rows,
                               double* __restrict__ part) {
  const long long r0 = rows * blockIdx.x / gridDim.x, r1 = rows * (blockIdx.x + 1) / gridDim.x;
  for (int c = threadIdx.x; c < ncol; c += blockDim.x) {
    double s = 0;
    for (long long r = r0; r < r1; ++r) s += (double)x[(size_t)r * ld + c];
    part[(size_t)c * gridDim.x + blockIdx.x] = s;
  }
}

// gMU(T)[v][p] = gmu[v][p] - exp(MU(T)[v][p] - S(T)[p]) * colsum_p(gmu)
template <typename T>
__global__ void top_grad_kernel(const double* __restrict__ gmu, const T* __restrict__ mh,
                                const T* __restrict__ ml, const double* __restrict__ S,
                                const double* __restrict__ cs, long long n, int Pn, T* __restrict__ gMU) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int p = (int)(i % Pn);
  const T Sh = (T)S[p], Sl = (T)(S[p] - (double)Sh);
  const T x = (mh[i] - Sh) + (ml[i] - Sl);
  gMU[i] = (T)(gmu[i] - cs[p] * (double)ex(x));
}

// Y = f - dEmin (the working Y of a restored state, the forward's operation;
// zero past Pe as the forward writes it)
template <typename T>
__global__ void restore_y_kernel(const T* __restrict__ f, const T* __restrict__ em, long long n,
                                 int Pp, int Pe, T* __restrict__ y) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = (int)(i % Pp) < Pe ? f[i] - em[i] : T(0);
}

template <typename T>
__global__ void copy_cast_kernel(const double* __restrict__ a, T* __restrict__ b, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (T)a[i];
}

template <typename T>
__global__ void fill_t_kernel(T* __restrict__ p, size_t n, T v) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    p[i] = v;
}

// --------------------------------------------- gradient through the maxima
// For each source s (source CSR): gVRe[s][q] = sum over its out-edges e whose
// destination v has its maximum at column q on e (A[v][q] == e) of gM[v][q].
// Step A, which holds gM[v][q] and reads A[v][q], makes the matching
// gdE[e][q] -= gM[v][q] and sets bit q of emask[e] (an OR: the same in any
// order), so this pass reads 8 bytes per out-edge.
template <typename T>
struct ScatArgs {
  const int4* items;
  const int* wsplit;
  const int* row_of;   // dst-CSR position of each src-CSR position
  const int* dst_of;   // destination vertex of each src-CSR position
  const unsigned long long* emask;  // [De] bit q: edge (dst-CSR position) is the maximum at column q
  const T* gM;
  T* gVRe;
  T* part;
  int Pp, Pe;
  int nranges;         // item ranges: warp w does range w, then claims from ctr
  int* ctr;            // (two zeroed ints, reset by the last warp; null: ranges
                       // w, w + warps, ...)
};

template <typename T, int NPOW, int NQV>
__global__ void ACG_ADJ_BOUNDS adj_scatter_kernel(const ScatArgs<T> a) {
  constexpr int W = AV<T>::W, S = 32 / NPOW, NQ = NQV * W;
  const int Pp = a.Pp, Pe = a.Pe, lane = threadIdx.x & 31, slot = lane / NPOW, qc = lane % NPOW;
  const int gw = (blockIdx.x * kT + threadIdx.x) >> 5;
  const int nw = (int)gridDim.x * (kT / 32);
  for (int r = gw; r < a.nranges;) {
  int rn = r + nw;  // the next range: claimed (in flight while this one runs) or strided
  if (a.ctr && lane == 0) rn = nw + atomicAdd(a.ctr, 1);
  for (int it = a.wsplit[r]; it < a.wsplit[r + 1]; ++it) {
    const int4 item = a.items[it];
    T acc[NQ];
#pragma unroll
    for (int k = 0; k < NQ; ++k) acc[k] = T(0);
    for (int base = item.y; base < item.z; base += S * kU) {
      int e[kU], vd[kU];
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        const int j = base + slot + S * u;
        const bool ok = j < item.z;
        e[u] = ok ? __ldg(a.row_of + j) : -1;
        vd[u] = ok ? __ldg(a.dst_of + j) : 0;
      }
      unsigned long long mk[kU];
#pragma unroll
      for (int u = 0; u < kU; ++u) mk[u] = e[u] >= 0 ? __ldg(a.emask + e[u]) : 0ull;
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        if (mk[u] == 0ull) continue;
#pragma unroll
        for (int k = 0; k < NQV; ++k) {
#pragma unroll
          for (int w = 0; w < W; ++w) {
            const int q = (qc + NPOW * k) * W + w;
            if (q < Pe && ((mk[u] >> q) & 1ull))
              acc[k * W + w] += a.gM[(size_t)vd[u] * Pp + q];
          }
        }
      }
    }
#pragma unroll
    for (int o = NPOW; o < 32; o <<= 1)
#pragma unroll
      for (int k = 0; k < NQ; ++k) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], o);
    if (slot == 0) {
      T* row = item.w >= 0 ? a.part + (size_t)item.w * Pp : a.gVRe + (size_t)item.x * Pp;
#pragma unroll
      for (int k = 0; k < NQV; ++k)
#pragma unroll
        for (int w = 0; w < W; ++w) {
          const int q = (qc + NPOW * k) * W + w;
          if (q < Pp) row[q] = acc[k * W + w];
        }
    }
    __syncwarp();
  }
  r = a.ctr ? __shfl_sync(0xffffffffu, rn, 0) : rn;
  }
  if (a.ctr && lane == 0) {
    __threadfence();  // this warp's claims come before its finish count
    if (atomicAdd(a.ctr + 1, 1) == nw - 1) {  // every warp has made its last claim
      a.ctr[0] = 0;
      a.ctr[1] = 0;
    }
  }
}

template <typename T>
__global__ void adj_sum_combine_kernel(const T* __restrict__ part, const int* __restrict__ hbase,
                                       const int* __restrict__ hcount, const int* __restrict__ hvert,
                                       int nheavy, int Pp, T* __restrict__ out) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= nheavy) return;
  for (int q = lane; q < Pp; q += 32) {
    T s = T(0);
    for (int c = 0; c < hcount[warp]; ++c) s += part[(size_t)(hbase[warp] + c) * Pp + q];
    out[(size_t)hvert[warp] * Pp + q] = s;
  }
}

// --------------------------------------------------------- vertex steps
// Lanes own pattern columns as in the forward's warp form: lane l owns edge
// columns q = l * QPL + k and pattern vertices p = l + 32 j.

// Step A (per vertex): the gradients into this iteration's messages, the max
// selections, and column sums: gaR, gaF (into the fills), GbR, GbF (into
// the log-sum-exps), with the argmax vertex of f and r per column.
template <typename T>
struct StepAArgs {
  const T* gMU;       // [Dn][Pn] gradient into MU(t)
  const T* gFd;       // [Dn][Pp] direct gradient into F(t) (null at t = T)
  const T* gRd;
  const T* f;         // [Dn][Pp] f(t-1) = VF(t-1) - cR(t-1)
  const T* r;         // [Dn][Pp] r(t-1)
  const T* M;         // [Dn][Pp] edge maxima of state t-1
  const int* A;       // [Dn][Pp] their first maximal destination-CSR positions
  T* gdE;             // accumulated [De][Pp]
  unsigned long long* emask;  // [De] out: the columns each edge is the maximum of (nonzero gradient)
  const T* dEmin;
  const double* glob; // statistics of state t-1
  const int* pat;
  T* gbR;             // out [Dn][Pp]
  T* gM;              // out [Dn][Pp]
  T* gdEmin;          // accumulated [Dn][Pp]
  T* gCV;             // accumulated [Dn][Pn]
  double* part;       // [4 Pe][blocks] sums
  double* pv;         // [2 Pe][blocks] argmax values
  int* pi;
  int Dn, Pn, Pe, Pp;
  const double* cnull;  // [Pe] the C-null term subtracted from both fills (option cnull), or null
};

template <typename T, int QPL, int PPL>
__global__ void __launch_bounds__(kT) adj_stepA_kernel(const StepAArgs<T> a) {
  extern __shared__ __align__(16) unsigned char sm[];
  const int Pe = a.Pe, Pn = a.Pn, Pp = a.Pp;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  T* sg = reinterpret_cast<T*>(sm) + (size_t)wib * 64 * PPL;       // gMU row of the warp's vertex
  double* red = reinterpret_cast<double*>(sm + sizeof(T) * kW * 64 * PPL);  // [kW][4 Pe]
  double* rv = red + (size_t)kW * 4 * Pe;                            // [kW][2 Pe]
  int* ri = reinterpret_cast<int*>(rv + (size_t)kW * 2 * Pe);        // [kW][2 Pe]
  const int* psrc = a.pat;
  const int* pdst = a.pat + Pe;
  const double* g = a.glob;
  const int x0 = 4 * Pe + Pn;
  const int qo = lane * QPL;
  T fR[QPL], fF[QPL], dRh[QPL], dRl[QPL], dFh[QPL], dFl[QPL];
  int qd[QPL], qs[QPL];
  double sa[QPL][4];
  T bf[QPL], br[QPL];
  int af[QPL], ar[QPL];
#pragma unroll
  for (int k = 0; k < QPL; ++k) {
    const int q = qo + k;
    fR[k] = fF[k] = dRh[k] = dRl[k] = dFh[k] = dFl[k] = T(0);
    qd[k] = qs[k] = 0;
    if (q < Pe) {
      qd[k] = pdst[q];
      qs[k] = psrc[q];
      // the fills and constants exactly as the forward's vertex phase forms them
      double fr = g[q] + g[x0 + q] - g[4 * Pe + qd[k]];
      double ff = g[Pe + q] + g[x0 + Pe + q] - g[4 * Pe + qs[k]];
      if (a.cnull) {
        fr -= a.cnull[q];
        ff -= a.cnull[q];
      }
      fR[k] = (T)fr;
      fF[k] = (T)ff;
      const double dR = g[2 * Pe + q], dF = g[3 * Pe + q];
      dRh[k] = (T)dR;
      dRl[k] = (T)(dR - (double)dRh[k]);
      dFh[k] = (T)dF;
      dFl[k] = (T)(dF - (double)dFh[k]);
    }
#pragma unroll
    for (int c = 0; c < 4; ++c) sa[k][c] = 0;
    bf[k] = br[k] = neg_inf<T>();
    af[k] = ar[k] = -1;
  }
  const long long nw = (long long)gridDim.x * kW, gw = (long long)blockIdx.x * kW + wib;
  const int vb = (int)(gw * a.Dn / nw), ve = (int)((gw + 1) * a.Dn / nw);
  for (int v = vb; v < ve; ++v) {
#pragma unroll
    for (int j = 0; j < PPL; ++j) {
      const int p = lane + 32 * j;
      if (p < Pn) {
        const T x = a.gMU[(size_t)v * Pn + p];
        sg[p] = x;
        a.gCV[(size_t)v * Pn + p] -= x;
      }
    }
    __syncwarp();
#pragma unroll
    for (int k = 0; k < QPL; ++k) {
      const int q = qo + k;
      if (q >= Pe) continue;
      const size_t i = (size_t)v * Pp + q;
      const T gF = sg[qd[k]] + (a.gFd ? a.gFd[i] : T(0));
      const T gR = sg[qs[k]] + (a.gRd ? a.gRd[i] : T(0));
      const T f = a.f[i], r = a.r[i];
      const T Y = f - a.dEmin[i];
      const bool sR = ((Y - dRh[k]) - dRl[k]) > fR[k];
      const bool sF = ((a.M[i] - dFh[k]) - dFl[k]) > fF[k];
      const T gb = sR ? gR : T(0), gm = sF ? gF : T(0);
      a.gbR[i] = gb;
      a.gM[i] = gm;
      // the maximum's -dE term: each (edge, column) is the maximum of one vertex
      if (gm != T(0)) {
        const int e = __ldg(a.A + i);
        a.gdE[(size_t)e * Pp + q] -= gm;
        atomicOr(a.emask + e, 1ull << q);
      }
      a.gdEmin[i] -= gb;
      sa[k][0] += sR ? 0.0 : (double)gR;
      sa[k][1] += sF ? 0.0 : (double)gF;
      sa[k][2] += (double)gb;
      sa[k][3] += (double)gm;
      if (af[k] < 0 || f > bf[k]) {
        bf[k] = f;
        af[k] = v;
      }
      if (ar[k] < 0 || r > br[k]) {
        br[k] = r;
        ar[k] = v;
      }
    }
    __syncwarp();
  }
#pragma unroll
  for (int k = 0; k < QPL; ++k) {
    const int q = qo + k;
    if (q < Pe) {
#pragma unroll
      for (int c = 0; c < 4; ++c) red[(size_t)wib * 4 * Pe + c * Pe + q] = sa[k][c];
      rv[(size_t)wib * 2 * Pe + q] = (double)bf[k];
      ri[(size_t)wib * 2 * Pe + q] = af[k];
      rv[(size_t)wib * 2 * Pe + Pe + q] = (double)br[k];
      ri[(size_t)wib * 2 * Pe + Pe + q] = ar[k];
    }
  }
  block_sums_out(red, 4 * Pe, a.part);
  block_argmax_out(rv, ri, 2 * Pe, a.pv, a.pi);
}

// Step B (per vertex): gradients into VF(t-1), VR(t-1) -- b of R, the fills'
// argmax vertices, the log-sum-exps' softmax weights, the edge maxima through
// gVRe -- then into MU(t-1) (gathered over each pattern vertex's edges, plus
// the column log-sum-exp S(t-1) of MU(t-1) through its softmax), and the direct
// terms -gVF, -gVR into F(t-1), R(t-1).
template <typename T>
struct StepBArgs {
  const T* gbR;
  const T* gVRe;
  const double* cols;  // gaR | gaF | GbR | GbF  (Pe each)
  const int* colsi;    // argmax vertex of f | of r (Pe each)
  const T* f;
  const T* r;
  const T* B;
  const double* glob;  // statistics of state t-1
  const T* mh;         // MU(t-1) hi, lo (null at t - 1 = 0: S(0) is constant)
  const T* ml;
  const int* pat;
  T* gB;               // accumulated
  T* gMU;              // out [Dn][Pn] gradient into MU(t-1)
  T* gFd;              // out [Dn][Pp] -gVF(t-1)
  T* gRd;
  int Dn, Pn, Pe, Pp, maxdeg;
};

template <typename T, int QPL, int PPL>
__global__ void __launch_bounds__(kT) adj_stepB_kernel(const StepBArgs<T> a) {
  extern __shared__ __align__(16) unsigned char sm[];
  const int Pe = a.Pe, Pn = a.Pn, Pp = a.Pp, maxdeg = a.maxdeg;
  const int tid = threadIdx.x, lane = tid & 31, wib = tid >> 5;
  constexpr int kZ = 2 * 32 * QPL;  // a zero in the per-warp gVF | gVR array
  int* s_inc = reinterpret_cast<int*>(sm);                              // [PPL][maxdeg][32]
  T* sgr = reinterpret_cast<T*>(sm + ((sizeof(int) * (size_t)PPL * maxdeg * 32 + 15) & ~size_t(15))) +
           (size_t)wib * (kZ + 4);
  const int* psrc = a.pat;
  const int* pdst = a.pat + Pe;
  const int* inoff = a.pat + 2 * Pe;
  const int* inq = inoff + Pn + 1;
  const int* outoff = inq + Pe;
  const int* outq = outoff + Pn + 1;
  for (int i = tid; i < PPL * maxdeg * 32; i += kT) {
    const int l = i & 31, t = (i >> 5) % maxdeg, j = (i >> 5) / maxdeg, p = l + 32 * j;
    int code = kZ;
    if (p < Pn) {
      const int nin = inoff[p + 1] - inoff[p], nout = outoff[p + 1] - outoff[p];
      if (t < nin)
        code = inq[inoff[p] + t];
      else if (t < nin + nout)
        code = 32 * QPL + outq[outoff[p] + t - nin];
    }
    s_inc[i] = code;
  }
  if (lane < 4) sgr[kZ + lane] = T(0);
  const double* g = a.glob;
  const int qo = lane * QPL;
  T gaR[QPL], gaF[QPL], glR[QPL], glF[QPL], dRh[QPL], dRl[QPL], dFh[QPL], dFl[QPL];
  int vfa[QPL], vra[QPL];
#pragma unroll
  for (int k = 0; k < QPL; ++k) {
    const int q = qo + k;
    gaR[k] = gaF[k] = glR[k] = glF[k] = dRh[k] = dRl[k] = dFh[k] = dFl[k] = T(0);
    vfa[k] = vra[k] = -1;
    if (q < Pe) {
      gaR[k] = (T)a.cols[q];
      gaF[k] = (T)a.cols[Pe + q];
      glR[k] = (T)(-a.cols[2 * Pe + q]);
      glF[k] = (T)(-a.cols[3 * Pe + q]);
      vfa[k] = a.colsi[q];
      vra[k] = a.colsi[Pe + q];
      const double dR = g[2 * Pe + q], dF = g[3 * Pe + q];
      dRh[k] = (T)dR;
      dRl[k] = (T)(dR - (double)dRh[k]);
      dFh[k] = (T)dF;
      dFl[k] = (T)(dF - (double)dFh[k]);
    }
  }
  // gradient into S(t-1)[p]: minus the fills' shares of its edges
  T gS[PPL], Sh[PPL], Sl[PPL];
#pragma unroll
  for (int j = 0; j < PPL; ++j) {
    const int p = lane + 32 * j;
    double x = 0;
    if (p < Pn) {
      for (int t = inoff[p]; t < inoff[p + 1]; ++t) x -= a.cols[inq[t]];        // dst_q = p: gaR
      for (int t = outoff[p]; t < outoff[p + 1]; ++t) x -= a.cols[Pe + outq[t]];  // src_q = p: gaF
    }
    gS[j] = (T)x;
    const double S = p < Pn ? g[4 * Pe + p] : 0.0;
    Sh[j] = (T)S;
    Sl[j] = (T)(S - (double)Sh[j]);
  }
  __syncthreads();
  const long long nw = (long long)gridDim.x * kW, gw = (long long)blockIdx.x * kW + wib;
  const int vb = (int)(gw * a.Dn / nw), ve = (int)((gw + 1) * a.Dn / nw);
  for (int v = vb; v < ve; ++v) {
#pragma unroll
    for (int k = 0; k < QPL; ++k) {
      const int q = qo + k;
      if (q >= Pp) continue;
      const size_t i = (size_t)v * Pp + q;
      T gvf = T(0), gvr = T(0);
      if (q < Pe) {
        const T b = a.B[i];
        // softmax weights of the log-sum-exps (no out-edges: B = -inf, weight 0)
        const bool hb = b > neg_inf<T>();
        const T wR = hb ? ex(((a.f[i] + b) - dRh[k]) - dRl[k]) : T(0);
        const T wF = hb ? ex(((a.r[i] + b) - dFh[k]) - dFl[k]) : T(0);
        gvf = a.gbR[i] + (v == vfa[k] ? gaR[k] : T(0)) + glR[k] * wR;
        gvr = a.gVRe[i] + (v == vra[k] ? gaF[k] : T(0)) + glF[k] * wF;
        a.gB[i] += glR[k] * wR + glF[k] * wF;
      }
      a.gFd[i] = -gvf;
      a.gRd[i] = -gvr;
      sgr[q] = gvf;
      sgr[32 * QPL + q] = gvr;
    }
    __syncwarp();
#pragma unroll
    for (int j = 0; j < PPL; ++j) {
      const int p = lane + 32 * j;
      if (p >= Pn) continue;
      T acc = T(0);
      const int* inc = s_inc + j * maxdeg * 32 + lane;
      for (int t = 0; t < maxdeg; ++t) acc += sgr[inc[t * 32]];
      if (a.mh) {
        const size_t i = (size_t)v * Pn + p;
        acc += gS[j] * ex((a.mh[i] - Sh[j]) + (a.ml[i] - Sl[j]));
      }
      a.gMU[(size_t)v * Pn + p] = acc;
    }
    __syncwarp();
  }
}

// ------------------------------------------------------------- init step
// The first messages R0 = max(vfmax0, Rbuf - lbuf), F0 = max(vrmax0, Fbuf -
// lbuf) (the init kernel's arithmetic): gradients into the quirk maxima (gRb,
// gFb, columns < qcov), column sums -(sum gRb + sum gFb) into lbuf and the
// fills' shares, and the argmax vertex of each column of MU0.
template <typename T>
struct InitBArgs {
  const int* d_off;
  const int* s_off;
  const T* gR0;
  const T* gF0;
  const T* Rq;
  const T* Fq;
  const T* mh;         // MU0 hi, lo
  const T* ml;
  const double* gv;
  const double* ge;
  const long long* qlim_col;
  const int* pat;
  T* gRb;              // out [Dn][Pqc]
  T* gFb;
  double* part;        // [3 Pe][blocks]: glbuf | gvf0 | gvr0
  double* pv;          // [Pn][blocks] argmax of MU0 columns
  int* pi;
  long long De;
  int Dn, Pn, Pe, Pp, Pqc, qcov;
};

template <typename T, int QPL, int PPL>
__global__ void __launch_bounds__(kT) adj_initB_kernel(const InitBArgs<T> a) {
  extern __shared__ __align__(16) unsigned char sm[];
  const int Pe = a.Pe, Pn = a.Pn, Pp = a.Pp, Pqc = a.Pqc, qcov = a.qcov;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  double* red = reinterpret_cast<double*>(sm);            // [kW][3 Pe]
  double* rv = red + (size_t)kW * 3 * Pe;                 // [kW][Pn]
  int* ri = reinterpret_cast<int*>(rv + (size_t)kW * Pn);
  const int* psrc = a.pat;
  const int* pdst = a.pat + Pe;
  const double* gv = a.gv;
  const int qo = lane * QPL;
  T vfm[QPL], vrm[QPL], lbh[QPL], lbl[QPL];
  double sa[QPL][3];
#pragma unroll
  for (int k = 0; k < QPL; ++k) {
    const int q = qo + k;
    vfm[k] = vrm[k] = lbh[k] = lbl[k] = T(0);
    sa[k][0] = sa[k][1] = sa[k][2] = 0;
    if (q < Pe) {
      vfm[k] = (T)(gv[pdst[q]] - gv[2 * Pn + pdst[q]]);
      vrm[k] = (T)(gv[psrc[q]] - gv[2 * Pn + psrc[q]]);
      long long covered = a.qlim_col[q];
      covered = covered < 0 ? 0 : (covered > a.De ? a.De : covered);
      LseD r;
      r.init();
      if (a.ge[q] > -CUDART_INF) r.merge(a.ge[q], 1.0);
      if (a.De - covered > 0) r.merge(0.0, (double)(a.De - covered));
      const double lb = r.value();
      lbh[k] = (T)lb;
      lbl[k] = (T)(lb - (double)lbh[k]);
    }
  }
  T bm[PPL], bl[PPL];
  int am[PPL];
#pragma unroll
  for (int j = 0; j < PPL; ++j) {
    bm[j] = bl[j] = neg_inf<T>();
    am[j] = -1;
  }
  const long long nw = (long long)gridDim.x * kW, gw = (long long)blockIdx.x * kW + wib;
  const int vb = (int)(gw * a.Dn / nw), ve = (int)((gw + 1) * a.Dn / nw);
  for (int v = vb; v < ve; ++v) {
    const bool hin = a.d_off[v + 1] > a.d_off[v], hout = a.s_off[v + 1] > a.s_off[v];
#pragma unroll
    for (int k = 0; k < QPL; ++k) {
      const int q = qo + k;
      if (q >= Pe) continue;
      const size_t i = (size_t)v * Pp + q;
      const T rb = q < qcov ? a.Rq[(size_t)v * Pqc + q] : T(0);
      const T fb = q < qcov ? a.Fq[(size_t)v * Pqc + q] : T(0);
      const bool sR = hout && ((rb - lbh[k]) - lbl[k]) > vfm[k];
      const bool sF = hin && ((fb - lbh[k]) - lbl[k]) > vrm[k];
      const T gR = a.gR0[i], gF = a.gF0[i];
      if (q < Pqc) {
        a.gRb[(size_t)v * Pqc + q] = sR ? gR : T(0);
        a.gFb[(size_t)v * Pqc + q] = sF ? gF : T(0);
      }
      sa[k][0] -= (sR ? (double)gR : 0.0) + (sF ? (double)gF : 0.0);
      sa[k][1] += sR ? 0.0 : (double)gR;
      sa[k][2] += sF ? 0.0 : (double)gF;
    }
#pragma unroll
    for (int j = 0; j < PPL; ++j) {
      const int p = lane + 32 * j;
      if (p >= Pn) continue;
      // MU0 = hi + lo compared as the pair (the maximum of -dV the init used)
      const T xh = a.mh[(size_t)v * Pn + p], xl = a.ml[(size_t)v * Pn + p];
      if (am[j] < 0 || xh > bm[j] || (xh == bm[j] && xl > bl[j])) {
        bm[j] = xh;
        bl[j] = xl;
        am[j] = v;
      }
    }
  }
#pragma unroll
  for (int k = 0; k < QPL; ++k) {
    const int q = qo + k;
    if (q < Pe)
#pragma unroll
      for (int c = 0; c < 3; ++c) red[(size_t)wib * 3 * Pe + c * Pe + q] = sa[k][c];
  }
#pragma unroll
  for (int j = 0; j < PPL; ++j) {
    const int p = lane + 32 * j;
    if (p < Pn) {
      rv[(size_t)wib * Pn + p] = (double)bm[j] + (double)bl[j];
      ri[(size_t)wib * Pn + p] = am[j];
    }
  }
  block_sums_out(red, 3 * Pe, a.part);
  block_argmax_out(rv, ri, Pn, a.pv, a.pi);
}

// gMU0[argmax_v MU0[., p]][p] += the fills' shares of p's edges
__global__ void adj_init_fill_kernel(const double* __restrict__ cols, const int* __restrict__ am,
                                     const int* __restrict__ pat, int Pn, int Pe, double* g64,
                                     float* g32) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= Pn || am[p] < 0) return;
  const int* inoff = pat + 2 * Pe;
  const int* inq = inoff + Pn + 1;
  const int* outoff = inq + Pe;
  const int* outq = outoff + Pn + 1;
  double x = 0;
  for (int t = inoff[p]; t < inoff[p + 1]; ++t) x += cols[Pe + inq[t]];         // gvf0: dst_q = p
  for (int t = outoff[p]; t < outoff[p + 1]; ++t) x += cols[2 * Pe + outq[t]];  // gvr0: src_q = p
  const size_t i = (size_t)am[p] * Pn + p;
  if (g64) g64[i] += x;
  else g32[i] += (float)x;
}

// ------------------------------------------- quirk rows, destination side
// Per in-edge element of the covered columns: the lbuf softmax term into gdE
// (buf = -dE where covered), and the first maximal element of each vertex's
// quirk maximum, which receives gFb when it is a covered one.
template <typename T>
struct QuirkArgs {
  const int4* items;
  const int* wsplit;
  const int* eid;
  const T* dE;
  const T* gFb;        // [Dn][Pqc]
  const double* ge;
  const long long* qlim_col;
  const double* cols;  // glbuf in [0, Pe)
  T* gdE;
  T* pval;             // [npartial][Pqc]
  int* ppos;           // [npartial][2 Pqc]: position, covered
  long long De;
  int Pp, Pqc, qcov;
  int nranges;         // item ranges; warp w does ranges w, w + warps, ...
};

template <typename T, int NPOW, int NQV>
__global__ void __launch_bounds__(kT) adj_quirk_dst_kernel(const QuirkArgs<T> a) {
  constexpr int W = AV<T>::W, S = 32 / NPOW, NQ = NQV * W;
  const int Pp = a.Pp, Pqc = a.Pqc, lane = threadIdx.x & 31, slot = lane / NPOW, qc = lane % NPOW;
  const int gw = (blockIdx.x * kT + threadIdx.x) >> 5;
  long long qlim[NQ];
  double lb[NQ], gl[NQ];
#pragma unroll
  for (int k = 0; k < NQ; ++k) {
    const int q = (qc + NPOW * (k / W)) * W + k % W;
    qlim[k] = q < a.qcov ? a.qlim_col[q] : 0;
    lb[k] = 0;
    gl[k] = 0;
    if (q < a.qcov) {
      long long covered = qlim[k] < 0 ? 0 : (qlim[k] > a.De ? a.De : qlim[k]);
      LseD r;
      r.init();
      if (a.ge[q] > -CUDART_INF) r.merge(a.ge[q], 1.0);
      if (a.De - covered > 0) r.merge(0.0, (double)(a.De - covered));
      lb[k] = r.value();
      gl[k] = a.cols[q];
    }
  }
  const int nw = (int)gridDim.x * (kT / 32);
  for (int r = gw; r < a.nranges; r += nw)
  for (int it = a.wsplit[r]; it < a.wsplit[r + 1]; ++it) {
    const int4 item = a.items[it];
    T best[NQ];
    int pos[NQ], cov[NQ];
#pragma unroll
    for (int k = 0; k < NQ; ++k) {
      best[k] = neg_inf<T>();
      pos[k] = -1;
      cov[k] = 0;
    }
    for (int e = item.y + slot; e < item.z; e += S) {
      const long long id = __ldg(a.eid + e);
#pragma unroll
      for (int k = 0; k < NQ; ++k) {
        const int q = (qc + NPOW * (k / W)) * W + k % W;
        if (q >= a.qcov) continue;
        const bool c = id < qlim[k];
        const size_t i = (size_t)e * Pp + q;
        const T d = a.dE[i];
        const T buf = c ? -d : T(0);
        if (c) a.gdE[i] -= (T)(gl[k] * exp((double)buf - lb[k]));
        if (pos[k] < 0 || buf > best[k]) {
          best[k] = buf;
          pos[k] = e;
          cov[k] = c;
        }
      }
    }
#pragma unroll
    for (int o = NPOW; o < 32; o <<= 1)
#pragma unroll
      for (int k = 0; k < NQ; ++k) {
        const T ob = __shfl_xor_sync(0xffffffffu, best[k], o);
        const int op = __shfl_xor_sync(0xffffffffu, pos[k], o);
        const int oc = __shfl_xor_sync(0xffffffffu, cov[k], o);
        if (op >= 0 && (pos[k] < 0 || ob > best[k] || (ob == best[k] && op < pos[k]))) {
          best[k] = ob;
          pos[k] = op;
          cov[k] = oc;
        }
      }
    __syncwarp();
    if (slot == 0) {
#pragma unroll
      for (int k = 0; k < NQ; ++k) {
        const int q = (qc + NPOW * (k / W)) * W + k % W;
        if (q >= Pqc) continue;
        if (item.w >= 0) {
          a.pval[(size_t)item.w * Pqc + q] = best[k];
          a.ppos[(size_t)item.w * 2 * Pqc + q] = pos[k];
          a.ppos[(size_t)item.w * 2 * Pqc + Pqc + q] = cov[k];
        } else if (q < a.qcov && pos[k] >= 0 && cov[k]) {
          a.gdE[(size_t)pos[k] * Pp + q] -= a.gFb[(size_t)item.x * Pqc + q];
        }
      }
    }
    __syncwarp();
  }
}

template <typename T>
__global__ void adj_quirk_combine_kernel(const T* __restrict__ pval, const int* __restrict__ ppos,
                                         const int* __restrict__ hbase, const int* __restrict__ hcount,
                                         const int* __restrict__ hvert, int nheavy, int Pp, int Pqc,
                                         int qcov, const T* __restrict__ gb, T* __restrict__ gdE) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= nheavy) return;
  for (int q = lane; q < qcov; q += 32) {
    T b = neg_inf<T>();
    int bi = -1, bc = 0;
    for (int c = 0; c < hcount[warp]; ++c) {
      const size_t r = (size_t)(hbase[warp] + c);
      const int pp = ppos[r * 2 * Pqc + q];
      if (pp >= 0 && (bi < 0 || pval[r * Pqc + q] > b)) {
        b = pval[r * Pqc + q];
        bi = pp;
        bc = ppos[r * 2 * Pqc + Pqc + q];
      }
    }
    if (bi >= 0 && bc) gdE[(size_t)bi * Pp + q] -= gb[(size_t)hvert[warp] * Pqc + q];
  }
}

// ------------------------------------------- source side: dEmin, B, quirk
// Per out-edge element: the B softmax term into gdE; the first minimal edge of
// each (vertex, column), which receives gdEmin; the first maximal quirk
// element (columns < qcov), which receives gRb when covered.  Ties are broken
// by source-CSR position (increasing original edge id).
template <typename T>
struct SrcBackArgs {
  const int4* items;
  const int* wsplit;
  const int* row_of;
  const int* eid;
  const T* dE;
  const T* B;
  const T* gB;
  const T* gdEmin;
  const T* gRb;        // [Dn][Pqc]
  const long long* qlim_col;
  T* gdE;
  T* pval;             // [npartial][2 Pp]: min value | quirk max value
  int* ppos;           // [npartial][3 Pp]: min position | quirk position | covered
  int Pp, Pe, Pqc, qcov;
  int nranges;         // item ranges; warp w does ranges w, w + warps, ...
};

template <typename T, int NPOW, int NQV>
__global__ void __launch_bounds__(kT) adj_src_back_kernel(const SrcBackArgs<T> a) {
  constexpr int W = AV<T>::W, S = 32 / NPOW, NQ = NQV * W;
  const int Pp = a.Pp, Pqc = a.Pqc, lane = threadIdx.x & 31, slot = lane / NPOW, qc = lane % NPOW;
  const int gw = (blockIdx.x * kT + threadIdx.x) >> 5;
  long long qlim[NQ];
#pragma unroll
  for (int k = 0; k < NQ; ++k) {
    const int q = (qc + NPOW * (k / W)) * W + k % W;
    qlim[k] = q < a.qcov ? a.qlim_col[q] : 0;
  }
  const int nw = (int)gridDim.x * (kT / 32);
  for (int r = gw; r < a.nranges; r += nw)
  for (int it = a.wsplit[r]; it < a.wsplit[r + 1]; ++it) {
    const int4 item = a.items[it];
    const size_t vrow = (size_t)item.x * Pp;
    T mn[NQ], bq[NQ], Bv[NQ], gBv[NQ];
    int mp[NQ], bp[NQ], bc[NQ];
#pragma unroll
    for (int k = 0; k < NQ; ++k) {
      const int q = (qc + NPOW * (k / W)) * W + k % W;
      mn[k] = pos_inf<T>();
      bq[k] = neg_inf<T>();
      mp[k] = bp[k] = -1;
      bc[k] = 0;
      Bv[k] = q < Pp ? a.B[vrow + q] : T(0);
      gBv[k] = q < Pp ? a.gB[vrow + q] : T(0);
    }
    for (int j = item.y + slot; j < item.z; j += S) {
      const int e = __ldg(a.row_of + j);
      const long long id = __ldg(a.eid + j);
#pragma unroll
      for (int k = 0; k < NQ; ++k) {
        const int q = (qc + NPOW * (k / W)) * W + k % W;
        if (q >= Pp) continue;
        const size_t i = (size_t)e * Pp + q;
        const T d = a.dE[i];
        if (q < a.Pe) a.gdE[i] -= gBv[k] * ex(-d - Bv[k]);
        if (mp[k] < 0 || d < mn[k]) {
          mn[k] = d;
          mp[k] = j;
        }
        if (q < a.qcov) {
          const bool c = id < qlim[k];
          const T buf = c ? -d : T(0);
          if (bp[k] < 0 || buf > bq[k]) {
            bq[k] = buf;
            bp[k] = j;
            bc[k] = c;
          }
        }
      }
    }
#pragma unroll
    for (int o = NPOW; o < 32; o <<= 1)
#pragma unroll
      for (int k = 0; k < NQ; ++k) {
        const T om = __shfl_xor_sync(0xffffffffu, mn[k], o);
        const int omp = __shfl_xor_sync(0xffffffffu, mp[k], o);
        if (omp >= 0 && (mp[k] < 0 || om < mn[k] || (om == mn[k] && omp < mp[k]))) {
          mn[k] = om;
          mp[k] = omp;
        }
        const T ob = __shfl_xor_sync(0xffffffffu, bq[k], o);
        const int obp = __shfl_xor_sync(0xffffffffu, bp[k], o);
        const int obc = __shfl_xor_sync(0xffffffffu, bc[k], o);
        if (obp >= 0 && (bp[k] < 0 || ob > bq[k] || (ob == bq[k] && obp < bp[k]))) {
          bq[k] = ob;
          bp[k] = obp;
          bc[k] = obc;
        }
      }
    __syncwarp();  // this item's elementwise updates are visible to the routing below
    if (slot == 0) {
#pragma unroll
      for (int k = 0; k < NQ; ++k) {
        const int q = (qc + NPOW * (k / W)) * W + k % W;
        if (q >= Pp) continue;
        if (item.w >= 0) {
          const size_t r = (size_t)item.w;
          a.pval[r * 2 * Pp + q] = mn[k];
          a.pval[r * 2 * Pp + Pp + q] = bq[k];
          a.ppos[r * 3 * Pp + q] = mp[k];
          a.ppos[r * 3 * Pp + Pp + q] = bp[k];
          a.ppos[r * 3 * Pp + 2 * Pp + q] = bc[k];
        } else {
          if (mp[k] >= 0) a.gdE[(size_t)__ldg(a.row_of + mp[k]) * Pp + q] += a.gdEmin[vrow + q];
          if (q < a.qcov && bp[k] >= 0 && bc[k])
            a.gdE[(size_t)__ldg(a.row_of + bp[k]) * Pp + q] -= a.gRb[(size_t)item.x * Pqc + q];
        }
      }
    }
    __syncwarp();
  }
}

template <typename T>
__global__ void adj_src_combine_kernel(const T* __restrict__ pval, const int* __restrict__ ppos,
                                       const int* __restrict__ hbase, const int* __restrict__ hcount,
                                       const int* __restrict__ hvert, int nheavy, int Pp, int Pqc,
                                       int qcov, const int* __restrict__ row_of,
                                       const T* __restrict__ gdEmin, const T* __restrict__ gRb,
                                       T* __restrict__ gdE) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= nheavy) return;
  const size_t v = (size_t)hvert[warp];
  for (int q = lane; q < Pp; q += 32) {
    T m = pos_inf<T>(), b = neg_inf<T>();
    int mpos = -1, bpos = -1, bcov = 0;
    for (int c = 0; c < hcount[warp]; ++c) {
      const size_t r = (size_t)(hbase[warp] + c);
      const int mp = ppos[r * 3 * Pp + q], bp = ppos[r * 3 * Pp + Pp + q];
      if (mp >= 0 && (mpos < 0 || pval[r * 2 * Pp + q] < m)) {
        m = pval[r * 2 * Pp + q];
        mpos = mp;
      }
      if (bp >= 0 && (bpos < 0 || pval[r * 2 * Pp + Pp + q] > b)) {
        b = pval[r * 2 * Pp + Pp + q];
        bpos = bp;
        bcov = ppos[r * 3 * Pp + 2 * Pp + q];
      }
    }
    if (mpos >= 0) gdE[(size_t)row_of[mpos] * Pp + q] += gdEmin[v * Pp + q];
    if (q < qcov && bpos >= 0 && bcov) gdE[(size_t)row_of[bpos] * Pp + q] -= gRb[v * Pqc + q];
  }
}

// ---------------------------------------------------- vertex cost matrix
// gdV = -gMU0 + exp(MU0) colsum(gMU0) + gCV - exp(CV) colsum(gCV), written in
// place of gMU0 (MU0 = -dV - LSE(-dV) and CV = dV - LSE(dV), per column).
template <typename T>
__global__ void adj_dv_kernel(T* __restrict__ gMU0, const T* __restrict__ gCV, const T* __restrict__ mh,
                              const T* __restrict__ ml, const T* __restrict__ CV, const T* __restrict__ CVlo,
                              const double* __restrict__ cs, long long n, int Pn, int Pnp) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const long long v = i / Pn;
  const int p = (int)(i - v * Pn);
  const T cv = CV[(size_t)v * Pnp + p] + (CVlo ? CVlo[(size_t)v * Pnp + p] : T(0));
  const double g = -(double)gMU0[i] + (double)ex(mh[i] + ml[i]) * cs[p] + (double)gCV[i] -
                   (double)ex(cv) * cs[Pn + p];
  gMU0[i] = (T)g;
}

// ------------------------------------------------------------------ cdist
// One thread per row r of d = ||x_row(r) - y_q||: recomputes d in the forward's
// arithmetic, writes rr = g / d in place of g (0 where d = 0) and the row's
// feature gradient sum_q rr (x - y_q) to out[orow(r)] (FP64).
template <typename T, typename F, int KM>
__global__ void __launch_bounds__(kT)
adj_cdist_rows_kernel(const F* __restrict__ x, const int* __restrict__ row, int kstride, int K,
                      const double* __restrict__ y, int P, T* __restrict__ g, int ldg, long long nrows,
                      const int* __restrict__ orow, double* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char sm[];
  T* s_y = reinterpret_cast<T*>(sm);  // [P][KM]
  for (int t = threadIdx.x; t < P * KM; t += kT) {
    const int q = t / KM, k = t % KM;
    s_y[t] = k < K ? (T)y[(size_t)q * K + k] : T(0);
  }
  __syncthreads();
  for (long long r = (long long)blockIdx.x * kT + threadIdx.x; r < nrows; r += (long long)gridDim.x * kT) {
    const long long src = row ? (long long)row[r] : r;
    T xr[KM], gx[KM];
#pragma unroll
    for (int k = 0; k < KM; ++k) {
      xr[k] = k < K ? (T)x[(size_t)src * kstride + k] : T(0);
      gx[k] = T(0);
    }
    T* gr = g + (size_t)r * ldg;
    for (int q = 0; q < P; ++q) {
      T acc = T(0);
#pragma unroll
      for (int k = 0; k < KM; ++k) {
        const T t = xr[k] - s_y[q * KM + k];
        acc = fma(t, t, acc);
      }
      const T d = sqrt(acc);
      const T rr = d > T(0) ? gr[q] / d : T(0);
      gr[q] = rr;
#pragma unroll
      for (int k = 0; k < KM; ++k) gx[k] += rr * (xr[k] - s_y[q * KM + k]);
    }
    const size_t o = (size_t)(orow ? orow[r] : r) * K;
    for (int k = 0; k < K; ++k) out[o + k] = (double)gx[k];
  }
}

// Pattern side: part[block][q][k] = sum over the block's rows of rr[r][q] *
// x[r][k] (k < K) and rr[r][q] (k = K).  The block's rows are staged through
// shared memory kPR at a time (coalesced loads); each thread owns up to kPO
// outputs, summed per tile in T and across tiles in FP64, in row order.
constexpr int kPR = 32;
constexpr int kPO = 9;  // ceil(64 * 33 / 256): P <= 64, K <= 32
template <typename T, typename F>
__global__ void __launch_bounds__(256)
adj_cdist_pat_kernel(const F* __restrict__ x, const int* __restrict__ row, int kstride, int K,
                     const T* __restrict__ rr, int ldg, int P, long long nrows, double* __restrict__ part) {
  extern __shared__ __align__(16) unsigned char sm[];
  const int K1 = K + 1, nout = P * K1;
  T* s_r = reinterpret_cast<T*>(sm);  // [kPR][P]
  T* s_x = s_r + kPR * P;             // [kPR][K + 1], column K = 1
  const long long r0 = nrows * blockIdx.x / gridDim.x, r1 = nrows * (blockIdx.x + 1) / gridDim.x;
  double acc[kPO];
#pragma unroll
  for (int j = 0; j < kPO; ++j) acc[j] = 0;
  for (long long t0 = r0; t0 < r1; t0 += kPR) {
    const int nr = (int)min((long long)kPR, r1 - t0);
    __syncthreads();  // the previous tile is consumed
    for (int i = threadIdx.x; i < kPR * P; i += 256) {
      const int r = i / P, q = i - r * P;
      s_r[i] = r < nr ? rr[(size_t)(t0 + r) * ldg + q] : T(0);
    }
    for (int i = threadIdx.x; i < kPR * K1; i += 256) {
      const int r = i / K1, k = i - r * K1;
      T v = T(0);
      if (r < nr) {
        const long long src = row ? (long long)row[t0 + r] : t0 + r;
        v = k < K ? (T)x[(size_t)src * kstride + k] : T(1);
      }
      s_x[i] = v;
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kPO; ++j) {
      const int o = threadIdx.x + 256 * j;
      if (o < nout) {
        const int q = o / K1, k = o - q * K1;
        T sum = T(0);
#pragma unroll 8
        for (int r = 0; r < kPR; ++r) sum = fma(s_r[r * P + q], s_x[r * K1 + k], sum);
        acc[j] += (double)sum;
      }
    }
  }
#pragma unroll
  for (int j = 0; j < kPO; ++j) {
    const int o = threadIdx.x + 256 * j;
    if (o < nout) part[(size_t)blockIdx.x * nout + o] = acc[j];
  }
}

// gy[q][k] = -sum_r rr x_k + y[q][k] sum_r rr: one warp per output, the
// blocks' partials in a fixed lane-strided order and shuffle tree.
__global__ void adj_cdist_pat_final_kernel(const double* __restrict__ part, int nblk, int P, int K,
                                           const double* __restrict__ y, double* __restrict__ gy) {
  const int o = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
  if (o >= P * K) return;
  const int q = o / K, k = o % K, nout = P * (K + 1);
  double sx = 0, s1 = 0;
  for (int b = lane; b < nblk; b += 32) {
    sx += part[(size_t)b * nout + q * (K + 1) + k];
    s1 += part[(size_t)b * nout + q * (K + 1) + K];
  }
#pragma unroll
  for (int w = 16; w > 0; w >>= 1) {
    sx += __shfl_down_sync(0xffffffffu, sx, w);
    s1 += __shfl_down_sync(0xffffffffu, s1, w);
  }
  if (lane == 0) gy[o] = -sx + y[o] * s1;
}

#define ADJ_SHAPES(X) X(1, 1) X(2, 1) X(4, 1) X(8, 1) X(16, 1) X(32, 1) X(32, 2) X(32, 4)

template <typename F>
bool adj_warp_form(int pn, int pp, F&& f) {
  if (pp > 64 || pn > 64) return false;
  if (pp <= 32 && pn <= 32) f.template operator()<1, 1>();
  else if (pp <= 32) f.template operator()<1, 2>();
  else if (pn <= 32) f.template operator()<2, 1>();
  else f.template operator()<2, 2>();
  return true;
}

// ------------------------------------------------------------- C-null term
// (option cnull) Every iteration subtracts cnull[q] from both fills of column
// q, so the term's gradient is minus the gradients into the two fills, summed
// over the iterations (W->cols after each step A: into fR at [0, Pe), into fF
// at [Pe, 2 Pe)).
__global__ void adj_cnull_acc_kernel(const double* __restrict__ cols, int Pe, double* __restrict__ gcn) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < Pe) gcn[q] -= cols[q] + cols[Pe + q];
}

// cnull[q] = cn[q] - LSE_q cn[q] with cn[q] = max(||pe_q||, max_e L(dE)[q][e]).
// The second term is a log-softmax, never above 0 <= ||pe_q||, so cn[q] is the
// norm (a tie at 0 sends the gradient to the norm too): the gradient reaches
// the pattern edge features only,
//   gpe[q] += (gcn[q] - w_q sum_q' gcn[q']) pe_q / ||pe_q||,  w_q = exp(cnull[q]),
// added to what the cost matrix's adjoint wrote (none at ||pe_q|| = 0).  One
// block; the sum in column order.
__global__ void adj_cnull_pe_kernel(const double* __restrict__ gcn, const double* __restrict__ cnull,
                                    const double* __restrict__ pe, int Pe, int Ke,
                                    double* __restrict__ gpe) {
  __shared__ double s_tot;
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < Pe; ++q) t += gcn[q];
    s_tot = t;
  }
  __syncthreads();
  for (int q = threadIdx.x; q < Pe; q += blockDim.x) {
    double nn = 0.0;
    for (int k = 0; k < Ke; ++k) nn += pe[(size_t)q * Ke + k] * pe[(size_t)q * Ke + k];
    const double norm = sqrt(nn);
    if (!(norm > 0.0)) continue;
    const double c = (gcn[q] - exp(cnull[q]) * s_tot) / norm;
    for (int k = 0; k < Ke; ++k) gpe[(size_t)q * Ke + k] += c * pe[(size_t)q * Ke + k];
  }
}

// ------------------------------------------------------------- host side
template <typename T>
struct Adj {
  acg_plan* P;
  acg_data* D;
  AdjWork* W;
  cudaStream_t s;
  int Dn, De, Pn, Pe, Pp, Pnp, Pqc, nsm, vblocks;

  size_t vrow() const { return (size_t)Dn * Pp; }
  size_t prow() const { return (size_t)Dn * Pn; }

  acg_status fill(void* p, size_t n, T v) {
    if (n == 0) return ACG_OK;
    fill_t_kernel<T><<<(unsigned)std::min<size_t>((n + 255) / 256, 4096), 256, 0, s>>>((T*)p, n, v);
    ACG_LAUNCH_CHECK();
    return ACG_OK;
  }

  acg_status col_final(int nsum, int narg, int nblk) {
    const int n = nsum + narg;
    if (n == 0) return ACG_OK;
    col_final_kernel<<<ceil_div(32LL * n, 256), 256, 0, s>>>(W->part, nsum, W->part + (size_t)nsum * nblk, W->parti,
                                                        narg, nblk, W->cols, W->colsi);
    ACG_LAUNCH_CHECK();
    return ACG_OK;
  }

  // column sums of x [rows][ld] (ncol columns) into W->cols[off..]
  template <typename S>
  acg_status col_sums(const S* x, int ld, int ncol, long long rows, int off) {
    const int nb = std::max(1, std::min(nsm * 2, (int)std::min<long long>(rows, 1 << 20)));
    col_sum_kernel<S><<<nb, 128, 0, s>>>(x, ld, ncol, rows, W->part);
    ACG_LAUNCH_CHECK();
    col_final_kernel<<<ceil_div(32LL * ncol, 256), 256, 0, s>>>(W->part, ncol, nullptr, nullptr, 0, nb, W->cols + off,
                                                          nullptr);
    ACG_LAUNCH_CHECK();
    return ACG_OK;
  }

  // state pointers of state t (a checkpoint or a segment slot)
  void state(int t, int t0, const T** f, const T** r, const T** mh, const T** ml, const double** g) {
    if (W->ck.has(t)) {
      *f = (const T*)W->ck.f[t];
      *r = (const T*)W->ck.r[t];
      *mh = (const T*)W->ck.mh[t];
      *ml = (const T*)W->ck.ml[t];
      *g = W->ck.glob[t];
    } else {
      const int i = t - t0 - 1;
      *f = (const T*)W->sf[i];
      *r = (const T*)W->sr[i];
      *mh = (const T*)W->smh[i];
      *ml = (const T*)W->sml[i];
      *g = W->sglob[i];
    }
  }

  acg_status scatter() {
    ScatArgs<T> a{P->sw.items, P->sw.wsplit, D->pos_in_dst, D->scsr.other, W->emask, (const T*)W->gM,
                  (T*)W->gVRe, (T*)W->pscat, Pp, Pe, P->sw.nparts, P->range_ctr};
    ACG_TRY(fill(W->gVRe, vrow(), T(0)));  // sources without out-edges
    bool done = false;
#define ADJ_SC(NP_, NQ_)                                                        \
    if (!done && P->ws.npow == NP_ && P->ws.nqv == NQ_) {                       \
      adj_scatter_kernel<T, NP_, NQ_><<<P->src_blocks, kT, 0, s>>>(a);          \
      done = true;                                                              \
    }
    ADJ_SHAPES(ADJ_SC)
#undef ADJ_SC
    ACG_LAUNCH_CHECK();
    if (P->sw.nheavy > 0) {
      adj_sum_combine_kernel<T><<<ceil_div(P->sw.nheavy, 8), 256, 0, s>>>(
          (const T*)W->pscat, P->sw.hbase, P->sw.hcount, P->sw.hvert, P->sw.nheavy, Pp, (T*)W->gVRe);
      ACG_LAUNCH_CHECK();
    }
    return ACG_OK;
  }

  // adjoint of iteration t (messages F(t), R(t) from state t - 1); on entry
  // W->gMU holds the gradient into MU(t), gFd/gRd the direct ones (unless
  // first); on exit gMU holds the gradient into MU(t - 1) and gFd/gRd into
  // F(t - 1), R(t - 1).
  acg_status step(int t, int t0, bool first) {
    const T *f, *r, *mh, *ml;
    const double* g;
    state(t - 1, t0, &f, &r, &mh, &ml, &g);
    // the edge maxima of state t - 1 and their argmax, recorded by the edge
    // phase of iteration t (in the recorded forward or the segment recompute)
    const T* M;
    const int* A;
    if (W->ck.has_am(t - 1)) {
      M = (const T*)W->ck.m[t - 1];
      A = W->ck.a[t - 1];
    } else {
      M = (const T*)W->sm[t - 1 - t0];
      A = W->sa[t - 1 - t0];
    }
    if (De > 0) ACG_CUDA_TRY(cudaMemsetAsync(W->emask, 0, sizeof(unsigned long long) * (size_t)De, s));
    StepAArgs<T> sa{(const T*)W->gMU, first ? nullptr : (const T*)W->gFd,
                    first ? nullptr : (const T*)W->gRd, f, r, M, A, (T*)W->gdE, W->emask, (const T*)P->dEmin, g,
                    P->pat, (T*)W->gbR, (T*)W->gM, (T*)W->gdEmin, (T*)W->gCV, W->part,
                    W->part + (size_t)4 * Pe * vblocks, W->parti, Dn, Pn, Pe, Pp, P->cnull};
    const size_t smA = sizeof(T) * kW * 64 * 2 + sizeof(double) * kW * 6 * std::max(1, Pe) +
                       sizeof(int) * kW * 2 * std::max(1, Pe) + 64;
    cudaError_t le = cudaSuccess;
    adj_warp_form(Pn, Pp, [&]<int QPL, int PPL>() {
      if (smA > 48 * 1024)
        cudaFuncSetAttribute(adj_stepA_kernel<T, QPL, PPL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smA);
      adj_stepA_kernel<T, QPL, PPL><<<vblocks, kT, smA, s>>>(sa);
      le = cudaGetLastError();
    });
    if (le != cudaSuccess) return set_error(ACG_ERR_CUDA, "adj_stepA: %s", cudaGetErrorString(le));
    ACG_TRY(col_final(4 * Pe, 2 * Pe, vblocks));
    if (W->gcn && Pe > 0) {  // minus the gradients into both fills
      adj_cnull_acc_kernel<<<ceil_div(Pe, 128), 128, 0, s>>>(W->cols, Pe, W->gcn);
      ACG_LAUNCH_CHECK();
    }
    if (Pe > 0) ACG_TRY(scatter());
    else ACG_TRY(fill(W->gVRe, vrow(), T(0)));
    // state t - 1 = 0 has no S term (MU0 is normalised: S(0) is identically 0)
    StepBArgs<T> sb{(const T*)W->gbR, (const T*)W->gVRe, W->cols, W->colsi, f, r, (const T*)P->B, g,
                    t - 1 >= 1 ? mh : nullptr, t - 1 >= 1 ? ml : nullptr, P->pat, (T*)W->gB,
                    (T*)W->gMU2, (T*)W->gFd, (T*)W->gRd, Dn, Pn, Pe, Pp, std::max(1, P->maxdeg)};
    const size_t smB = ((sizeof(int) * 2 * std::max(1, P->maxdeg) * 32 + 15) & ~size_t(15)) +
                       sizeof(T) * kW * (2 * 32 * 2 + 4) + 64;
    adj_warp_form(Pn, Pp, [&]<int QPL, int PPL>() {
      if (smB > 48 * 1024)
        cudaFuncSetAttribute(adj_stepB_kernel<T, QPL, PPL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smB);
      adj_stepB_kernel<T, QPL, PPL><<<vblocks, kT, smB, s>>>(sb);
      le = cudaGetLastError();
    });
    if (le != cudaSuccess) return set_error(ACG_ERR_CUDA, "adj_stepB: %s", cudaGetErrorString(le));
    std::swap(W->gMU, W->gMU2);
    return ACG_OK;
  }

  acg_status restore(int t0) {
    restore_y_kernel<T><<<(unsigned)((vrow() + 255) / 256), 256, 0, s>>>(
        (const T*)W->ck.f[t0], (const T*)P->dEmin, (long long)vrow(), Pp, Pe, (T*)P->vf);
    ACG_LAUNCH_CHECK();
    ACG_CUDA_TRY(cudaMemcpyAsync(P->vr[t0 & 1], W->ck.r[t0], sizeof(T) * vrow(), cudaMemcpyDeviceToDevice, s));
    ACG_CUDA_TRY(cudaMemcpyAsync(P->gi[t0 & 1], W->ck.glob[t0], sizeof(double) * glob_doubles(Pn, Pe),
                                 cudaMemcpyDeviceToDevice, s));
    return ACG_OK;
  }

  acg_status backward(const double* gmu, double* gdnf, double* gdef, double* gpnf, double* gpef) {
    const int T_ = W->T;
    // zero the accumulators
    ACG_TRY(fill(W->gdEmin, vrow(), T(0)));
    ACG_TRY(fill(W->gB, vrow(), T(0)));
    ACG_TRY(fill(W->gCV, prow(), T(0)));
    ACG_TRY(fill(W->gdE, (size_t)De * Pp, T(0)));
    if (W->gcn) ACG_CUDA_TRY(cudaMemsetAsync(W->gcn, 0, sizeof(double) * std::max(1, Pe), s));
    // the gradient into MU(T): mu = MU(T) - S(T)
    ACG_TRY(col_sums(gmu, Pn, Pn, Dn, 0));
    {
      const long long n = (long long)prow();
      const T *f, *r, *mh, *ml;
      const double* g;
      state(T_, 0, &f, &r, &mh, &ml, &g);
      if (T_ > 0) {
        top_grad_kernel<T><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(gmu, mh, ml, g + 4 * Pe, W->cols, n, Pn,
                                                                       (T*)W->gMU);
        ACG_LAUNCH_CHECK();
      }
    }
    // segments from the last
    const StateRec* saved = P->rec;
    StateRec seg;
    bool first = true;
    for (int c = (int)W->ck_t.size() - 2; c >= 0 && T_ > 0; --c) {
      const int t0 = W->ck_t[c], t1 = W->ck_t[c + 1];
      if (t1 - t0 > 1) {  // recompute the states strictly between the checkpoints
        seg.resize(T_ + 1);
        seg.ppos = W->ppos;
        for (int t = t0 + 1; t < t1; ++t) {
          const int i = t - t0 - 1;
          seg.f[t] = W->sf[i];
          seg.r[t] = W->sr[i];
          seg.mh[t] = W->smh[i];
          seg.ml[t] = W->sml[i];
          seg.glob[t] = W->sglob[i];
          seg.m[t - 1] = W->sm[i];  // state t - 1 (t0 .. t1 - 2) from iteration t's edge phase
          seg.a[t - 1] = W->sa[i];
        }
        ACG_TRY(restore(t0));
        P->rec = &seg;
        acg_status st = ACG_OK;
        for (int t = t0 + 1; t < t1 && st == ACG_OK; ++t) st = run_iteration_any(P, t, nullptr, s);
        P->rec = saved;
        ACG_TRY(st);
      }
      for (int t = t1; t > t0; --t) {
        ACG_TRY(step(t, t0, first));
        first = false;
      }
    }
    // the gradient into MU0 is W->gMU; into F(0), R(0): gFd, gRd (zero when T = 0)
    if (T_ == 0) {
      // mu = MU0: copy gmu
      ACG_TRY(copy_gmu(gmu));
      ACG_TRY(fill(W->gFd, vrow(), T(0)));
      ACG_TRY(fill(W->gRd, vrow(), T(0)));
    }
    const T *f0, *r0, *mh0, *ml0;
    const double* g0;
    state(0, 0, &f0, &r0, &mh0, &ml0, &g0);
    // init messages
    {
      InitBArgs<T> a{D->dcsr.off, D->scsr.off, (const T*)W->gRd, (const T*)W->gFd, (const T*)P->Rq,
                     (const T*)P->Fq, mh0, ml0, P->gv, P->ge, P->qlim_col, P->pat, (T*)W->gRb,
                     (T*)W->gFb, W->part, W->part + (size_t)3 * Pe * vblocks, W->parti, (long long)De,
                     Dn, Pn, Pe, Pp, Pqc, P->qcov};
      const size_t smI = sizeof(double) * kW * (3 * std::max(1, Pe) + Pn) + sizeof(int) * kW * Pn + 64;
      cudaError_t le = cudaSuccess;
      adj_warp_form(Pn, Pp, [&]<int QPL, int PPL>() {
        if (smI > 48 * 1024)
          cudaFuncSetAttribute(adj_initB_kernel<T, QPL, PPL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smI);
        adj_initB_kernel<T, QPL, PPL><<<vblocks, kT, smI, s>>>(a);
        le = cudaGetLastError();
      });
      if (le != cudaSuccess) return set_error(ACG_ERR_CUDA, "adj_initB: %s", cudaGetErrorString(le));
      ACG_TRY(col_final(3 * Pe, Pn, vblocks));
      adj_init_fill_kernel<<<ceil_div(Pn, 64), 64, 0, s>>>(W->cols, W->colsi, P->pat, Pn, Pe,
                                                           sizeof(T) == 8 ? (double*)W->gMU : nullptr,
                                                           sizeof(T) == 4 ? (float*)W->gMU : nullptr);
      ACG_LAUNCH_CHECK();
    }
    // quirk rows over in-edges (covered columns), then the source side
    if (De > 0 && P->qcov > 0) {
      QuirkArgs<T> a{P->ew.items, P->ew.wsplit, D->dcsr.eid, (const T*)P->dE, (const T*)W->gFb, P->ge,
                     P->qlim_col, W->cols, (T*)W->gdE, (T*)W->pq, W->pqi, (long long)De, Pp, Pqc, P->qcov,
                     P->ew.nparts};
      bool done = false;
#define ADJ_Q(NP_, NQ_)                                                         \
      if (!done && P->qws.npow == NP_ && P->qws.nqv == NQ_) {                   \
        adj_quirk_dst_kernel<T, NP_, NQ_><<<P->edge_blocks, kT, 0, s>>>(a);     \
        done = true;                                                            \
      }
      ADJ_SHAPES(ADJ_Q)
#undef ADJ_Q
      ACG_LAUNCH_CHECK();
      if (P->ew.nheavy > 0) {
        adj_quirk_combine_kernel<T><<<ceil_div(P->ew.nheavy, 8), 256, 0, s>>>(
            (const T*)W->pq, W->pqi, P->ew.hbase, P->ew.hcount, P->ew.hvert, P->ew.nheavy, Pp, Pqc,
            P->qcov, (const T*)W->gFb, (T*)W->gdE);
        ACG_LAUNCH_CHECK();
      }
    }
    if (De > 0 && Pe > 0) {
      SrcBackArgs<T> a{P->sw.items, P->sw.wsplit, D->pos_in_dst, D->scsr.eid, (const T*)P->dE,
                       (const T*)P->B, (const T*)W->gB, (const T*)W->gdEmin, (const T*)W->gRb,
                       P->qlim_col, (T*)W->gdE, (T*)W->pstat, W->pstati, Pp, Pe, Pqc, P->qcov,
                       P->sw.nparts};
      bool done = false;
#define ADJ_S(NP_, NQ_)                                                         \
      if (!done && P->ws.npow == NP_ && P->ws.nqv == NQ_) {                     \
        adj_src_back_kernel<T, NP_, NQ_><<<P->src_blocks, kT, 0, s>>>(a);       \
        done = true;                                                            \
      }
      ADJ_SHAPES(ADJ_S)
#undef ADJ_S
      ACG_LAUNCH_CHECK();
      if (P->sw.nheavy > 0) {
        adj_src_combine_kernel<T><<<ceil_div(P->sw.nheavy, 8), 256, 0, s>>>(
            (const T*)W->pstat, W->pstati, P->sw.hbase, P->sw.hcount, P->sw.hvert, P->sw.nheavy, Pp, Pqc,
            P->qcov, D->pos_in_dst, (const T*)W->gdEmin, (const T*)W->gRb, (T*)W->gdE);
        ACG_LAUNCH_CHECK();
      }
    }
    // vertex cost: gdV in place of gMU0
    ACG_TRY(col_sums((const T*)W->gMU, Pn, Pn, Dn, 0));
    ACG_TRY(col_sums((const T*)W->gCV, Pn, Pn, Dn, Pn));
    {
      const long long n = (long long)prow();
      adj_dv_kernel<T><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(
          (T*)W->gMU, (const T*)W->gCV, mh0, ml0, (const T*)P->CV, (const T*)P->CVlo, W->cols, n, Pn, P->Pnp);
      ACG_LAUNCH_CHECK();
    }
    // cdist: data-side rows, then the pattern side
    ACG_TRY(cdist_back(true, gdnf, gpnf));
    if (De > 0 && Pe > 0) ACG_TRY(cdist_back(false, gdef, gpef));
    else if (Pe > 0)
      ACG_CUDA_TRY(cudaMemsetAsync(gpef, 0, sizeof(double) * Pe * D->Ke, s));
    if (W->gcn && Pe > 0) {  // the C-null term, a function of the pattern edge features
      adj_cnull_pe_kernel<<<1, 256, 0, s>>>(W->gcn, P->cnull, P->pe, Pe, D->Ke, gpef);
      ACG_LAUNCH_CHECK();
    }
    return ACG_OK;
  }

  acg_status copy_gmu(const double* gmu) {
    const long long n = (long long)prow();
    copy_cast_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(gmu, (T*)W->gMU, n);
    ACG_LAUNCH_CHECK();
    return ACG_OK;
  }


  // vertex == true: dV (rows = data vertices, columns = pattern vertices,
  // gradient W->gMU); else dE (rows in destination-CSR order, W->gdE).
  acg_status cdist_back(bool vertex, double* gx, double* gy) {
    const int K = vertex ? D->Kv : D->Ke, P_ = vertex ? Pn : Pe, ld = vertex ? Pn : Pp;
    const long long nrows = vertex ? Dn : De;
    T* g = (T*)(vertex ? W->gMU : W->gdE);
    const double* y = vertex ? P->pv : P->pe;
    if (K == 0 || nrows == 0 || P_ == 0) return ACG_OK;
    const int km = (K + 3) / 4 * 4;
    const size_t sm = sizeof(T) * (size_t)P_ * km;
    const int blocks = std::max(1, std::min(ceil_div(std::max<long long>(1, nrows), kT), nsm * 8));
    // data features: the FP32 copies (mixed; edges in destination-CSR order) or
    // the caller's FP64 arrays (edges gathered by original id)
    const bool f32 = sizeof(T) == 4;
    const int* row = vertex ? nullptr : (f32 ? nullptr : D->dcsr.eid);
    const int* orow = vertex ? nullptr : D->dcsr.eid;
    const int kstride = f32 ? (vertex ? D->kv32 : D->ke32) : K;
    cudaError_t le = cudaSuccess;
    auto launch = [&](auto kmc) {
      constexpr int KM = decltype(kmc)::value;
      if constexpr (sizeof(T) == 4) {
        const float* x = vertex ? D->nf32 : D->ef32;
        adj_cdist_rows_kernel<T, float, KM><<<blocks, kT, sm, s>>>(x, row, kstride, K, y, P_, g, ld, nrows, orow, gx);
      } else {
        const double* x = vertex ? D->node_feats : D->edge_feats;
        adj_cdist_rows_kernel<T, double, KM><<<blocks, kT, sm, s>>>(x, row, kstride, K, y, P_, g, ld, nrows, orow, gx);
      }
      le = cudaGetLastError();
    };
    switch (km) {
      case 4: launch(std::integral_constant<int, 4>{}); break;
      case 8: launch(std::integral_constant<int, 8>{}); break;
      case 12: launch(std::integral_constant<int, 12>{}); break;
      case 16: launch(std::integral_constant<int, 16>{}); break;
      case 20: launch(std::integral_constant<int, 20>{}); break;
      case 24: launch(std::integral_constant<int, 24>{}); break;
      case 28: launch(std::integral_constant<int, 28>{}); break;
      case 32: launch(std::integral_constant<int, 32>{}); break;
      default: return set_error(ACG_ERR_UNSUPPORTED, "acg_backward: feature dimension %d above 32", K);
    }
    if (le != cudaSuccess) return set_error(ACG_ERR_CUDA, "adj_cdist_rows: %s", cudaGetErrorString(le));
    // pattern side
    const int pb = std::max(1, std::min(nsm * 4, ceil_div(nrows, 4 * kPR)));
    const size_t psm = sizeof(T) * (size_t)kPR * (P_ + K + 1);
    if constexpr (sizeof(T) == 4) {
      const float* x = vertex ? D->nf32 : D->ef32;
      adj_cdist_pat_kernel<T, float><<<pb, 256, psm, s>>>(x, nullptr, kstride, K, g, ld, P_, nrows, W->ypart);
    } else {
      const double* x = vertex ? D->node_feats : D->edge_feats;
      adj_cdist_pat_kernel<T, double><<<pb, 256, psm, s>>>(x, row, kstride, K, g, ld, P_, nrows, W->ypart);
    }
    ACG_LAUNCH_CHECK();
    adj_cdist_pat_final_kernel<<<ceil_div(32LL * P_ * K, 256), 256, 0, s>>>(W->ypart, pb, P_, K, y, gy);
    ACG_LAUNCH_CHECK();
    return ACG_OK;
  }
};

}  // namespace

// ------------------------------------------------------------ entry points
namespace {

acg_status adj_buf(AdjWork* W, size_t bytes, void** out, cudaStream_t s) {
  return dev_alloc(&W->owned, std::max<size_t>(bytes, 16), out, s);
}

acg_status adj_check(acg_plan* P, const char* who) {
  if (!P) return set_error(ACG_ERR_INVALID_ARGUMENT, "%s: plan is null", who);
  if (P->is_union) return set_error(ACG_ERR_UNSUPPORTED, "%s: a batch group has no adjoint", who);
  if (P->Pp > 64 || P->Pn > 64 || !P->init_warp)
    return set_error(ACG_ERR_UNSUPPORTED,
                     "%s: the adjoint is built for patterns of at most 64 vertices and 64 padded edge columns",
                     who);
  if (P->data->Kv > 32 || P->data->Ke > 32)
    return set_error(ACG_ERR_UNSUPPORTED, "%s: feature dimension above 32", who);
  if (P->data->Dn == 0) return set_error(ACG_ERR_INVALID_ARGUMENT, "%s: empty data graph", who);
  return ACG_OK;
}

// Checkpoints (states 0, k, 2k, ..., T), the segment slots between them and
// the work buffers; kept across calls while (k, T) stays the same.
acg_status adj_alloc(acg_plan* P, int every, cudaStream_t s) {
  acg_data* D = P->data;
  const int T_ = P->iters;
  if (P->adj && P->adj->every == every && P->adj->T == T_) return ACG_OK;
  adj_free(P);
  P->adj = new AdjWork();
  AdjWork* W = P->adj;
  W->every = every;
  W->T = T_;
  for (int t = 0; t < T_; t += every) W->ck_t.push_back(t);
  W->ck_t.push_back(T_);
  int gap = 1;
  for (size_t i = 0; i + 1 < W->ck_t.size(); ++i) gap = std::max(gap, W->ck_t[i + 1] - W->ck_t[i]);
  const size_t eb = P->prec == ACG_PREC_FP64 ? 8 : 4;
  const size_t Dn = D->Dn, De = D->De, Pn = P->Pn, Pe = P->Pe, Pp = P->Pp;
  const size_t Pqc = std::max(1, P->Pqc);
  const size_t vrow = Dn * Pp * eb, prow = Dn * Pn * eb, gb = sizeof(double) * glob_doubles(P->Pn, P->Pe);
  W->ck.resize(T_ + 1);
  W->ck.ppos = nullptr;  // set below (W->ppos)
  for (int t : W->ck_t) {
    if (t >= 1) {  // the edge maxima of state t - 1, from iteration t of the recorded match
      ACG_TRY(adj_buf(W, vrow, &W->ck.m[t - 1], s));
      ACG_TRY(adj_buf(W, Dn * Pp * sizeof(int), (void**)&W->ck.a[t - 1], s));
    }
    if (t < T_ || t == 0) {  // the last state needs only MU_raw and its statistics
      ACG_TRY(adj_buf(W, vrow, &W->ck.f[t], s));
      ACG_TRY(adj_buf(W, vrow, &W->ck.r[t], s));
    }
    ACG_TRY(adj_buf(W, prow, &W->ck.mh[t], s));
    ACG_TRY(adj_buf(W, prow, &W->ck.ml[t], s));
    ACG_TRY(adj_buf(W, gb, (void**)&W->ck.glob[t], s));
  }
  const int nslot = gap - 1;
  W->sf.assign(nslot, nullptr);
  W->sr.assign(nslot, nullptr);
  W->smh.assign(nslot, nullptr);
  W->sml.assign(nslot, nullptr);
  W->sglob.assign(nslot, nullptr);
  W->sm.assign(nslot, nullptr);
  W->sa.assign(nslot, nullptr);
  for (int i = 0; i < nslot; ++i) {
    ACG_TRY(adj_buf(W, vrow, &W->sm[i], s));
    ACG_TRY(adj_buf(W, Dn * Pp * sizeof(int), (void**)&W->sa[i], s));
    ACG_TRY(adj_buf(W, vrow, &W->sf[i], s));
    ACG_TRY(adj_buf(W, vrow, &W->sr[i], s));
    ACG_TRY(adj_buf(W, prow, &W->smh[i], s));
    ACG_TRY(adj_buf(W, prow, &W->sml[i], s));
    ACG_TRY(adj_buf(W, gb, (void**)&W->sglob[i], s));
  }
  const int nsm = D->num_sms;
  W->vblocks = nsm * 2;
  const size_t vb = W->vblocks;
  for (void** b : {&W->gMU, &W->gMU2, &W->gCV}) ACG_TRY(adj_buf(W, prow, b, s));
  for (void** b : {&W->gFd, &W->gRd, &W->gbR, &W->gM, &W->gVRe, &W->gdEmin, &W->gB})
    ACG_TRY(adj_buf(W, vrow, b, s));
  ACG_TRY(adj_buf(W, De * sizeof(unsigned long long), (void**)&W->emask, s));
  ACG_TRY(adj_buf(W, De * Pp * eb, &W->gdE, s));
  ACG_TRY(adj_buf(W, Dn * Pqc * eb, &W->gRb, s));
  ACG_TRY(adj_buf(W, Dn * Pqc * eb, &W->gFb, s));
  const size_t enp = P->ew.npartial, snp = P->sw.npartial;
  ACG_TRY(adj_buf(W, enp * Pp * sizeof(int), (void**)&W->ppos, s));
  W->ck.ppos = W->ppos;
  ACG_TRY(adj_buf(W, snp * Pp * eb, &W->pscat, s));
  ACG_TRY(adj_buf(W, snp * 2 * Pp * eb, &W->pstat, s));
  ACG_TRY(adj_buf(W, snp * 3 * Pp * sizeof(int), (void**)&W->pstati, s));
  ACG_TRY(adj_buf(W, enp * Pqc * eb, &W->pq, s));
  ACG_TRY(adj_buf(W, enp * 2 * Pqc * sizeof(int), (void**)&W->pqi, s));
  const size_t npart = std::max({6 * Pe * vb, (3 * Pe + Pn) * vb, Pn * 2 * (size_t)nsm});
  ACG_TRY(adj_buf(W, sizeof(double) * npart, (void**)&W->part, s));
  ACG_TRY(adj_buf(W, sizeof(int) * std::max(2 * Pe, Pn) * vb, (void**)&W->parti, s));
  ACG_TRY(adj_buf(W, sizeof(double) * (8 * Pe + 2 * Pn + 8), (void**)&W->cols, s));
  ACG_TRY(adj_buf(W, sizeof(int) * (2 * Pe + Pn + 1), (void**)&W->colsi, s));
  const size_t ny = 4 * (size_t)nsm * std::max(Pn * (D->Kv + 1), Pe * (D->Ke + 1));
  ACG_TRY(adj_buf(W, sizeof(double) * ny, (void**)&W->ypart, s));
  if (P->cnull) ACG_TRY(adj_buf(W, sizeof(double) * std::max<size_t>(1, Pe), (void**)&W->gcn, s));
  return ACG_OK;
}

template <typename T>
acg_status run_backward(acg_plan* P, const double* gmu, double* gdn, double* gde, double* gpn,
                        double* gpe, cudaStream_t s) {
  Adj<T> A;
  A.P = P;
  A.D = P->data;
  A.W = P->adj;
  A.s = s;
  A.Dn = A.D->Dn;
  A.De = A.D->De;
  A.Pn = P->Pn;
  A.Pe = P->Pe;
  A.Pp = P->Pp;
  A.Pnp = P->Pnp;
  A.Pqc = P->Pqc;
  A.nsm = A.D->num_sms;
  A.vblocks = P->adj->vblocks;
  return A.backward(gmu, gdn, gde, gpn, gpe);
}

}  // namespace

extern "C" {

acg_status acg_match_record(acg_plan* P, double* mu_out, int32_t checkpoint_every, void* stream) {
  clear_error();
  ACG_TRY(adj_check(P, "acg_match_record"));
  if (!mu_out) return set_error(ACG_ERR_INVALID_ARGUMENT, "acg_match_record: mu_out is null");
  cudaStream_t s = (cudaStream_t)stream;
  const int every = checkpoint_every > 0 ? checkpoint_every : 4;
  ACG_TRY(adj_alloc(P, every, s));
  P->adj->recorded = false;
  P->adj->drop_graph();  // recorded afresh: the next backward is captured again
  P->last_stream = s;
  P->rec = &P->adj->ck;
  const acg_status st = run_match_any(P, mu_out, s, nullptr);
  P->rec = nullptr;
  P->ran = st == ACG_OK;
  P->adj->recorded = st == ACG_OK;
  return st;
}

acg_status acg_backward(acg_plan* P, const double* grad_mu, double* g_data_node, double* g_data_edge,
                        double* g_pat_node, double* g_pat_edge, void* stream) {
  clear_error();
  ACG_TRY(adj_check(P, "acg_backward"));
  if (!P->adj || !P->adj->recorded)
    return set_error(ACG_ERR_INVALID_ARGUMENT, "acg_backward: no acg_match_record has run on this plan");
  const acg_data* D = P->data;
  if (!grad_mu) return set_error(ACG_ERR_INVALID_ARGUMENT, "acg_backward: grad_mu is null");
  if ((!g_data_node && (long long)D->Dn * D->Kv > 0) || (!g_data_edge && (long long)D->De * D->Ke > 0) ||
      (!g_pat_node && (long long)P->Pn * D->Kv > 0) || (!g_pat_edge && (long long)P->Pe * D->Ke > 0))
    return set_error(ACG_ERR_INVALID_ARGUMENT, "acg_backward: a gradient output is null");
  cudaStream_t s = (cudaStream_t)stream;
  auto run = [&](cudaStream_t rs) {
    return P->prec == ACG_PREC_FP64
               ? run_backward<double>(P, grad_mu, g_data_node, g_data_edge, g_pat_node, g_pat_edge, rs)
               : run_backward<float>(P, grad_mu, g_data_node, g_data_edge, g_pat_node, g_pat_edge, rs);
  };
  // About 150 launches, each short at small sizes: replayed as one graph.  A
  // caller's stream that is itself being captured, and plans that time their
  // phases with events, get the launches directly.
  AdjWork* W = P->adj;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (W->gfailed || P->kernel_timing || cudaStreamIsCapturing(s, &cap) != cudaSuccess ||
      cap != cudaStreamCaptureStatusNone) {
    cudaGetLastError();
    return run(s);
  }
  const void* key[5] = {grad_mu, g_data_node, g_data_edge, g_pat_node, g_pat_edge};
  if (W->gexec && !std::equal(key, key + 5, W->gkey)) W->drop_graph();
  if (!W->gexec) {
    if (!W->gstream) ACG_CUDA_TRY(cudaStreamCreateWithFlags(&W->gstream, cudaStreamNonBlocking));
    ACG_CUDA_TRY(cudaStreamBeginCapture(W->gstream, cudaStreamCaptureModeThreadLocal));
    const acg_status st = run(W->gstream);
    cudaGraph_t g = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(W->gstream, &g);
    if (st != ACG_OK) {
      if (g) cudaGraphDestroy(g);
      return st;
    }
    if (ce != cudaSuccess || !g || cudaGraphInstantiate(&W->gexec, g, 0) != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      cudaGetLastError();
      W->gexec = nullptr;
      W->gfailed = true;
      return run(s);
    }
    cudaGraphDestroy(g);
    std::copy(key, key + 5, W->gkey);
  }
  ACG_CUDA_TRY(cudaGraphLaunch(W->gexec, s));
  return ACG_OK;
}

}  // extern "C"
