// acg_iter.cuh -- one BP iteration: edge phase + vertex phase (acg_iter.cu).
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "acg_internal.h"

namespace acg {

// Phase A work item = {vertex, first dst-CSR position, end position, partial
// row or -1}: a light vertex with all its in-edges (its maxima go to M), or one
// chunk of a heavy vertex (maxima go to the partial row).
template <typename T>
struct EdgeMaxArgs {
  const int4* items;
  int nitems;
  const int* wsplit;   // [nranges + 1]: range r is items [wsplit[r], wsplit[r+1])
  const int* src_of;   // [De] source vertex of each dst-CSR position
  const T* dE;         // [De][Pp]
  const T* vr_in;      // [Dn][Pp]
  T* M;                // [Dn][Pp] out: max over in-edges of VR' - dE
  T* partial;          // [npartial][Pp]
  int Pp;
  // Recording for the adjoint (null otherwise): the first maximal dst-CSR
  // position of each maximum ([Dn][Pp]; ppos: [npartial][Pp] for the chunks)
  int* argpos = nullptr;
  int* ppos = nullptr;
  // Item ranges: warp w first does range w; with `ctr` (two zeroed ints: the
  // next range past the warps' first ones, and the warps finished) further
  // ranges are claimed from the counter, and the last warp to finish resets
  // both.  Without it nranges must equal the launched warps.
  int nranges = 0;
  int* ctr = nullptr;
  // Heavy vertices combined in the kernel (FP32 without argmax, with hcnt,
  // [nheavy] zeroed counters): the warp that completes a heavy vertex's last
  // chunk takes the max of its partial rows into M and resets the counter.
  // Otherwise heavy_combine(_arg)_kernel does it after the launch.
  const int* pheavy = nullptr;  // [npartial] heavy index of each partial row
  const int* hbase = nullptr;
  const int* hcount = nullptr;
  const int* hvert = nullptr;
  int* hcnt = nullptr;
};

// Column statistics of one iteration (FP64), double-buffered across iterations:
//   [0,Pe) max_v VF'-cR | [Pe,2Pe) max_v VR'-cF | [2Pe,3Pe) dR = LSE_v(VF'-cR+B)
//   | [3Pe,4Pe) dF = LSE_v(VR'-cF+B) | [4Pe,4Pe+Pn) S = LSE_v MU_raw
//   | then from 4Pe+Pn: cR, cF (the shifts the stored Y, Z carry), and the
//   absolute lR, lF of the iteration before (the next shifts).
inline int glob_doubles(int pn, int pe) { return 8 * pe + pn; }

template <typename T>
struct VertexUpdArgs {
  const int* d_off;    // [Dn+1] (in-degree: empty rows of M are -inf)
  const T* M;          // [Dn][Pp] max over in-edges of Z[src] - dE
  T* vf;               // [Dn][Pp] Y = VF' - dEmin - cR: read then overwritten
  T* vr_out;           // [Dn][Pp] Z = VR' - cF
  const T* dEmin;      // [Dn][Pp]
  const T* B;          // [Dn][Pp]
  const T* CV;         // [Dn][Pnp]
  const T* CVlo;       // [Dn][Pnp] low parts (FP32 only, else null)
  const double* glob_in;
  double* glob_out;    // this iteration's shifts (block 0; the rest by stat_finalize)
  double* bpart;       // [slot][gridDim.x]
  double* mu_raw;      // [Dn][Pn] (last iteration)
  const int* pat;
  int Dn, Pn, Pe, Pp, Pnp;
  int maxdeg;          // max over pattern vertices of in- plus out-degree
  const int* iters_p;  // [Pn] iteration count of each pattern vertex's pattern:
                       // MU_raw is written at iteration t == iters_p[p]
  int t;               // this iteration (1-based)
  int first, last;     // first iteration; last iteration of every pattern
  // Recording for the adjoint (all null otherwise): the state this iteration
  // produces -- f = VF' - cR and r = VR' - cF ([Dn][Pp], zero past Pe; not on
  // the last iteration) and MU_raw as hi + lo ([Dn][Pn]).
  T* rec_f = nullptr;
  T* rec_r = nullptr;
  T* rec_mh = nullptr;
  T* rec_ml = nullptr;
  // C-null term ([Pe], subtracted from both fills of each column; null: none)
  const double* cnull = nullptr;
  // warp form (Pn <= 64, Pp <= 64): the per-lane schedule of the compensated
  // MU_raw sums of one stage, [vterms][32] (vertex_warp_schedule)
  const uint32_t* vsched = nullptr;
  int vterms = 0;
};
// The warp form's schedule for a pattern (pat: the incidence arrays of
// build_incidence): per lane, the terms of its (staged vertex, pattern vertex)
// sums in order.  Returns the terms per lane, 0 when the pattern takes the
// tile form.
int vertex_warp_schedule(const int* pat, int pn, int pe, int pp, int pnp, std::vector<uint32_t>* out);
// S_final[p] = S[p] of this iteration where it is p's last (S = the column
// log-sum-exp of MU_raw in the statistics just finalised).
acg_status launch_capture_s(const double* S, const int* iters_p, int t, double* S_final, int Pn,
                            cudaStream_t s);

// Edge phase of FP32 plans with the costs recomputed on the tensor cores
// (acg_edge_tc.cu): M[v][q] = max over in-edges e of z[s_e][q] - ||x_e - y_q||,
// d formed as the tensor-core edge cost matrix forms it.  One CTA per part of
// the item split (items of at most 128 positions; heavy vertices chunked).
struct EdgeTcArgs {
  const float* x;      // [De][KM] FP32 edge features in dst-CSR order (zero past K)
  const double* y;     // [P][K] pattern edge features
  const int* src_of;   // [De] source vertex of each dst-CSR position
  const float* z;      // [Dn][Pp] gathered by source
  float* M;            // [Dn][Pp] out (rows of vertices without in-edges untouched)
  const int4* items;   // {vertex, first position, end position, partial row or -1}
  const int* wsplit;   // [parts + 1]: CTA b does items [wsplit[b], wsplit[b+1])
  float* partial;      // [npartial][Pp] rows of heavy-vertex chunks
  const int* pheavy;   // [npartial] heavy vertex of each partial row
  const int* hbase;    // per heavy vertex: first partial row, chunk count, vertex
  const int* hcount;
  const int* hvert;
  int* hcnt;           // [nheavy] chunks done, zero before and after a launch
  int* err;            // set to 1 when a bounded wait gave up
  long long De;
  int K, KM, P, Pp;
  // set by launch_edge_tc
  int N = 0, tcols = 0;
};
bool edge_tc_eligible(int K, int kstride, int P, int Pp);
size_t edge_tc_smem(int kstride, int Pp);
constexpr int kEdgeTcChunk = 128;  // positions per chunk of a heavy vertex (one tile)
acg_status launch_edge_tc(const EdgeTcArgs& a, int parts, cudaStream_t s);

struct WarpShape {
  int npow;  // lanes covering one [Pp] row (power of two <= 32)
  int nqv;   // 16-byte vectors per lane per row
};
WarpShape choose_warp_shape(int elem_bytes, int pp);
// In-edges loaded per warp step by the edge phase.
int edge_step(WarpShape ws);

template <typename T>
acg_status launch_edge_max(const EdgeMaxArgs<T>& a, WarpShape ws, int blocks, cudaStream_t s);
template <typename T>
acg_status launch_heavy_combine(const T* partial, const int* hbase, const int* hcount,
                                const int* hvert, int nheavy, int Pp, T* M, cudaStream_t s);
// The same with the argmax positions of the chunks (earlier chunks win ties).
template <typename T>
acg_status launch_heavy_combine_arg(const T* partial, const int* ppos, const int* hbase,
                                    const int* hcount, const int* hvert, int nheavy, int Pp, T* M,
                                    int* A, cudaStream_t s);
template <typename T>
acg_status launch_vertex_update(const VertexUpdArgs<T>& a, int blocks, cudaStream_t s);
template <typename T>
int vertex_update_blocks_per_sm(int pn, int pe, int pp);
// Grid of the vertex phase: the warp form (Pp <= 64, Pn <= 64) runs one wave
// of resident blocks; the tile form one block per tile up to resident blocks.
template <typename T>
int vertex_update_blocks(int pn, int pe, int pp, int pnp, int nterms, int num_sms, int dn);
// Set every element of p[0, n) to v.
template <typename T>
acg_status launch_fill(T* p, size_t n, T v, cudaStream_t s);
// Resident blocks per SM of the edge kernel for this shape (the grid is one
// wave of them: the warp ranges are static, so every warp must be resident).
template <typename T>
int edge_max_blocks_per_sm(WarpShape ws);

}  // namespace acg
