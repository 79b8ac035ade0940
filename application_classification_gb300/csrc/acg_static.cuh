// acg_static.cuh -- the static per-vertex reductions of a match (acg_static.cu):
// what the reference computes once before its BP loop from the edge cost
// matrix (main.cu:110-146), restated as per-vertex quantities.
#pragma once

#include <cuda_runtime.h>

#include "acg_bp.cuh"
#include "acg_internal.h"
#include "acg_iter.cuh"

namespace acg {

// Quirk buffer of main.cu:113-114: element (q, e) holds -dE[q, e] if its flat
// index q * De + e is below lim = Pn * Dn, else 0: column q covers the original
// edge ids below qlim[q] = lim - q * De.  Only columns q < qcov = ceil(lim / De)
// hold any -dE; the later ones are all zero.  (A group of patterns matched as
// one disjoint union keeps each pattern's own Pn and local q in qlim, with the
// covered columns of all its patterns ordered first.)
inline int quirk_columns(long long lim, long long de, int pe) {
  if (de <= 0) return 0;
  const long long c = (lim + de - 1) / de;
  return (int)(c < pe ? c : pe);
}

// Source-side reductions over each vertex's out-edges, walked in the
// source-sorted CSR with the dE rows gathered from their destination-sorted
// position: dEmin = min dE, B = log sum exp(-dE), and the quirk-buffer maximum
// of the columns q < qcov.
template <typename T>
struct SrcStatsArgs {
  const int4* items;
  int nitems;
  const int* wsplit;
  const int* row_of;   // [De] dE row (destination order) of each source-order position
  const int* eid;      // [De] original edge id of each source-order position
  const T* dE;         // [De][Pp]
  T* dEmin;            // [Dn][Pp]
  T* B;                // [Dn][Pp]
  T* Rq;               // [Dn][Pqc] quirk maximum over out-edges (columns < qcov)
  T* partial;          // [npartial][3 Pp + Pqc]: min | lse max | lse sum | quirk
  const long long* qlim_col;  // [Pp] column q covers original edge ids < qlim_col[q]
  long long De, lim;
  int Pp, Pqc, qcov;
  // item ranges, as the edge phase's: warp w first does range w, then claims
  // ranges from ctr (two zeroed ints, reset by the last warp to finish)
  int nranges = 0;
  int* ctr = nullptr;
};
template <typename T>
acg_status launch_src_stats(const SrcStatsArgs<T>& a, WarpShape ws, int blocks, cudaStream_t s);
// Combine the partial rows of the vertices split into chunks, in chunk order.
template <typename T>
acg_status launch_src_stats_combine(const SrcStatsArgs<T>& a, const WarpWork& w, cudaStream_t s);

// Destination-side quirk maximum over each vertex's in-edges (consecutive rows
// of the destination-sorted dE), columns q < qcov only, and per column the
// log-sum-exp of -dE over its covered elements (block partials, StatSpec{0,
// Pqc}; every edge is an in-edge of exactly one item).
template <typename T>
struct DstQuirkArgs {
  const int4* items;
  int nitems;
  const int* wsplit;
  const int* eid;      // [De] original edge id of each destination-order position
  const T* dE;         // [De][dstride]: the cost rows, or their covered columns
  T* Fq;               // [Dn][Pqc]
  T* partial;          // [npartial][Pqc]
  double* bpart;       // [2 Pqc][blocks]
  const long long* qlim_col;  // [Pp] as for the source side
  long long De, lim;
  int Pp, Pqc, qcov;
  int nranges = 0;     // item ranges (wsplit has nranges + 1 entries); warp w
                       // does ranges w, w + warps, ...
  int dstride = 0;     // row stride of dE as given: Pp, or Pqc for the compact
                       // copy of the covered columns (0: Pp)
};
template <typename T>
acg_status launch_dst_quirk(const DstQuirkArgs<T>& a, WarpShape ws, int blocks, cudaStream_t s);

// The init pass in warp form, for Pp <= 64 and Pn <= 64 (the group form in
// acg_bp.cu runs for larger patterns): its grid (one wave of resident blocks;
// 0 if the pattern is too large) and its launch.
template <typename T>
int init_warp_blocks(int pn, int pe, int pp, int num_sms);
template <typename T>
acg_status launch_init_warp(const InitArgs<T>& a, int blocks, cudaStream_t s);

// Warps per launch that the source-side pass is split over (one wave).
template <typename T>
int src_stats_blocks_per_sm(WarpShape ws);

}  // namespace acg
