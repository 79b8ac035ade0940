// acg_iter.cuh -- one BP iteration: edge phase + vertex phase (acg_iter.cu).
#pragma once

#include <cuda_runtime.h>

#include "acg_internal.h"

namespace acg {

// Phase A work item = {vertex, first dst-CSR position, end position, partial
// row or -1}: a light vertex with all its in-edges (its maxima go to M), or one
// chunk of a heavy vertex (maxima go to the partial row).
template <typename T>
struct EdgeMaxArgs {
  const int4* items;
  int nitems;
  const int* wsplit;   // [warps + 1]: warp w does items [wsplit[w], wsplit[w+1])
  const int* src_of;   // [De] source vertex of each dst-CSR position
  const T* dE;         // [De][Pp]
  const T* vr_in;      // [Dn][Pp]
  T* M;                // [Dn][Pp] out: max over in-edges of VR' - dE
  T* partial;          // [npartial][Pp]
  int Pp;
};

template <typename T>
struct VertexUpdArgs {
  const int* d_off;    // [Dn+1] (in-degree: empty rows of M are -inf)
  const T* M;          // [Dn][Pp]
  T* vf;               // [Dn][Pp] read then overwritten
  T* vr_out;           // [Dn][Pp]
  const T* dEmin;      // [Dn][Pp]
  const T* B;          // [Dn][Pp]
  const T* CV;         // [Dn][Pnp]
  const double* glob_in;
  double* bpart;       // [slot][gridDim.x]
  double* mu_raw;      // [Dn][Pn] (last iteration)
  const int* pat;
  int Dn, Pn, Pe, Pp, Pnp;
  int last;
};

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
template <typename T>
acg_status launch_vertex_update(const VertexUpdArgs<T>& a, int blocks, cudaStream_t s);
template <typename T>
int vertex_update_blocks_per_sm(int pn, int pe, int pp);

}  // namespace acg
