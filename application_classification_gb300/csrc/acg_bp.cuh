// acg_bp.cuh -- declarations of the matcher kernels (acg_bp.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "acg_internal.h"

namespace acg {

// Pattern incidence, as one int array on the device:
//   psrc[Pe] pdst[Pe] in_off[Pn+1] in_q[Pe] out_off[Pn+1] out_q[Pe]
// in_q lists, for each pattern vertex p, the pattern edges q with dst_q == p
// (ascending q); out_q those with src_q == p.
__host__ __device__ inline int pattern_ints(int pn, int pe) { return 4 * pe + 2 * (pn + 1); }

// Statistics produced by a kernel as per-block partials and combined by
// stat_finalize: `nmax` maxima, then `nlse` log-sum-exps (each an (m, s) pair
// in the partial buffer).  Partial layout: slot-major, [slot][block].
struct StatSpec {
  int nmax;
  int nlse;
  __host__ __device__ int slots() const { return nmax + 2 * nlse; }
  __host__ __device__ int outs() const { return nmax + nlse; }
};

// Launch configuration chosen per (value type, Pp, Pn).
struct GroupShape {
  int G;    // lanes per vertex
  int NQV;  // 16-byte vectors per lane
};
GroupShape choose_shape(int elem_bytes, int pp, int pn);

acg_status launch_finalize(const double* bpart, int nblocks, StatSpec spec, double* out,
                           cudaStream_t s);

// ---- initialisation kernels
// F: element type of the stored features (double: the caller's arrays;
// float: the data graph's FP32 copy used by the mixed path).
template <typename T, typename F>
struct CdistVArgs {
  const F* dv;       // [Dn][kstride]
  const double* pv;  // [Pn][Kv]
  T* dV;             // [Dn][Pnp] raw distances (normalised in place by init_vertex)
  double* bpart;     // stats: max(-dV) (Pn), LSE(dV) (Pn), LSE(-dV) (Pn)
  int Dn, Pn, Kv, kstride, Pnp;
};
template <typename T, typename F>
acg_status launch_cdist_v(const CdistVArgs<T, F>& a, int blocks, cudaStream_t s);

template <typename T, typename F>
struct CdistEArgs {
  const F* ef;        // features: gather ? [De][kstride] original order : dst-CSR order
  const int* eid;     // [De] original edge id at each dst-CSR position
  const double* pe;   // [Pe][Ke]
  T* dE;              // [De][Pp] out, dst-CSR order
  double* bpart;      // stats: LSE over covered elements of -dE (Pe)
  long long De;
  int Pe, Pp, Ke, kstride;
  int gather;         // 1: row = eid[i]; 0: row = i
  long long lim;      // Pn * Dn: flat positions below it hold -dE in the quirk buffer
};
template <typename T, typename F>
acg_status launch_cdist_e(const CdistEArgs<T, F>& a, int blocks, cudaStream_t s);

// dst[i][k] = (float)src[row ? row[i] : i][k] for k < K, zero up to kstride.
acg_status launch_convert_rows(const double* src, const int* row, long long n, int K, float* dst,
                               int kstride, cudaStream_t s);

// Static per-vertex reductions over a CSR of dE rows.
//   src mode: dEmin, B = LSE(-dE), Rbuf = max of the quirk buffer, over out-edges
//   dst mode: Fbuf = max of the quirk buffer, over in-edges
template <typename T>
struct RowPassArgs {
  const int4* items;
  int nitems;
  const int* row_of;  // src mode: dst-CSR row of each src-CSR position; dst mode: null
  const int* eid_of_row;  // [De] original edge id of each dst-CSR row
  const T* dE;
  T* partial;         // [npartial][4][Pp]
  const int* hbase;
  const int* hcount;
  const int* hvert;
  int nheavy;
  int chunk;
  const int* off;     // CSR offsets (for chunk index)
  T* out_min;         // src: dEmin
  T* out_lse;         // src: B
  T* out_buf;         // src: Rbuf, dst: Fbuf
  long long De;
  long long lim;
  int Dn, Pe, Pp;
  int src_mode;
};
template <typename T>
acg_status launch_row_pass(const RowPassArgs<T>& a, GroupShape gs, int blocks, bool heavy,
                           cudaStream_t s);

template <typename T>
struct InitArgs {
  const int* d_off;
  const int* s_off;
  T* CV;               // [Dn][Pnp]: raw dV in, normalised cost out
  T* CVlo;             // [Dn][Pnp] out: low part of the cost (FP32 only, else null)
  const T* Rbuf;       // [Dn][Pp]
  const T* Fbuf;       // [Dn][Pp]
  const T* B;          // [Dn][Pp]
  const T* dEmin;      // [Dn][Pp]
  T* vf;               // [Dn][Pp] out: Y = VF - dEmin of iteration 1 (shift 0)
  T* vr;               // [Dn][Pp] out: Z = VR of iteration 1 (shift 0)
  const double* gv;    // [maxneg(Pn) | lse_pos(Pn) | lse_neg(Pn)]
  const double* ge;    // [Pe] LSE over covered quirk elements
  double* bpart;       // stats: mVF, mVR (max), lR, lF (lse)
  const int* pat;
  long long De;
  long long lim;
  int Dn, Pn, Pe, Pp, Pnp;
};
template <typename T>
acg_status launch_init_vertex(const InitArgs<T>& a, GroupShape gs, int blocks, cudaStream_t s);

// mu[v][p] -= S[p]
acg_status launch_mu_output(double* mu, const double* S, long long Dn, int Pn, cudaStream_t s);

}  // namespace acg
