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
  int f32 = 0;  // merge with the FP32 exponential (statistics of FP32 kernels)
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

// dst[i][k] = (float)src[row ? row[i] : i][k] for k < K, zero up to kstride.
acg_status launch_convert_rows(const double* src, const int* row, long long n, int K, float* dst,
                               int kstride, cudaStream_t s);
// Rows [e0, e1) of src (original edge order) to FP32 (zero padded to kstride):
// into x32 in the same order and into dst at row pos[e].
acg_status launch_convert_scatter(const double* src, long long e0, long long e1, int K, const int* pos,
                                  float* x32, float* dst, int kstride, cudaStream_t s);
// pos[perm[r]] = r for r < n
acg_status launch_inverse_perm(const int* perm, long long n, int* pos, cudaStream_t s);

template <typename T>
struct InitArgs {
  const int* d_off;
  const int* s_off;
  T* CV;               // [Dn][Pnp]: raw dV in, normalised cost out
  T* CVlo;             // [Dn][Pnp] out: low part of the cost (FP32 only, else null)
  const T* Rq;         // [Dn][Pqc] quirk maximum over out-edges, columns < qcov
  const T* Fq;         // [Dn][Pqc] quirk maximum over in-edges, columns < qcov
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
  int Pqc, qcov;       // (the later quirk columns are zero over any edge)
  const long long* qlim_col;  // [Pe] column q covers original edge ids < qlim_col[q]
  // Recording for the adjoint (warp form only; null otherwise): f = VF of the
  // first iteration ([Dn][Pp], zero past Pe) and MU0 as hi + lo ([Dn][Pn]).
  T* rec_f = nullptr;
  T* rec_mh = nullptr;
  T* rec_ml = nullptr;
};
template <typename T>
acg_status launch_init_vertex(const InitArgs<T>& a, GroupShape gs, int blocks, cudaStream_t s);

// mu[v][p] -= S[p]
acg_status launch_mu_output(double* mu, const double* S, long long Dn, int Pn, cudaStream_t s);

}  // namespace acg
