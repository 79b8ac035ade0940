// acg_cdist.cuh -- register-blocked SIMT cost matrices (acg_cdist.cu).
#pragma once

#include <cuda_runtime.h>

#include "acg_internal.h"

namespace acg {

constexpr int kCdistEdge = 0;    // stats: LSE of -d over the covered quirk elements
constexpr int kCdistVertex = 1;  // stats: max(-d), LSE(d), LSE(-d)

// out[r][q] = || x[row(r)] - y[q] || for r < nrows, q < P; out[r][q] = 0 for
// P <= q < Pp.  row(r) = row ? row[r] : r.
template <typename T, typename F>
struct CdistRbArgs {
  const F* x;          // data features, row stride kstride
  const int* row;      // optional row index per output row
  const int* eid;      // edge mode: original edge id per output row (quirk test)
  const double* y;     // [P][K] pattern features
  T* out;              // [nrows][ostride]
  double* bpart;       // block partials (StatSpec{0,P} edge, {P,2P} vertex)
  long long nrows;
  long long De;
  long long lim;       // Pn * Dn
  int K, kstride, P, Pp, ostride;
};

template <typename T, typename F>
acg_status launch_cdist_rb(const CdistRbArgs<T, F>& a, int mode, int blocks, cudaStream_t s);
// The edge cost matrix without statistics (the covered-element log-sum-exps
// come from the destination-side quirk pass): one thread per row for K <= 32,
// else the tiled kernel.
template <typename T, typename F>
acg_status launch_cdist_edges(const CdistRbArgs<T, F>& a, int blocks, cudaStream_t s);

// The edge cost matrix of the mixed path on the tensor cores (acg_cdist_tc.cu):
// out[rowmap ? rowmap[r] : r][q] = ||x[r] - y[q]|| for q < P, 0 for P <= q < Pp;
// x FP32 rows of stride kstride.  With outq, the same rows' columns q < qcols
// (a multiple of 4, at most 16) also go to outq[row][qcols].  *err is set to 1
// if a bounded wait gave up.
bool cdist_tc_eligible(int K, int kstride, int P, int Pp);
acg_status launch_cdist_edges_tc(const float* x, int kstride, int K, const double* y, int P, int Pp,
                                 float* out, long long nrows, int* err, int num_sms, cudaStream_t s,
                                 const int* rowmap = nullptr, float* outq = nullptr, int qcols = 0);
// The vertex cost matrix of the mixed path on the tensor cores, with the
// per-column statistics of kCdistVertex as block partials (StatSpec{P, 2P}),
// one partial column per CTA: at most max_grid CTAs (0: no cap), the count
// used returned in *grid_used (at least 1; with no rows the partials are empty).
acg_status launch_cdist_vertex_tc(const float* x, int kstride, int K, const double* y, int P, int Pp,
                                  float* out, double* bpart, long long nrows, int max_grid, int* grid_used,
                                  int* err, int num_sms, cudaStream_t s);

}  // namespace acg
