// acg_cnull.cu -- the C-null term of the PNNL formulation (optional).
//
// The reference leaves it out (main.cu:83 "Ignoring for now"; test.py:93-97
// has it commented out and uses zeros).  When acg_options.cnull is set:
//   cn[q]    = max(||pe_q||_2, max_e L(dE)[q][e]),  L(dE)[q][e] = dE[q][e] - LSE_e dE[q][e]
//   cnull[q] = cn[q] - LSE_q cn[q]                   (normprob over the pattern edges;
//                                                     in a union, over each member's)
// and every BP iteration subtracts cnull[q] from both fills of column q
// (test.py:139-140: fwd_max = max(fwd_max, v_bak_max - cnull), likewise bak_max).
// The column statistics of dE are one pass over the [De][Pp] matrix: per
// block partial maxima and log-sum-exps, combined by stat_finalize.
#include <cuda_runtime.h>

#include "acg_bp.cuh"
#include "acg_device.cuh"
#include "acg_plan.h"

namespace acg {

namespace {

constexpr int kNT = 256;

// Block (x, y): rows [De x / gridDim.x, De (x + 1) / gridDim.x), columns
// [y * cw, y * cw + cw).  Thread t: column t % cw, rows t / cw + k * (kNT / cw).
template <typename T>
__global__ void __launch_bounds__(kNT)
cnull_stats_kernel(const T* __restrict__ dE, long long De, int Pe, int Pp, int cw,
                   double* __restrict__ part) {
  __shared__ double s_m[kNT], s_l[kNT], s_s[kNT];
  const int nb = gridDim.x, rs = kNT / cw;
  const int c = threadIdx.x % cw, rl = threadIdx.x / cw;
  const int q = blockIdx.y * cw + c;
  const long long r0 = De * blockIdx.x / nb, r1 = De * (blockIdx.x + 1) / nb;
  double mx = -CUDART_INF, lm = -CUDART_INF, ls = 0.0;
  if (rl < rs && q < Pe) {
    for (long long r = r0 + rl; r < r1; r += rs) {
      const double x = (double)dE[(size_t)r * Pp + q];
      mx = fmax(mx, x);
      lse_merge(lm, ls, x, 1.0);
    }
  }
  s_m[threadIdx.x] = mx;
  s_l[threadIdx.x] = lm;
  s_s[threadIdx.x] = ls;
  __syncthreads();
  if (threadIdx.x < cw && q < Pe) {
    for (int k = 1; k < rs; ++k) {
      const int i = k * cw + c;
      mx = fmax(mx, s_m[i]);
      lse_merge(lm, ls, s_l[i], s_s[i]);
    }
    // StatSpec{Pe, Pe} layout: maxima in slots [0, Pe), then (m, s) pairs
    part[(size_t)q * nb + blockIdx.x] = mx;
    part[(size_t)(Pe + 2 * q) * nb + blockIdx.x] = lm;
    part[(size_t)(Pe + 2 * q + 1) * nb + blockIdx.x] = ls;
  }
}

// One block: cnull from the column statistics and the pattern edge features.
// The normaliser runs over each member's columns (a union of patterns: its
// columns' member ids in qmember; a single pattern: qmember null), one thread
// per member merging its columns in column order.
__global__ void __launch_bounds__(kNT)
cnull_final_kernel(const double* __restrict__ st, const double* __restrict__ pe, int Pe, int Ke,
                   long long De, const int* __restrict__ qmember, int nmembers,
                   double* __restrict__ cnull) {
  __shared__ double s_L[kNT];
  for (int q = threadIdx.x; q < Pe; q += kNT) {
    double nn = 0.0;
    for (int k = 0; k < Ke; ++k) nn += pe[(size_t)q * Ke + k] * pe[(size_t)q * Ke + k];
    double cn = sqrt(nn);
    if (De > 0) cn = fmax(cn, st[q] - st[Pe + q]);  // max_e L(dE)[q][e]
    cnull[q] = cn;
  }
  __syncthreads();
  for (int m = threadIdx.x; m < nmembers; m += kNT) {
    double lm = -CUDART_INF, ls = 0.0;
    for (int q = 0; q < Pe; ++q)
      if (!qmember || qmember[q] == m) lse_merge(lm, ls, cnull[q], 1.0);
    s_L[m] = lm + log(ls);
  }
  __syncthreads();
  for (int q = threadIdx.x; q < Pe; q += kNT) cnull[q] -= s_L[qmember ? qmember[q] : 0];
}

}  // namespace

int cnull_blocks(int num_sms) { return 2 * num_sms; }

acg_status run_cnull(acg_plan* P, cudaStream_t s) {
  const int Pe = P->Pe, Pp = P->Pp;
  if (!P->cnull || Pe == 0) return ACG_OK;
  const long long De = P->data->De;
  double* st = P->cnull + Pe;  // [2 Pe]: max dE, LSE dE per column
  if (De > 0) {
    const int cw = Pe < kNT ? Pe : kNT;
    const dim3 grid(cnull_blocks(P->data->num_sms), (Pe + cw - 1) / cw);
    if (P->prec == ACG_PREC_FP64)
      cnull_stats_kernel<double><<<grid, kNT, 0, s>>>((const double*)P->dE, De, Pe, Pp, cw, P->cnull_part);
    else
      cnull_stats_kernel<float><<<grid, kNT, 0, s>>>((const float*)P->dE, De, Pe, Pp, cw, P->cnull_part);
    ACG_LAUNCH_CHECK();
    ACG_TRY(launch_finalize(P->cnull_part, (int)grid.x, StatSpec{Pe, Pe}, st, s));
    P->launches += 2;
  }
  if (P->nmembers < 1 || P->nmembers > kNT)
    return set_error(ACG_ERR_UNSUPPORTED, "run_cnull: %d patterns in one group", P->nmembers);
  cnull_final_kernel<<<1, kNT, 0, s>>>(st, P->pe, Pe, P->data->Ke, De, P->qmember, P->nmembers,
                                       P->cnull);
  ACG_LAUNCH_CHECK();
  P->launches += 1;
  return ACG_OK;
}

}  // namespace acg
