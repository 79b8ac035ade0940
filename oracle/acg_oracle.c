/*
 * acg_oracle.c -- TEST INFRASTRUCTURE: CPU restatement of the reference's
 * ApplicationClassification matcher (porumbes/application_classification,
 * src/main.cu:66-257 and src/ac.hxx:17-186), in plain C with OpenMP, FP64.
 *
 * This file is the checker.  It is linked only by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg; the product
 * library never calls it.  It follows the reference pass by pass -- the same
 * buffers, the same order of normalisations, the same un-shifted
 * log(exp(x)) - log(sum exp) normaliser, the same fill-then-scatter edge
 * maxima -- so that it is an independent check of the GPU kernels, which use
 * an algebraically restructured form.
 *
 * Parity pin: tests/test_oracle.py checks this restatement against golden
 * outputs of the unmodified reference compiled for the CPU (oracle/_ref, built
 * by `make -C oracle ref` with Thrust's OpenMP backend) on seeded inputs, stored
 * under tests/golden/.
 *
 * Determinism: every reduction sums fixed 4096-element chunks and then the
 * chunk partials in order, so results do not depend on the thread count.
 * Build with -ffp-contract=off so that no FMA contraction changes rounding.
 *
 * Reference quirk kept (main.cu:113-114): RE_t and FE_t are set to -CE_t only
 * on their first Pn*Dn elements; the rest of those Pe*De buffers is what
 * cudaMalloc returned, which this restatement takes as zero (fresh device
 * allocations are zero-filled in practice, and the CPU build of the reference
 * zero-fills them).  When Pn*Dn > Pe*De the reference reads and writes past the
 * end of its buffers; here the negation is clamped to Pe*De.
 */
#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "acg_oracle.h"

#define CHUNK 4096

/* ac.hxx:33-56 -- out[j * n_b + i] = || a_j - b_i ||_2, summed over the
 * feature index in order, then sqrt. */
static void cdist(uint64_t n_a, uint64_t n_b, uint64_t dim, const double* a,
                  const double* b, double* out) {
#pragma omp parallel for schedule(static)
  for (int64_t j = 0; j < (int64_t)n_a; ++j)
    for (uint64_t i = 0; i < n_b; ++i) {
      const double* v1 = a + (uint64_t)j * dim;
      const double* v2 = b + i * dim;
      double dist = 0.0;
      for (uint64_t k = 0; k < dim; ++k) dist += (v1[k] - v2[k]) * (v1[k] - v2[k]);
      out[(uint64_t)j * n_b + i] = sqrt(dist);
    }
}

/* Deterministic sum of x[0..n): fixed chunks, then partials in order. */
static double chunked_sum(const double* x, uint64_t n) {
  const uint64_t nch = (n + CHUNK - 1) / CHUNK;
  if (nch <= 1) {
    double s = 0.0;
    for (uint64_t i = 0; i < n; ++i) s += x[i];
    return s;
  }
  double* part = (double*)malloc(sizeof(double) * nch);
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < (int64_t)nch; ++c) {
    const uint64_t lo = (uint64_t)c * CHUNK, hi = lo + CHUNK < n ? lo + CHUNK : n;
    double s = 0.0;
    for (uint64_t i = lo; i < hi; ++i) s += x[i];
    part[c] = s;
  }
  double s = 0.0;
  for (uint64_t c = 0; c < nch; ++c) s += part[c];
  free(part);
  return s;
}

/* ac.hxx:77-106 (RowSoftmax2_prealloc): x = exp(x); tmp[r] = sum_c x[r,c];
 * tmp = log(tmp); x = log(x); x[r,c] -= tmp[r].  No max shift. */
static void row_softmax(uint64_t n_row, uint64_t n_col, double* x) {
  const uint64_t n = n_row * n_col;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)n; ++i) x[i] = exp(x[i]);
  double* tmp = (double*)malloc(sizeof(double) * (n_row ? n_row : 1));
  for (uint64_t r = 0; r < n_row; ++r) tmp[r] = log(chunked_sum(x + r * n_col, n_col));
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)n; ++i) x[i] = log(x[i]);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)n; ++i) x[i] -= tmp[(uint64_t)i / n_col];
  free(tmp);
}

/* ac.hxx:58-75 (RowMax2): out[r] = max_c x[r,c]. */
static void row_max(uint64_t n_row, uint64_t n_col, const double* x, double* out) {
#pragma omp parallel for schedule(static)
  for (int64_t r = 0; r < (int64_t)n_row; ++r) {
    const double* row = x + (uint64_t)r * n_col;
    double m = n_col ? row[0] : 0.0;
    for (uint64_t c = 1; c < n_col; ++c) m = row[c] > m ? row[c] : m;
    out[r] = m;
  }
}

/* ac.hxx:115-149 (EdgeMaxReduce2_t) with the CAS max of helpers.hxx:36-55:
 * XMax[r, v] = VYMax[r] for every data vertex v, then for every data edge e,
 * XMax[r, nodes[e]] = fmax(XE[r, e], XMax[r, nodes[e]]).  Rows are
 * independent, so each row runs its scatter serially (no atomics needed). */
static void edge_max_reduce(uint64_t n_col_in, uint64_t n_col_out, uint64_t n_row,
                            const double* vymax, const double* xe, double* xmax,
                            const uint64_t* nodes) {
#pragma omp parallel for schedule(static)
  for (int64_t r = 0; r < (int64_t)n_row; ++r) {
    double* out = xmax + (uint64_t)r * n_col_out;
    for (uint64_t v = 0; v < n_col_out; ++v) out[v] = vymax[r];
    const double* in = xe + (uint64_t)r * n_col_in;
    for (uint64_t e = 0; e < n_col_in; ++e) {
      double* t = out + nodes[e];
      *t = fmax(in[e], *t);
    }
  }
}

/* ac.hxx:151-186 (ComputeMU2_t): MU = -CV; then for every pattern edge q and
 * data vertex v: MU[dst_q, v] += FMax[q, v]; MU[src_q, v] += RMax[q, v].
 * Summed in q order (the reference's atomicAdd order is unspecified). */
static void compute_mu(uint64_t dn, uint64_t pe, uint64_t pn, const double* cv,
                       const double* fmax_t, const double* rmax_t,
                       const uint64_t* psrc, const uint64_t* pdst, double* mu) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)(pn * dn); ++i) mu[i] = -cv[i];
#pragma omp parallel for schedule(static)
  for (int64_t v = 0; v < (int64_t)dn; ++v)
    for (uint64_t q = 0; q < pe; ++q) {
      mu[pdst[q] * dn + (uint64_t)v] += fmax_t[q * dn + (uint64_t)v];
      mu[psrc[q] * dn + (uint64_t)v] += rmax_t[q * dn + (uint64_t)v];
    }
}

static double now_us(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec * 1e6 + (double)ts.tv_nsec * 1e-3;
}

int acg_oracle_check(const acg_oracle_graph* data, const acg_oracle_graph* patt) {
  if (!data || !patt) return 1;
  if (patt->num_nodes == 0) return 1;
  if (data->node_feat_dim != patt->node_feat_dim) return 1;
  if (data->edge_feat_dim != patt->edge_feat_dim) return 1;
  for (uint64_t e = 0; e < data->num_edges; ++e)
    if (data->srcs[e] >= data->num_nodes || data->dsts[e] >= data->num_nodes) return 3;
  for (uint64_t q = 0; q < patt->num_edges; ++q)
    if (patt->srcs[q] >= patt->num_nodes || patt->dsts[q] >= patt->num_nodes) return 3;
  return 0;
}

int acg_oracle_match(const acg_oracle_graph* data, const acg_oracle_graph* patt,
                     int64_t num_iters, double* mu_out, double* elapsed_us) {
  return acg_oracle_match_opts(data, patt, num_iters, 0, mu_out, elapsed_us);
}

int acg_oracle_match_opts(const acg_oracle_graph* data, const acg_oracle_graph* patt,
                          int64_t num_iters, int cnull_on, double* mu_out, double* elapsed_us) {
  const int chk = acg_oracle_check(data, patt);
  if (chk) return chk;
  const uint64_t dn = data->num_nodes, de = data->num_edges;
  const uint64_t pn = patt->num_nodes, pe = patt->num_edges;
  const uint64_t iters = num_iters < 0 ? pn : (uint64_t)num_iters;

  /* main.cu:80-99 -- the reference's buffers, zero-filled. */
  double* cv_t = (double*)calloc(pn * dn + 1, sizeof(double));
  double* mu_t = (double*)calloc(pn * dn + 1, sizeof(double));
  double* vrmax = (double*)calloc(pe + 1, sizeof(double));
  double* vfmax = (double*)calloc(pe + 1, sizeof(double));
  double* ce_t = (double*)calloc(pe * de + 1, sizeof(double));
  double* re_t = (double*)calloc(pe * de + 1, sizeof(double));
  double* fe_t = (double*)calloc(pe * de + 1, sizeof(double));
  double* vr_t = (double*)calloc(pe * dn + 1, sizeof(double));
  double* vf_t = (double*)calloc(pe * dn + 1, sizeof(double));
  double* rmax_t = (double*)calloc(pe * dn + 1, sizeof(double));
  double* fmax_t = (double*)calloc(pe * dn + 1, sizeof(double));
  if (!cv_t || !mu_t || !vrmax || !vfmax || !ce_t || !re_t || !fe_t || !vr_t || !vf_t ||
      !rmax_t || !fmax_t) {
    free(cv_t); free(mu_t); free(vrmax); free(vfmax); free(ce_t); free(re_t);
    free(fe_t); free(vr_t); free(vf_t); free(rmax_t); free(fmax_t);
    return 2;
  }
  const double t0 = now_us();

  /* prep, main.cu:109-146 */
  cdist(pn, dn, patt->node_feat_dim, patt->node_feats, data->node_feats, cv_t);
  cdist(pe, de, patt->edge_feat_dim, patt->edge_feats, data->edge_feats, ce_t);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)(pn * dn); ++i) mu_t[i] = -cv_t[i];
  {
    const uint64_t nneg = pn * dn < pe * de ? pn * dn : pe * de; /* main.cu:113-114 */
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)nneg; ++i) {
      re_t[i] = -ce_t[i];
      fe_t[i] = -ce_t[i];
    }
  }
  row_softmax(pn, dn, cv_t); /* main.cu:116-120 */
  row_softmax(pn, dn, mu_t);
  row_softmax(pe, de, ce_t);
  row_softmax(pe, de, re_t);
  row_softmax(pe, de, fe_t);
#pragma omp parallel for schedule(static) /* main.cu:122-133 init_VX */
  for (int64_t off = 0; off < (int64_t)(dn * pe); ++off) {
    const uint64_t i = (uint64_t)off % dn, j = (uint64_t)off / dn;
    vr_t[off] = mu_t[dn * patt->srcs[j] + i];
    vf_t[off] = mu_t[dn * patt->dsts[j] + i];
  }
  row_max(pe, dn, vf_t, vfmax); /* main.cu:135-136 */
  row_max(pe, dn, vr_t, vrmax);
  edge_max_reduce(de, dn, pe, vfmax, re_t, rmax_t, data->srcs); /* main.cu:138-141 */
  edge_max_reduce(de, dn, pe, vrmax, fe_t, fmax_t, data->dsts); /* main.cu:143-146 */

  /* Optional C-null term, test.py:93-97 (commented out there; the reference's
   * main.cu:83 leaves it out): cnull = normprob over q of
   * max(||pe_q||, max_e L(ce)[q][e]); ce_t holds L(ce) here. */
  double* cnull = NULL;
  if (cnull_on && pe > 0) {
    cnull = (double*)calloc(pe, sizeof(double));
    if (!cnull) {
      free(cv_t); free(mu_t); free(vrmax); free(vfmax); free(ce_t); free(re_t);
      free(fe_t); free(vr_t); free(vf_t); free(rmax_t); free(fmax_t);
      return 2;
    }
    const uint64_t ke = patt->edge_feat_dim;
    double cmax = -INFINITY;
    for (uint64_t q = 0; q < pe; ++q) {
      double nn = 0.0;
      for (uint64_t k = 0; k < ke; ++k) nn += patt->edge_feats[q * ke + k] * patt->edge_feats[q * ke + k];
      double m = sqrt(nn);
      for (uint64_t e = 0; e < de; ++e) m = fmax(m, ce_t[q * de + e]);
      cnull[q] = m;
      cmax = fmax(cmax, m);
    }
    double ssum = 0.0;
    for (uint64_t q = 0; q < pe; ++q) ssum += exp(cnull[q] - cmax);
    const double lse = cmax + log(ssum);
    for (uint64_t q = 0; q < pe; ++q) cnull[q] -= lse;
  }

  /* loop, main.cu:160-245 */
  for (uint64_t it = 0; it < iters; ++it) {
#pragma omp parallel for schedule(static) /* step1, main.cu:165-176 */
    for (int64_t off = 0; off < (int64_t)(dn * pe); ++off) {
      const uint64_t r = (uint64_t)off / dn, c = (uint64_t)off % dn;
      vf_t[off] = mu_t[dn * patt->dsts[r] + c] - fmax_t[off];
      vr_t[off] = mu_t[dn * patt->srcs[r] + c] - rmax_t[off];
    }
#pragma omp parallel for schedule(static) /* step2, main.cu:181-192 */
    for (int64_t off = 0; off < (int64_t)(de * pe); ++off) {
      const uint64_t r = (uint64_t)off / de, c = (uint64_t)off % de;
      fe_t[off] = vr_t[dn * r + data->srcs[c]] - ce_t[off];
      re_t[off] = vf_t[dn * r + data->srcs[c]] - ce_t[off];
    }
    row_max(pe, dn, vf_t, vfmax);                                 /* step3_a */
    if (cnull) /* test.py:140: bak_max = max(bak_max, v_fwd_max - cnull) */
      for (uint64_t q = 0; q < pe; ++q) vfmax[q] -= cnull[q];
    row_softmax(pe, de, re_t);                                    /* step3_b */
    edge_max_reduce(de, dn, pe, vfmax, re_t, rmax_t, data->srcs); /* step3_c */
    row_max(pe, dn, vr_t, vrmax);                                 /* step4 */
    if (cnull) /* test.py:139: fwd_max = max(fwd_max, v_bak_max - cnull) */
      for (uint64_t q = 0; q < pe; ++q) vrmax[q] -= cnull[q];
    row_softmax(pe, de, fe_t);
    edge_max_reduce(de, dn, pe, vrmax, fe_t, fmax_t, data->dsts);
    compute_mu(dn, pe, pn, cv_t, fmax_t, rmax_t, patt->srcs, patt->dsts, mu_t); /* step5 */
    row_softmax(pn, dn, mu_t);
  }

  /* main.cu:247 transpose [Pn][Dn] -> [Dn][Pn] (ac.hxx:17-31) */
#pragma omp parallel for schedule(static)
  for (int64_t off = 0; off < (int64_t)(pn * dn); ++off) {
    const uint64_t r = (uint64_t)off / dn, c = (uint64_t)off % dn;
    mu_out[c * pn + r] = mu_t[off];
  }
  if (elapsed_us) *elapsed_us = now_us() - t0;

  free(cv_t); free(mu_t); free(vrmax); free(vfmax); free(ce_t); free(re_t);
  free(fe_t); free(vr_t); free(vf_t); free(rmax_t); free(fmax_t);
  free(cnull);
  return 0;
}

int acg_oracle_threads(void) { return omp_get_max_threads(); }
void acg_oracle_set_threads(int n) {
  if (n > 0) omp_set_num_threads(n);
}
