/*
 * acg_oracle.h -- TEST INFRASTRUCTURE: CPU FP64 restatement of the reference
 * matcher (src/main.cu:66-257, src/ac.hxx:17-186).  Used only as the checker by
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg.
 */
#ifndef ACG_ORACLE_H
#define ACG_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same field layout as `struct Graph` (main.cu:8-19), host pointers. */
typedef struct acg_oracle_graph {
  uint64_t num_nodes;
  uint64_t node_feat_dim;
  uint64_t num_edges;
  uint64_t edge_feat_dim;
  const double* node_feats;
  const double* edge_feats;
  const uint64_t* srcs;
  const uint64_t* dsts;
} acg_oracle_graph;

/* 0 if the pair is valid; 1 bad sizes; 3 an endpoint out of range. */
int acg_oracle_check(const acg_oracle_graph* data, const acg_oracle_graph* patt);

/* Run the reference pipeline; mu_out is [data nodes][pattern nodes].
 * num_iters < 0 runs pattern num_nodes iterations (main.cu:160).
 * elapsed_us (may be NULL) receives the time of the window the reference
 * times (main.cu:104-249).  Returns 0, 1 (bad argument), 2 (out of memory) or
 * 3 (index out of range). */
int acg_oracle_match(const acg_oracle_graph* data, const acg_oracle_graph* patt,
                     int64_t num_iters, double* mu_out, double* elapsed_us);

/* The same with the optional C-null term (test.py:93-97, left out by the
 * reference: main.cu:83) when cnull_on is nonzero. */
int acg_oracle_match_opts(const acg_oracle_graph* data, const acg_oracle_graph* patt,
                          int64_t num_iters, int cnull_on, double* mu_out, double* elapsed_us);

int acg_oracle_threads(void);
void acg_oracle_set_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
