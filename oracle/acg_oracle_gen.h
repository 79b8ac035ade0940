/*
 * acg_oracle_gen.h -- TEST INFRASTRUCTURE: seeded synthetic workloads for the
 * oracle checks and the CPU baseline, built without the product library (the
 * same graphs, byte for byte, as the product's generators for the same
 * arguments).  Return codes: 0 ok, 1 bad argument, 2 out of memory.
 */
#ifndef ACG_ORACLE_GEN_H
#define ACG_ORACLE_GEN_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* A host graph in the layout of `struct Graph` (main.cu:8-19); arrays malloc'd. */
typedef struct acgo_graph {
  uint64_t num_nodes;
  uint64_t node_feat_dim;
  uint64_t num_edges;
  uint64_t edge_feat_dim;
  double* node_feats;
  double* edge_feats;
  uint64_t* srcs;
  uint64_t* dsts;
} acgo_graph;

void acgo_free(acgo_graph* g);
int acgo_gen_er(uint64_t n, uint64_t m, uint64_t kv, uint64_t ke, uint64_t seed, acgo_graph* out);
int acgo_gen_rmat(int scale, int edge_factor, double a, double b, double c, uint64_t kv, uint64_t ke,
                  uint64_t seed, acgo_graph* out);
int acgo_fill_edges(acgo_graph* g, uint64_t m, uint64_t seed);
int acgo_plant(acgo_graph* data, uint64_t pn, uint64_t pe, double noise, uint64_t seed, acgo_graph* pat,
               uint64_t* truth_vertex, uint64_t* truth_edge);

#ifdef __cplusplus
}
#endif
#endif
