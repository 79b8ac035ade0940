/*
 * acg_io.h -- host-side graph I/O and seeded graph generators.
 *
 * These functions run on the CPU only and never touch a GPU.  They keep the
 * reference front end's file formats so that the new host driver is a drop-in
 * for the reference's `main data.bin pattern.bin`:
 *
 *   binary graph  (reader: src/main.cu:21-63 `loadGraph`;
 *                  writer: prob2bin.py:42-62)
 *       u64 num_nodes, u64 node_feat_dim, u64 num_edges, u64 edge_feat_dim,
 *       f64 node_feats[num_nodes][node_feat_dim],
 *       f64 edge_feats[num_edges][edge_feat_dim],
 *       u64 srcs[num_edges], u64 dsts[num_edges]              (native endian)
 *
 *   CSV pair      (reader semantics: prob2bin.py:11-40)
 *       <name>.Vertex.csv : header "N C", then rows "id f_1 .. f_{C-1}"
 *       <name>.Edges.csv  : header "M C", then rows "src dst f_1 .. f_{C-2}"
 *       space separated; vertex ids must equal the row number
 *       (prob2bin.py:28-29 asserts this).
 *
 * All functions return an acg_status (0 = OK) and, on failure, set the
 * thread-local message returned by acg_last_error().
 */
#ifndef ACG_IO_H
#define ACG_IO_H

#include <stdint.h>
#include "acg.h"

#ifdef __cplusplus
extern "C" {
#endif

/* A graph whose arrays live in host memory (malloc'd by these functions). */
typedef struct acg_host_graph {
  uint64_t num_nodes;
  uint64_t node_feat_dim;
  uint64_t num_edges;
  uint64_t edge_feat_dim;
  double* node_feats;  /* [num_nodes][node_feat_dim] */
  double* edge_feats;  /* [num_edges][edge_feat_dim] */
  uint64_t* srcs;      /* [num_edges] */
  uint64_t* dsts;      /* [num_edges] */
  uint64_t edge_capacity; /* edges the arrays can hold; appends within it keep
                             every pointer valid */
} acg_host_graph;

/* Allocate zeroed arrays for the given sizes (replaces anything held; `g`
 * must be zeroed or hold a graph from these functions). */
acg_status acg_host_graph_alloc(acg_host_graph* g, uint64_t num_nodes,
                                uint64_t node_feat_dim, uint64_t num_edges,
                                uint64_t edge_feat_dim);
/* Free the arrays and zero the struct.  Safe on a zeroed struct. */
void acg_host_graph_free(acg_host_graph* g);
/* View of a host graph as an acg_graph (pointers shared, no copy). */
acg_graph acg_host_graph_view(const acg_host_graph* g);

/* Binary format; replaces `loadGraph`'s file read (main.cu:21-44), with the
 * header and every array length checked against the file size. */
acg_status acg_graph_read_bin(const char* path, acg_host_graph* out);
/* Binary format writer (prob2bin.py:42-62 layout). */
acg_status acg_graph_write_bin(const char* path, const acg_host_graph* g);

/* CSV pair reader (prob2bin.py:11-40).  Either path may be NULL: a NULL edges
 * path yields a graph with no edges and edge_feat_dim 0. */
acg_status acg_graph_read_csv(const char* vertex_csv, const char* edges_csv,
                              acg_host_graph* out);
/* CSV pair writer; floats as "%.17g" so that a write/read round trip is exact. */
acg_status acg_graph_write_csv(const char* vertex_csv, const char* edges_csv,
                               const acg_host_graph* g);

/* ---------------- mu output -------------------------------------------- */
/* Write mu [rows][cols] (row-major, host memory) as text, one "%e" value per
 * line, exactly the characters the reference's printf loop prints
 * (main.cu:255-257), formatted in parallel.  path NULL writes to stdout. */
acg_status acg_mu_write_text(const char* path, const double* mu, uint64_t rows,
                             uint64_t cols);
/* Write mu [rows][cols] as raw native-endian f64 (no header). */
acg_status acg_mu_write_bin(const char* path, const double* mu, uint64_t rows,
                            uint64_t cols);

/* ---------------- seeded generators ------------------------------------ */
/* Every random value is a pure function of (seed, stream, index), so results
 * do not depend on the thread count.  Features are i.i.d. N(0,1) by the
 * Box-Muller transform. */

/* Generated graphs reserve room for ACG_EDGE_RESERVE more edges, so that
 * acg_gen_plant / acg_gen_fill_edges append in place without moving arrays. */
#define ACG_EDGE_RESERVE 4096

/* Directed Erdos-Renyi graph with exactly `m` distinct edges, no self-loops. */
acg_status acg_gen_er(uint64_t n, uint64_t m, uint64_t node_feat_dim,
                      uint64_t edge_feat_dim, uint64_t seed,
                      acg_host_graph* out);

/* R-MAT graph: 2^scale vertices, edge_factor * 2^scale sampled edges with
 * quadrant probabilities (a, b, c, 1-a-b-c); self-loops and duplicate edges
 * removed; edges kept in sampling order (first occurrence). */
acg_status acg_gen_rmat(int scale, int edge_factor, double a, double b,
                        double c, uint64_t node_feat_dim,
                        uint64_t edge_feat_dim, uint64_t seed,
                        acg_host_graph* out);

/* Plant a pattern into `data`: grow a weakly connected set of `pn` data
 * vertices by a random walk, keep its walk tree plus random induced edges up
 * to `pe` pattern edges (adding new data edges among the set, with fresh
 * N(0,1) features, when the induced subgraph has fewer than `pe`), relabel the
 * set by a random permutation, and copy features with N(0, noise^2) added.
 * `data` may grow (edges appended).  truth_vertex[i] (may be NULL) receives
 * the data vertex planted as pattern vertex i; truth_edge[j] (may be NULL)
 * the data edge planted as pattern edge j. */
acg_status acg_gen_plant(acg_host_graph* data, uint64_t pn, uint64_t pe,
                         double noise, uint64_t seed,
                         acg_host_graph* pattern_out, uint64_t* truth_vertex,
                         uint64_t* truth_edge);

/* Top a graph up with uniformly random new edges (no self-loops, no
 * duplicates, fresh N(0,1) features) until it has exactly `m` edges. */
acg_status acg_gen_fill_edges(acg_host_graph* g, uint64_t m, uint64_t seed);

#ifdef __cplusplus
}
#endif
#endif /* ACG_IO_H */
