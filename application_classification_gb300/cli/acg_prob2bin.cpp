// acg_prob2bin -- the reference's prob2bin.py (CSV pair -> binary graph,
// prob2bin.py:11-63) as a native tool, and the way back.
//
//   acg_prob2bin VERTEX.csv EDGES.csv OUT.bin
//   acg_prob2bin --to-csv IN.bin VERTEX.csv EDGES.csv
//
// The CSV layout is the reference's: a header line "N C", then rows "id f..."
// (vertices, ids equal to the row number, prob2bin.py:28-29) or
// "src dst f..." (edges), space separated.  The binary layout is the one
// loadGraph reads (main.cu:21-44).  Exit status 0 on success.
#include <cstdio>
#include <cstring>

#include "acg_io.h"

int main(int argc, char** argv) {
  acg_host_graph g{};
  acg_status st;
  if (argc == 5 && std::strcmp(argv[1], "--to-csv") == 0) {
    st = acg_graph_read_bin(argv[2], &g);
    if (st == ACG_OK) st = acg_graph_write_csv(argv[3], argv[4], &g);
  } else if (argc == 4 && argv[1][0] != '-') {
    st = acg_graph_read_csv(argv[1], argv[2], &g);
    if (st == ACG_OK) st = acg_graph_write_bin(argv[3], &g);
  } else {
    std::fprintf(stderr,
                 "usage: acg_prob2bin VERTEX.csv EDGES.csv OUT.bin\n"
                 "       acg_prob2bin --to-csv IN.bin VERTEX.csv EDGES.csv\n");
    return 2;
  }
  if (st != ACG_OK) std::fprintf(stderr, "acg_prob2bin: %s\n", acg_last_error());
  else std::printf("%llu vertices x %llu features, %llu edges x %llu features\n",
                   (unsigned long long)g.num_nodes, (unsigned long long)g.node_feat_dim,
                   (unsigned long long)g.num_edges, (unsigned long long)g.edge_feat_dim);
  acg_host_graph_free(&g);
  return st == ACG_OK ? 0 : 1;
}
