// acg_main -- drop-in for the reference program `main data.bin pattern.bin`
// (src/main.cu).  It reads the two graphs, copies them to the GPU as
// loadGraph does (main.cu:21-63), runs the whole match through the C ABI,
// prints "elapsed=<microseconds>" on stderr for the window the reference
// times (main.cu:104-250: from the loaded device graphs to mu in [Dn][Pn]),
// and writes mu as one "%e" line per entry on stdout (main.cu:255-257).
//
//   acg_main [options] DATA PATTERN
//     --precision fp64|mixed   arithmetic of the match (default fp64, as the
//                              reference)
//     --iters N                BP iterations (default: the pattern's vertex
//                              count, main.cu:160)
//     --cnull                  add the C-null term the reference leaves out
//                              (acg_options.cnull)
//     --csv                    DATA and PATTERN are CSV prefixes: P.Vertex.csv
//                              and P.Edges.csv (the prob2bin.py layout)
//     --out PATH               write mu to PATH instead of stdout
//     --binary                 write mu as raw f64 instead of text
// Exit status 0 on success; otherwise the library's message on stderr.
#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "acg.h"
#include "acg_io.h"

namespace {

int fail(const char* what) {
  std::fprintf(stderr, "acg_main: %s: %s\n", what, acg_last_error());
  return 1;
}

int usage() {
  std::fprintf(stderr,
               "usage: acg_main [--precision fp64|mixed] [--iters N] [--cnull] [--csv] [--out PATH] "
               "[--binary] DATA PATTERN\n");
  return 2;
}

// Device copies of a host graph (the reference's loadGraph allocations).
struct DeviceGraph {
  acg_graph g{};
  std::vector<void*> bufs;
  ~DeviceGraph() {
    for (void* p : bufs) cudaFree(p);
  }
  bool upload(const acg_host_graph& h) {
    g.num_nodes = h.num_nodes;
    g.node_feat_dim = h.node_feat_dim;
    g.num_edges = h.num_edges;
    g.edge_feat_dim = h.edge_feat_dim;
    auto put = [&](const void* src, size_t bytes, void** dst) {
      *dst = nullptr;
      if (bytes == 0) return true;
      if (cudaMalloc(dst, bytes) != cudaSuccess) return false;
      bufs.push_back(*dst);
      return cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice) == cudaSuccess;
    };
    void *nf, *ef, *s, *d;
    const bool ok = put(h.node_feats, sizeof(double) * h.num_nodes * h.node_feat_dim, &nf) &&
                    put(h.edge_feats, sizeof(double) * h.num_edges * h.edge_feat_dim, &ef) &&
                    put(h.srcs, sizeof(uint64_t) * h.num_edges, &s) &&
                    put(h.dsts, sizeof(uint64_t) * h.num_edges, &d);
    g.node_feats = static_cast<const double*>(nf);
    g.edge_feats = static_cast<const double*>(ef);
    g.srcs = static_cast<const uint64_t*>(s);
    g.dsts = static_cast<const uint64_t*>(d);
    return ok;
  }
};

acg_status read_graph(const std::string& arg, bool csv, acg_host_graph* out) {
  if (!csv) return acg_graph_read_bin(arg.c_str(), out);
  const std::string v = arg + ".Vertex.csv", e = arg + ".Edges.csv";
  return acg_graph_read_csv(v.c_str(), e.c_str(), out);
}

}  // namespace

int main(int argc, char** argv) {
  acg_options opt;
  acg_options_default(&opt);
  bool csv = false, binary = false;
  const char* out_path = nullptr;
  std::vector<std::string> pos;
  for (int i = 1; i < argc; ++i) {
    const std::string a = argv[i];
    if (a == "--precision" && i + 1 < argc) {
      const std::string p = argv[++i];
      if (p == "fp64") opt.precision = ACG_PREC_FP64;
      else if (p == "mixed") opt.precision = ACG_PREC_MIXED;
      else return usage();
    } else if (a == "--iters" && i + 1 < argc) {
      opt.num_iters = std::atoi(argv[++i]);
    } else if (a == "--cnull") {
      opt.cnull = 1;
    } else if (a == "--csv") {
      csv = true;
    } else if (a == "--binary") {
      binary = true;
    } else if (a == "--out" && i + 1 < argc) {
      out_path = argv[++i];
    } else if (!a.empty() && a[0] == '-') {
      return usage();
    } else {
      pos.push_back(a);
    }
  }
  if (pos.size() != 2) return usage();
  if (binary && !out_path) {
    std::fprintf(stderr, "acg_main: --binary needs --out\n");
    return 2;
  }

  acg_host_graph hd{}, hp{};
  if (read_graph(pos[0], csv, &hd) != ACG_OK) return fail(pos[0].c_str());
  if (read_graph(pos[1], csv, &hp) != ACG_OK) {
    acg_host_graph_free(&hd);
    return fail(pos[1].c_str());
  }
  const uint64_t rows = hd.num_nodes, cols = hp.num_nodes;
  int rc = 0;
  {
    DeviceGraph dd, dp;
    double* mu = nullptr;
    if (!dd.upload(hd) || !dp.upload(hp) ||
        cudaMalloc(reinterpret_cast<void**>(&mu), sizeof(double) * rows * cols + 8) != cudaSuccess) {
      std::fprintf(stderr, "acg_main: device allocation or copy failed: %s\n",
                   cudaGetErrorString(cudaGetLastError()));
      rc = 1;
    } else {
      cudaDeviceSynchronize();
      const auto t0 = std::chrono::steady_clock::now();
      const acg_status st = acg_match_graphs(&dd.g, &dp.g, &opt, mu, nullptr);
      cudaDeviceSynchronize();
      const auto t1 = std::chrono::steady_clock::now();
      if (st != ACG_OK) {
        rc = fail("match");
      } else {
        std::fprintf(stderr, "elapsed=%lld\n",
                     (long long)std::chrono::duration_cast<std::chrono::microseconds>(t1 - t0).count());
        std::vector<double> h((size_t)(rows * cols));
        if (!h.empty() && cudaMemcpy(h.data(), mu, sizeof(double) * h.size(), cudaMemcpyDeviceToHost) != cudaSuccess) {
          std::fprintf(stderr, "acg_main: copy of mu failed\n");
          rc = 1;
        } else {
          const acg_status w = binary ? acg_mu_write_bin(out_path, h.data(), rows, cols)
                                      : acg_mu_write_text(out_path, h.data(), rows, cols);
          if (w != ACG_OK) rc = fail("write");
        }
      }
    }
    if (mu) cudaFree(mu);
  }
  acg_host_graph_free(&hd);
  acg_host_graph_free(&hp);
  return rc;
}
