// acg_host.cpp -- host-side graph I/O (binary + CSV) and seeded generators.
//
// Binary layout: the reader replaces `loadGraph` (src/main.cu:21-44) with
// every read checked; the writer follows prob2bin.py:42-62.  CSV layout:
// prob2bin.py:11-40 (header "N C", space separated rows, vertex ids equal to
// the row number).
#include <omp.h>

#include <algorithm>
#include <cerrno>
#include <charconv>
#include <cstdio>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "acg_common.h"
#include "acg_io.h"

using acg::set_error;

namespace {

// ---------------------------------------------------------------- RNG
// Counter-based: every draw is a pure function of (seed, stream, index), so
// generated graphs do not depend on how many threads produce them.
inline uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
inline uint64_t draw(uint64_t seed, uint64_t stream, uint64_t i) {
  return mix64(mix64(seed ^ (stream * 0xD1B54A32D192ED03ull)) + i);
}
inline double unif(uint64_t x) {  // (0, 1)
  return ((double)(x >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}
inline uint64_t below(uint64_t x, uint64_t n) {  // x mapped to [0, n)
  return (uint64_t)(((unsigned __int128)x * n) >> 64);
}

enum Stream : uint64_t {
  S_NODE_FEAT = 1,
  S_EDGE_FEAT = 2,
  S_RMAT = 3,
  S_ER = 4,
  S_WALK = 5,
  S_PICK = 6,
  S_NOISE_V = 7,
  S_NOISE_E = 8,
  S_NEW_EDGE = 9,
  S_NEW_FEAT = 10,
  S_FILL = 11,
  S_FILL_FEAT = 12,
};

// Fill x[0..n) with N(0,1) values by Box-Muller over index pairs.
void fill_normal(double* x, uint64_t n, uint64_t seed, uint64_t stream,
                 uint64_t index_base = 0) {
  const double two_pi = 6.283185307179586476925286766559;
  const int64_t npairs = (int64_t)((n + 1) / 2);
#pragma omp parallel for schedule(static)
  for (int64_t p = 0; p < npairs; ++p) {
    const uint64_t g = index_base / 2 + (uint64_t)p;  // pair id
    const double u1 = unif(draw(seed, stream, 2 * g));
    const double u2 = unif(draw(seed, stream, 2 * g + 1));
    const double r = std::sqrt(-2.0 * std::log(u1));
    const double th = two_pi * u2;
    const uint64_t i = 2 * (uint64_t)p;
    x[i] = r * std::cos(th);
    if (i + 1 < n) x[i + 1] = r * std::sin(th);
  }
}

// Stable LSD radix sort of (key, value) pairs on the low `bits` bits.
void radix_sort_pairs(std::vector<uint64_t>& k, std::vector<uint64_t>& v,
                      int bits) {
  const size_t n = k.size();
  std::vector<uint64_t> k2(n), v2(n);
  const int maxt = omp_get_max_threads();
  std::vector<size_t> hist((size_t)maxt * 256);
  for (int shift = 0; shift < bits; shift += 8) {
#pragma omp parallel
    {
      const int nt = omp_get_num_threads();
      const int t = omp_get_thread_num();
      const size_t lo = n * (size_t)t / nt, hi = n * (size_t)(t + 1) / nt;
      size_t* h = &hist[(size_t)t * 256];
      std::fill(h, h + 256, 0);
      for (size_t i = lo; i < hi; ++i) h[(k[i] >> shift) & 255]++;
#pragma omp barrier
#pragma omp single
      {
        size_t sum = 0;
        for (int d = 0; d < 256; ++d)
          for (int tt = 0; tt < nt; ++tt) {
            size_t c = hist[(size_t)tt * 256 + d];
            hist[(size_t)tt * 256 + d] = sum;
            sum += c;
          }
      }
      for (size_t i = lo; i < hi; ++i) {
        size_t pos = h[(k[i] >> shift) & 255]++;
        k2[pos] = k[i];
        v2[pos] = v[i];
      }
    }
    k.swap(k2);
    v.swap(v2);
  }
}

acg_status reserve_edges(acg_host_graph* g, uint64_t cap) {
  if (cap <= g->edge_capacity) return ACG_OK;
  const uint64_t ke = g->edge_feat_dim;
  double* ef = (double*)std::realloc(g->edge_feats, sizeof(double) * (ke ? cap * ke : 1));
  if (!ef) return set_error(ACG_ERR_OUT_OF_MEMORY, "reserve_edges: realloc failed");
  g->edge_feats = ef;
  uint64_t* s = (uint64_t*)std::realloc(g->srcs, sizeof(uint64_t) * cap);
  if (!s) return set_error(ACG_ERR_OUT_OF_MEMORY, "reserve_edges: realloc failed");
  g->srcs = s;
  uint64_t* d = (uint64_t*)std::realloc(g->dsts, sizeof(uint64_t) * cap);
  if (!d) return set_error(ACG_ERR_OUT_OF_MEMORY, "reserve_edges: realloc failed");
  g->dsts = d;
  g->edge_capacity = cap;
  return ACG_OK;
}

acg_status grow_edges(acg_host_graph* g, uint64_t new_m) {
  if (new_m <= g->num_edges) return ACG_OK;
  if (new_m <= g->edge_capacity) {
    g->num_edges = new_m;
    return ACG_OK;
  }
  const uint64_t ke = g->edge_feat_dim;
  double* ef = (double*)std::realloc(g->edge_feats, sizeof(double) * (ke ? new_m * ke : 1));
  if (!ef) return set_error(ACG_ERR_OUT_OF_MEMORY, "grow_edges: realloc failed");
  g->edge_feats = ef;
  uint64_t* s = (uint64_t*)std::realloc(g->srcs, sizeof(uint64_t) * new_m);
  if (!s) return set_error(ACG_ERR_OUT_OF_MEMORY, "grow_edges: realloc failed");
  g->srcs = s;
  uint64_t* d = (uint64_t*)std::realloc(g->dsts, sizeof(uint64_t) * new_m);
  if (!d) return set_error(ACG_ERR_OUT_OF_MEMORY, "grow_edges: realloc failed");
  g->dsts = d;
  g->num_edges = new_m;
  g->edge_capacity = new_m;
  return ACG_OK;
}

struct FileCloser {
  FILE* f;
  ~FileCloser() {
    if (f) std::fclose(f);
  }
};

}  // namespace

extern "C" {

acg_status acg_host_graph_alloc(acg_host_graph* g, uint64_t nv, uint64_t kv,
                                uint64_t ne, uint64_t ke) {
  if (!g) return set_error(ACG_ERR_INVALID_ARGUMENT, "acg_host_graph_alloc: null graph");
  acg_host_graph_free(g);
  g->num_nodes = nv;
  g->node_feat_dim = kv;
  g->num_edges = ne;
  g->edge_feat_dim = ke;
  g->node_feats = (double*)std::calloc((nv * kv) != 0 ? nv * kv : 1, sizeof(double));
  g->edge_feats = (double*)std::calloc((ne * ke) != 0 ? ne * ke : 1, sizeof(double));
  g->srcs = (uint64_t*)std::calloc(ne ? ne : 1, sizeof(uint64_t));
  g->dsts = (uint64_t*)std::calloc(ne ? ne : 1, sizeof(uint64_t));
  g->edge_capacity = ne;
  if (!g->node_feats || !g->edge_feats || !g->srcs || !g->dsts) {
    acg_host_graph_free(g);
    return set_error(ACG_ERR_OUT_OF_MEMORY, "acg_host_graph_alloc: calloc failed");
  }
  return ACG_OK;
}

void acg_host_graph_free(acg_host_graph* g) {
  if (!g) return;
  std::free(g->node_feats);
  std::free(g->edge_feats);
  std::free(g->srcs);
  std::free(g->dsts);
  std::memset(g, 0, sizeof *g);
}

acg_graph acg_host_graph_view(const acg_host_graph* g) {
  acg_graph v;
  v.num_nodes = g->num_nodes;
  v.node_feat_dim = g->node_feat_dim;
  v.num_edges = g->num_edges;
  v.edge_feat_dim = g->edge_feat_dim;
  v.node_feats = g->node_feats;
  v.edge_feats = g->edge_feats;
  v.srcs = g->srcs;
  v.dsts = g->dsts;
  return v;
}

// ------------------------------------------------------------ binary I/O
acg_status acg_graph_read_bin(const char* path, acg_host_graph* out) {
  if (!path || !out) return set_error(ACG_ERR_INVALID_ARGUMENT, "acg_graph_read_bin: null argument");
  FileCloser fc{std::fopen(path, "rb")};
  if (!fc.f) return set_error(ACG_ERR_IO, "cannot open %s: %s", path, std::strerror(errno));
  uint64_t hdr[4];
  if (std::fread(hdr, sizeof(uint64_t), 4, fc.f) != 4)
    return set_error(ACG_ERR_IO, "%s: truncated header", path);
  const uint64_t nv = hdr[0], kv = hdr[1], ne = hdr[2], ke = hdr[3];
  std::fseek(fc.f, 0, SEEK_END);
  const long long fsize = std::ftell(fc.f);
  std::fseek(fc.f, 32, SEEK_SET);
  const unsigned __int128 want =
      (unsigned __int128)32 + 8 * ((unsigned __int128)nv * kv + (unsigned __int128)ne * ke + 2 * (unsigned __int128)ne);
  if (fsize < 0 || want != (unsigned __int128)fsize)
    return set_error(ACG_ERR_IO,
                     "%s: header says %llu nodes x %llu, %llu edges x %llu but the file has %lld bytes",
                     path, (unsigned long long)nv, (unsigned long long)kv, (unsigned long long)ne,
                     (unsigned long long)ke, fsize);
  ACG_TRY(acg_host_graph_alloc(out, nv, kv, ne, ke));
  if (std::fread(out->node_feats, sizeof(double), nv * kv, fc.f) != nv * kv ||
      std::fread(out->edge_feats, sizeof(double), ne * ke, fc.f) != ne * ke ||
      std::fread(out->srcs, sizeof(uint64_t), ne, fc.f) != ne ||
      std::fread(out->dsts, sizeof(uint64_t), ne, fc.f) != ne) {
    acg_host_graph_free(out);
    return set_error(ACG_ERR_IO, "%s: short read", path);
  }
  return ACG_OK;
}

acg_status acg_graph_write_bin(const char* path, const acg_host_graph* g) {
  if (!path || !g) return set_error(ACG_ERR_INVALID_ARGUMENT, "acg_graph_write_bin: null argument");
  FileCloser fc{std::fopen(path, "wb")};
  if (!fc.f) return set_error(ACG_ERR_IO, "cannot create %s: %s", path, std::strerror(errno));
  const uint64_t hdr[4] = {g->num_nodes, g->node_feat_dim, g->num_edges, g->edge_feat_dim};
  const uint64_t nvk = g->num_nodes * g->node_feat_dim, nek = g->num_edges * g->edge_feat_dim;
  if (std::fwrite(hdr, sizeof(uint64_t), 4, fc.f) != 4 ||
      std::fwrite(g->node_feats, sizeof(double), nvk, fc.f) != nvk ||
      std::fwrite(g->edge_feats, sizeof(double), nek, fc.f) != nek ||
      std::fwrite(g->srcs, sizeof(uint64_t), g->num_edges, fc.f) != g->num_edges ||
      std::fwrite(g->dsts, sizeof(uint64_t), g->num_edges, fc.f) != g->num_edges)
    return set_error(ACG_ERR_IO, "%s: short write", path);
  if (std::fflush(fc.f) != 0) return set_error(ACG_ERR_IO, "%s: flush failed", path);
  return ACG_OK;
}

// --------------------------------------------------------------- CSV I/O
namespace {

struct CsvReader {
  std::vector<char> buf;
  const char* p = nullptr;
  const char* end = nullptr;

  acg_status load(const char* path) {
    FileCloser fc{std::fopen(path, "rb")};
    if (!fc.f) return set_error(ACG_ERR_IO, "cannot open %s: %s", path, std::strerror(errno));
    std::fseek(fc.f, 0, SEEK_END);
    long n = std::ftell(fc.f);
    std::fseek(fc.f, 0, SEEK_SET);
    if (n < 0) return set_error(ACG_ERR_IO, "%s: cannot size", path);
    buf.resize((size_t)n + 1);
    if (n && std::fread(buf.data(), 1, (size_t)n, fc.f) != (size_t)n)
      return set_error(ACG_ERR_IO, "%s: short read", path);
    buf[(size_t)n] = '\0';
    p = buf.data();
    end = buf.data() + n;
    return ACG_OK;
  }
  void skip_blank() {
    while (p < end && (*p == ' ' || *p == '\t' || *p == '\r')) ++p;
  }
  bool at_eol() {
    skip_blank();
    return p >= end || *p == '\n';
  }
  void next_line() {
    while (p < end && *p != '\n') ++p;
    if (p < end) ++p;
  }
  bool number(double* x) {
    skip_blank();
    if (p >= end || *p == '\n') return false;
    char* e = nullptr;
    *x = std::strtod(p, &e);
    if (e == p) return false;
    p = e;
    return true;
  }
};

// Reads an integer-valued field written either as "12" or "12.0".
bool as_index(double x, uint64_t* out) {
  if (!(x >= 0.0) || x != std::floor(x) || x > 18446744073709549568.0) return false;
  *out = (uint64_t)x;
  return true;
}

acg_status read_header(CsvReader& r, const char* path, uint64_t* rows, uint64_t* cols) {
  double a, b;
  if (!r.number(&a) || !r.number(&b) || !as_index(a, rows) || !as_index(b, cols) || !r.at_eol())
    return set_error(ACG_ERR_IO, "%s: bad header (want \"N C\")", path);
  r.next_line();
  return ACG_OK;
}

}  // namespace

acg_status acg_graph_read_csv(const char* vertex_csv, const char* edges_csv,
                              acg_host_graph* out) {
  if (!vertex_csv || !out) return set_error(ACG_ERR_INVALID_ARGUMENT, "acg_graph_read_csv: null argument");
  CsvReader rv;
  ACG_TRY(rv.load(vertex_csv));
  uint64_t nv, cv;
  ACG_TRY(read_header(rv, vertex_csv, &nv, &cv));
  if (cv < 1) return set_error(ACG_ERR_IO, "%s: need at least the id column", vertex_csv);
  const uint64_t kv = cv - 1;

  CsvReader re;
  uint64_t ne = 0, ce = 2;
  if (edges_csv) {
    ACG_TRY(re.load(edges_csv));
    ACG_TRY(read_header(re, edges_csv, &ne, &ce));
    if (ce < 2) return set_error(ACG_ERR_IO, "%s: need src and dst columns", edges_csv);
  }
  const uint64_t ke = ce - 2;
  ACG_TRY(acg_host_graph_alloc(out, nv, kv, ne, ke));

  for (uint64_t i = 0; i < nv; ++i) {
    double x;
    uint64_t id;
    if (!rv.number(&x) || !as_index(x, &id)) {
      acg_host_graph_free(out);
      return set_error(ACG_ERR_IO, "%s: row %llu: bad id", vertex_csv, (unsigned long long)i);
    }
    if (id != i) {  // prob2bin.py:28-29
      acg_host_graph_free(out);
      return set_error(ACG_ERR_IO, "%s: row %llu has id %llu (ids must equal the row number)",
                       vertex_csv, (unsigned long long)i, (unsigned long long)id);
    }
    for (uint64_t k = 0; k < kv; ++k)
      if (!rv.number(&out->node_feats[i * kv + k])) {
        acg_host_graph_free(out);
        return set_error(ACG_ERR_IO, "%s: row %llu: expected %llu features", vertex_csv,
                         (unsigned long long)i, (unsigned long long)kv);
      }
    if (!rv.at_eol()) {
      acg_host_graph_free(out);
      return set_error(ACG_ERR_IO, "%s: row %llu: extra columns", vertex_csv, (unsigned long long)i);
    }
    rv.next_line();
  }
  for (uint64_t j = 0; j < ne; ++j) {
    double s, d;
    if (!re.number(&s) || !re.number(&d) || !as_index(s, &out->srcs[j]) || !as_index(d, &out->dsts[j])) {
      acg_host_graph_free(out);
      return set_error(ACG_ERR_IO, "%s: row %llu: bad src/dst", edges_csv, (unsigned long long)j);
    }
    for (uint64_t k = 0; k < ke; ++k)
      if (!re.number(&out->edge_feats[j * ke + k])) {
        acg_host_graph_free(out);
        return set_error(ACG_ERR_IO, "%s: row %llu: expected %llu features", edges_csv,
                         (unsigned long long)j, (unsigned long long)ke);
      }
    if (!re.at_eol()) {
      acg_host_graph_free(out);
      return set_error(ACG_ERR_IO, "%s: row %llu: extra columns", edges_csv, (unsigned long long)j);
    }
    re.next_line();
  }
  return ACG_OK;
}

acg_status acg_graph_write_csv(const char* vertex_csv, const char* edges_csv,
                               const acg_host_graph* g) {
  if (!vertex_csv || !g) return set_error(ACG_ERR_INVALID_ARGUMENT, "acg_graph_write_csv: null argument");
  {
    FileCloser fc{std::fopen(vertex_csv, "wb")};
    if (!fc.f) return set_error(ACG_ERR_IO, "cannot create %s", vertex_csv);
    std::fprintf(fc.f, "%llu %llu\n", (unsigned long long)g->num_nodes,
                 (unsigned long long)(g->node_feat_dim + 1));
    for (uint64_t i = 0; i < g->num_nodes; ++i) {
      std::fprintf(fc.f, "%llu", (unsigned long long)i);
      for (uint64_t k = 0; k < g->node_feat_dim; ++k)
        std::fprintf(fc.f, " %.17g", g->node_feats[i * g->node_feat_dim + k]);
      std::fputc('\n', fc.f);
    }
    if (std::ferror(fc.f)) return set_error(ACG_ERR_IO, "%s: write failed", vertex_csv);
  }
  if (edges_csv) {
    FileCloser fc{std::fopen(edges_csv, "wb")};
    if (!fc.f) return set_error(ACG_ERR_IO, "cannot create %s", edges_csv);
    std::fprintf(fc.f, "%llu %llu\n", (unsigned long long)g->num_edges,
                 (unsigned long long)(g->edge_feat_dim + 2));
    for (uint64_t j = 0; j < g->num_edges; ++j) {
      std::fprintf(fc.f, "%llu %llu", (unsigned long long)g->srcs[j], (unsigned long long)g->dsts[j]);
      for (uint64_t k = 0; k < g->edge_feat_dim; ++k)
        std::fprintf(fc.f, " %.17g", g->edge_feats[j * g->edge_feat_dim + k]);
      std::fputc('\n', fc.f);
    }
    if (std::ferror(fc.f)) return set_error(ACG_ERR_IO, "%s: write failed", edges_csv);
  }
  return ACG_OK;
}

// ------------------------------------------------------------ generators
acg_status acg_gen_er(uint64_t n, uint64_t m, uint64_t kv, uint64_t ke,
                      uint64_t seed, acg_host_graph* out) {
  if (!out) return set_error(ACG_ERR_INVALID_ARGUMENT, "acg_gen_er: null graph");
  if (n == 0 || n > (1ull << 31) || (n > 1 && m > n * (n - 1)) || (n == 1 && m > 0))
    return set_error(ACG_ERR_INVALID_ARGUMENT, "acg_gen_er: %llu edges do not fit %llu vertices",
                     (unsigned long long)m, (unsigned long long)n);
  ACG_TRY(acg_host_graph_alloc(out, n, kv, m, ke));
  std::unordered_set<uint64_t> seen;
  seen.reserve(m * 2 + 16);
  uint64_t k = 0;
  for (uint64_t j = 0; j < m;) {
    const uint64_t x = draw(seed, S_ER, k++);
    const uint64_t u = below(x, n), v = below(mix64(x), n);
    if (u == v) continue;
    if (!seen.insert(u * n + v).second) continue;
    out->srcs[j] = u;
    out->dsts[j] = v;
    ++j;
  }
  fill_normal(out->node_feats, n * kv, seed, S_NODE_FEAT);
  fill_normal(out->edge_feats, m * ke, seed, S_EDGE_FEAT);
  return reserve_edges(out, m + ACG_EDGE_RESERVE);
}

acg_status acg_gen_rmat(int scale, int edge_factor, double a, double b, double c,
                        uint64_t kv, uint64_t ke, uint64_t seed, acg_host_graph* out) {
  if (!out) return set_error(ACG_ERR_INVALID_ARGUMENT, "acg_gen_rmat: null graph");
  if (scale < 1 || scale > 30 || edge_factor < 1 || a < 0 || b < 0 || c < 0 || a + b + c > 1.0)
    return set_error(ACG_ERR_INVALID_ARGUMENT, "acg_gen_rmat: bad parameters");
  const uint64_t n = 1ull << scale;
  const uint64_t m0 = (uint64_t)edge_factor << scale;
  const double ab = a + b, abc = a + b + c;
  std::vector<uint64_t> key(m0), idx(m0);
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < (int64_t)m0; ++e) {
    uint64_t u = 0, v = 0;
    for (int l = 0; l < scale; ++l) {
      const double r = unif(draw(seed, S_RMAT, (uint64_t)e * (uint64_t)scale + (uint64_t)l));
      const uint64_t bit = 1ull << (scale - 1 - l);
      if (r < a) {
      } else if (r < ab) {
        v |= bit;
      } else if (r < abc) {
        u |= bit;
      } else {
        u |= bit;
        v |= bit;
      }
    }
    key[(size_t)e] = (u << scale) | v;
    idx[(size_t)e] = (uint64_t)e;
  }
  // Dedup keeping first occurrences, then emit in sampling order.
  radix_sort_pairs(key, idx, 2 * scale);
  std::vector<uint8_t> keep(m0, 0);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)m0; ++i) {
    const uint64_t k = key[(size_t)i];
    const uint64_t u = k >> scale, v = k & (n - 1);
    if (u == v) continue;
    if (i > 0 && key[(size_t)i - 1] == k) continue;  // stable: first occurrence first
    keep[idx[(size_t)i]] = 1;
  }
  std::vector<uint64_t> kept_key;
  // the key of sampled edge e, recomputed from the sorted arrays
  std::vector<uint64_t> key_of(m0);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)m0; ++i) key_of[idx[(size_t)i]] = key[(size_t)i];
  uint64_t m = 0;
  for (uint64_t e = 0; e < m0; ++e) m += keep[e];
  ACG_TRY(acg_host_graph_alloc(out, n, kv, m, ke));
  uint64_t j = 0;
  for (uint64_t e = 0; e < m0; ++e)
    if (keep[e]) {
      out->srcs[j] = key_of[e] >> scale;
      out->dsts[j] = key_of[e] & (n - 1);
      ++j;
    }
  fill_normal(out->node_feats, n * kv, seed, S_NODE_FEAT);
  fill_normal(out->edge_feats, m * ke, seed, S_EDGE_FEAT);
  return reserve_edges(out, m + ACG_EDGE_RESERVE);
}

acg_status acg_gen_fill_edges(acg_host_graph* g, uint64_t m, uint64_t seed) {
  if (!g) return set_error(ACG_ERR_INVALID_ARGUMENT, "acg_gen_fill_edges: null graph");
  const uint64_t n = g->num_nodes;
  if (m <= g->num_edges) return ACG_OK;
  if (n < 2 || m > n * (n - 1))
    return set_error(ACG_ERR_INVALID_ARGUMENT, "acg_gen_fill_edges: %llu edges do not fit",
                     (unsigned long long)m);
  std::unordered_set<uint64_t> seen;
  seen.reserve(m * 2 + 16);
  for (uint64_t j = 0; j < g->num_edges; ++j) seen.insert(g->srcs[j] * n + g->dsts[j]);
  uint64_t j = g->num_edges;
  ACG_TRY(grow_edges(g, m));
  uint64_t k = 0;
  while (j < m) {
    const uint64_t x = draw(seed, S_FILL, k++);
    const uint64_t u = below(x, n), v = below(mix64(x), n);
    if (u == v || !seen.insert(u * n + v).second) continue;
    g->srcs[j] = u;
    g->dsts[j] = v;
    fill_normal(g->edge_feats + j * g->edge_feat_dim, g->edge_feat_dim, seed, S_FILL_FEAT,
                2 * j * g->edge_feat_dim);
    ++j;
  }
  return ACG_OK;
}

acg_status acg_gen_plant(acg_host_graph* data, uint64_t pn, uint64_t pe, double noise,
                         uint64_t seed, acg_host_graph* pattern, uint64_t* truth_vertex,
                         uint64_t* truth_edge) {
  if (!data || !pattern) return set_error(ACG_ERR_INVALID_ARGUMENT, "acg_gen_plant: null graph");
  const uint64_t n = data->num_nodes;
  if (pn == 0 || pn > n) return set_error(ACG_ERR_INVALID_ARGUMENT, "acg_gen_plant: bad pattern size");
  if (pe > pn * (pn - 1))
    return set_error(ACG_ERR_INVALID_ARGUMENT, "acg_gen_plant: %llu edges do not fit %llu vertices",
                     (unsigned long long)pe, (unsigned long long)pn);
  const uint64_t m = data->num_edges;

  // Undirected incidence lists: (neighbour, edge id) for both endpoints.
  std::vector<uint64_t> off(n + 1, 0);
  for (uint64_t e = 0; e < m; ++e) {
    off[data->srcs[e] + 1]++;
    off[data->dsts[e] + 1]++;
  }
  for (uint64_t v = 0; v < n; ++v) off[v + 1] += off[v];
  std::vector<uint64_t> nbr(2 * m), eid(2 * m), cur(off.begin(), off.end() - 1);
  for (uint64_t e = 0; e < m; ++e) {
    const uint64_t u = data->srcs[e], v = data->dsts[e];
    nbr[cur[u]] = v;
    eid[cur[u]++] = e;
    nbr[cur[v]] = u;
    eid[cur[v]++] = e;
  }

  // Random-walk growth of a weakly connected vertex set.
  std::vector<uint64_t> S, tree;
  std::unordered_map<uint64_t, uint64_t> pos;  // data vertex -> index in S
  uint64_t ctr = 0;
  for (int attempt = 0; attempt < 64 && S.size() < pn; ++attempt) {
    std::vector<uint64_t> s2, t2;
    std::unordered_map<uint64_t, uint64_t> p2;
    uint64_t start = m ? data->srcs[below(draw(seed, S_WALK, ctr++), m)]
                       : below(draw(seed, S_WALK, ctr++), n);
    s2.push_back(start);
    p2[start] = 0;
    for (uint64_t tries = 0; s2.size() < pn && tries < 400 * pn; ++tries) {
      const uint64_t u = s2[below(draw(seed, S_WALK, ctr++), s2.size())];
      const uint64_t deg = off[u + 1] - off[u];
      if (!deg) continue;
      const uint64_t k = off[u] + below(draw(seed, S_WALK, ctr++), deg);
      const uint64_t w = nbr[k];
      if (p2.count(w)) continue;
      p2[w] = s2.size();
      s2.push_back(w);
      t2.push_back(eid[k]);
    }
    if (s2.size() > S.size()) {
      S.swap(s2);
      tree.swap(t2);
      pos.swap(p2);
    }
  }
  // Still short (tiny components): connect fresh vertices with new edges.
  std::vector<std::pair<uint64_t, uint64_t>> new_edges;  // (src, dst) to append
  std::vector<int64_t> chosen;                          // >=0 data edge, <0 new edge -(k+1)
  while (S.size() < pn) {
    const uint64_t w = below(draw(seed, S_NEW_EDGE, ctr++), n);
    if (pos.count(w)) continue;
    const uint64_t u = S[below(draw(seed, S_NEW_EDGE, ctr++), S.size())];
    pos[w] = S.size();
    S.push_back(w);
    new_edges.push_back({u, w});
    chosen.push_back(-(int64_t)new_edges.size());
  }
  for (uint64_t e : tree) chosen.push_back((int64_t)e);
  if (chosen.size() > pe) chosen.resize(pe);

  // Induced data edges not yet chosen, in random order.
  std::unordered_set<uint64_t> have;  // (src,dst) keys among S, existing or chosen
  std::unordered_set<int64_t> taken(chosen.begin(), chosen.end());
  std::vector<uint64_t> extra;
  for (uint64_t u : S)
    for (uint64_t k = off[u]; k < off[u + 1]; ++k) {
      const uint64_t e = eid[k];
      if (data->srcs[e] != u || !pos.count(nbr[k]) || nbr[k] == u) continue;
      have.insert(u * n + nbr[k]);
      if (!taken.count((int64_t)e)) extra.push_back(e);
    }
  std::sort(extra.begin(), extra.end());
  extra.erase(std::unique(extra.begin(), extra.end()), extra.end());
  for (uint64_t i = extra.size(); i > 1; --i) std::swap(extra[i - 1], extra[below(draw(seed, S_PICK, i), i)]);
  for (size_t i = 0; i < extra.size() && chosen.size() < pe; ++i) chosen.push_back((int64_t)extra[i]);
  for (auto& ne : new_edges) have.insert(ne.first * n + ne.second);
  while (chosen.size() < pe) {  // plant new edges among S
    const uint64_t u = S[below(draw(seed, S_NEW_EDGE, ctr++), pn)];
    const uint64_t v = S[below(draw(seed, S_NEW_EDGE, ctr++), pn)];
    if (u == v || !have.insert(u * n + v).second) continue;
    new_edges.push_back({u, v});
    chosen.push_back(-(int64_t)new_edges.size());
  }

  // Append new data edges with fresh features.
  const uint64_t ke = data->edge_feat_dim;
  const uint64_t m_old = data->num_edges;
  if (!new_edges.empty()) {
    ACG_TRY(grow_edges(data, m_old + new_edges.size()));
    for (size_t i = 0; i < new_edges.size(); ++i) {
      data->srcs[m_old + i] = new_edges[i].first;
      data->dsts[m_old + i] = new_edges[i].second;
    }
    fill_normal(data->edge_feats + m_old * ke, new_edges.size() * ke, seed ^ m_old, S_NEW_FEAT);
  }
  std::vector<uint64_t> pedge(chosen.size());
  for (size_t j = 0; j < chosen.size(); ++j)
    pedge[j] = chosen[j] >= 0 ? (uint64_t)chosen[j] : m_old + (uint64_t)(-chosen[j] - 1);
  for (uint64_t i = pedge.size(); i > 1; --i) std::swap(pedge[i - 1], pedge[below(draw(seed, S_PICK, 1000003 + i), i)]);

  // Relabel by a random permutation and copy features with noise.
  std::vector<uint64_t> perm(pn);
  for (uint64_t i = 0; i < pn; ++i) perm[i] = i;
  for (uint64_t i = pn; i > 1; --i) std::swap(perm[i - 1], perm[below(draw(seed, S_PICK, 2000003 + i), i)]);
  std::unordered_map<uint64_t, uint64_t> label;
  for (uint64_t i = 0; i < pn; ++i) label[S[perm[i]]] = i;

  const uint64_t kv = data->node_feat_dim;
  ACG_TRY(acg_host_graph_alloc(pattern, pn, kv, pedge.size(), ke));
  fill_normal(pattern->node_feats, pn * kv, seed, S_NOISE_V);
  fill_normal(pattern->edge_feats, pedge.size() * ke, seed, S_NOISE_E);
  for (uint64_t i = 0; i < pn; ++i) {
    const uint64_t dv = S[perm[i]];
    if (truth_vertex) truth_vertex[i] = dv;
    for (uint64_t k = 0; k < kv; ++k)
      pattern->node_feats[i * kv + k] = data->node_feats[dv * kv + k] + noise * pattern->node_feats[i * kv + k];
  }
  for (size_t j = 0; j < pedge.size(); ++j) {
    const uint64_t e = pedge[j];
    if (truth_edge) truth_edge[j] = e;
    pattern->srcs[j] = label[data->srcs[e]];
    pattern->dsts[j] = label[data->dsts[e]];
    for (uint64_t k = 0; k < ke; ++k)
      pattern->edge_feats[j * ke + k] = data->edge_feats[e * ke + k] + noise * pattern->edge_feats[j * ke + k];
  }
  return ACG_OK;
}

// ---------------------------------------------------------------- mu output
// The reference prints MU with printf("%e\n") per entry, row-major
// (main.cu:255-257).  std::to_chars with the scientific format and precision 6
// produces the same characters as "%e" (a correctly rounded decimal, at least
// two exponent digits, "inf"/"nan" spelled the same); blocks of entries are
// formatted in parallel and written in order.
acg_status acg_mu_write_text(const char* path, const double* mu, uint64_t rows, uint64_t cols) {
  acg::clear_error();
  const uint64_t n = rows * cols;
  if (n && !mu) return acg::set_error(ACG_ERR_INVALID_ARGUMENT, "acg_mu_write_text: mu is null");
  FILE* f = path ? std::fopen(path, "wb") : stdout;
  if (!f) return acg::set_error(ACG_ERR_IO, "cannot open %s: %s", path, std::strerror(errno));
  constexpr uint64_t kBlock = 1 << 22;  // entries per block
  constexpr int kMaxChars = 32;         // "-1.234568e+308\n" and the like
  const int nt = std::max(1, omp_get_max_threads());
  std::vector<char> buf((size_t)std::min<uint64_t>(n, kBlock) * kMaxChars + 1);
  std::vector<size_t> len((size_t)nt + 1);
  acg_status st = ACG_OK;
  for (uint64_t b0 = 0; b0 < n && st == ACG_OK; b0 += kBlock) {
    const uint64_t bn = std::min<uint64_t>(kBlock, n - b0);
#pragma omp parallel num_threads(nt)
    {
      const int t = omp_get_thread_num(), T = omp_get_num_threads();
      const uint64_t i0 = bn * t / T, i1 = bn * (t + 1) / T;
      char* o = buf.data() + i0 * kMaxChars;
      char* p = o;
      for (uint64_t i = i0; i < i1; ++i) {
        auto r = std::to_chars(p, p + kMaxChars - 1, mu[b0 + i], std::chars_format::scientific, 6);
        p = r.ptr;
        *p++ = '\n';
      }
      len[(size_t)t] = (size_t)(p - o);
#pragma omp barrier
#pragma omp single
      {
        for (int u = 0; u < T && st == ACG_OK; ++u) {
          const uint64_t j0 = bn * u / T;
          const size_t L = len[(size_t)u];
          if (L && std::fwrite(buf.data() + j0 * kMaxChars, 1, L, f) != L)
            st = acg::set_error(ACG_ERR_IO, "write failed");
        }
      }
    }
  }
  if (path) {
    if (std::fclose(f) != 0 && st == ACG_OK) st = acg::set_error(ACG_ERR_IO, "close failed");
  } else {
    std::fflush(f);
  }
  return st;
}

acg_status acg_mu_write_bin(const char* path, const double* mu, uint64_t rows, uint64_t cols) {
  acg::clear_error();
  const uint64_t n = rows * cols;
  if (!path) return acg::set_error(ACG_ERR_INVALID_ARGUMENT, "acg_mu_write_bin: path is null");
  if (n && !mu) return acg::set_error(ACG_ERR_INVALID_ARGUMENT, "acg_mu_write_bin: mu is null");
  FILE* f = std::fopen(path, "wb");
  if (!f) return acg::set_error(ACG_ERR_IO, "cannot open %s: %s", path, std::strerror(errno));
  const size_t w = n ? std::fwrite(mu, sizeof(double), (size_t)n, f) : 0;
  const int c = std::fclose(f);
  if (w != n || c != 0) return acg::set_error(ACG_ERR_IO, "write to %s failed", path);
  return ACG_OK;
}

}  // extern "C"
