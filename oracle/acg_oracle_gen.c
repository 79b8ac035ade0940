/*
 * acg_oracle_gen.c -- TEST INFRASTRUCTURE: seeded synthetic workloads for the
 * CPU legs (the oracle checks and the CPU baseline), independent of the
 * product library.
 *
 * A restatement, in plain C, of the generators the matcher's benchmark and
 * tests use (R-MAT and Erdos-Renyi data graphs with N(0,1) features, a planted
 * pattern, random top-up edges): the same counter-based random stream, the
 * same sampling rules, so that a graph made here is byte-for-byte the graph
 * the product's generator makes for the same arguments (tests/test_oracle_gen.py
 * checks this).  The CPU baseline can then build its workload without loading
 * the product library.
 *
 * Random numbers: every draw is mix64(mix64(seed ^ stream * C) + index) (the
 * splitmix64 finaliser), so no value depends on the order it is computed in.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "acg_oracle_gen.h"

enum {
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
  S_FILL_FEAT = 12
};

static uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static uint64_t draw(uint64_t seed, uint64_t stream, uint64_t i) {
  return mix64(mix64(seed ^ (stream * 0xD1B54A32D192ED03ull)) + i);
}
static double unif(uint64_t x) { return ((double)(x >> 11) + 0.5) * (1.0 / 9007199254740992.0); }
static uint64_t below(uint64_t x, uint64_t n) { return (uint64_t)(((unsigned __int128)x * n) >> 64); }

/* N(0,1) values by Box-Muller over index pairs (pair g from draws 2g, 2g+1). */
static void fill_normal(double* x, uint64_t n, uint64_t seed, uint64_t stream, uint64_t index_base) {
  const double two_pi = 6.283185307179586476925286766559;
  const int64_t npairs = (int64_t)((n + 1) / 2);
#pragma omp parallel for schedule(static)
  for (int64_t p = 0; p < npairs; ++p) {
    const uint64_t g = index_base / 2 + (uint64_t)p;
    const double u1 = unif(draw(seed, stream, 2 * g));
    const double u2 = unif(draw(seed, stream, 2 * g + 1));
    const double r = sqrt(-2.0 * log(u1));
    const double th = two_pi * u2;
    const uint64_t i = 2 * (uint64_t)p;
    x[i] = r * cos(th);
    if (i + 1 < n) x[i + 1] = r * sin(th);
  }
}

/* ---- an open-addressing set of 64-bit keys (UINT64_MAX is the empty slot) */
typedef struct {
  uint64_t* slot;
  uint64_t mask;
  uint64_t count;
} kset;

static int kset_init(kset* s, uint64_t expect) {
  uint64_t cap = 16;
  while (cap < 2 * expect + 16) cap <<= 1;
  s->slot = (uint64_t*)malloc(sizeof(uint64_t) * cap);
  if (!s->slot) return 2;
  memset(s->slot, 0xff, sizeof(uint64_t) * cap);
  s->mask = cap - 1;
  s->count = 0;
  return 0;
}
static void kset_free(kset* s) {
  free(s->slot);
  s->slot = NULL;
}
static int kset_grow(kset* s) {
  kset t;
  if (kset_init(&t, 2 * (s->mask + 1))) return 2;
  for (uint64_t i = 0; i <= s->mask; ++i) {
    const uint64_t k = s->slot[i];
    if (k == UINT64_MAX) continue;
    uint64_t h = mix64(k) & t.mask;
    while (t.slot[h] != UINT64_MAX) h = (h + 1) & t.mask;
    t.slot[h] = k;
    t.count++;
  }
  free(s->slot);
  *s = t;
  return 0;
}
static int kset_has(const kset* s, uint64_t k) {
  uint64_t h = mix64(k) & s->mask;
  while (s->slot[h] != UINT64_MAX) {
    if (s->slot[h] == k) return 1;
    h = (h + 1) & s->mask;
  }
  return 0;
}
/* 1 if k was inserted, 0 if present, -1 out of memory */
static int kset_insert(kset* s, uint64_t k) {
  if (2 * (s->count + 1) > s->mask + 1 && kset_grow(s)) return -1;
  uint64_t h = mix64(k) & s->mask;
  while (s->slot[h] != UINT64_MAX) {
    if (s->slot[h] == k) return 0;
    h = (h + 1) & s->mask;
  }
  s->slot[h] = k;
  s->count++;
  return 1;
}

/* ---- growable u64 / i64 lists */
typedef struct {
  uint64_t* v;
  uint64_t n, cap;
} ulist;
static int ul_push(ulist* l, uint64_t x) {
  if (l->n == l->cap) {
    const uint64_t c = l->cap ? 2 * l->cap : 16;
    uint64_t* p = (uint64_t*)realloc(l->v, sizeof(uint64_t) * c);
    if (!p) return 2;
    l->v = p;
    l->cap = c;
  }
  l->v[l->n++] = x;
  return 0;
}
static int ul_has(const ulist* l, uint64_t x) {
  for (uint64_t i = 0; i < l->n; ++i)
    if (l->v[i] == x) return 1;
  return 0;
}
static void ul_free(ulist* l) {
  free(l->v);
  l->v = NULL;
  l->n = l->cap = 0;
}
static void ul_swap(ulist* a, ulist* b) {
  ulist t = *a;
  *a = *b;
  *b = t;
}

static int cmp_u64(const void* a, const void* b) {
  const uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
  return x < y ? -1 : (x > y);
}

void acgo_free(acgo_graph* g) {
  if (!g) return;
  free(g->node_feats);
  free(g->edge_feats);
  free(g->srcs);
  free(g->dsts);
  memset(g, 0, sizeof *g);
}

static int alloc_graph(acgo_graph* g, uint64_t n, uint64_t kv, uint64_t m, uint64_t ke) {
  memset(g, 0, sizeof *g);
  g->num_nodes = n;
  g->node_feat_dim = kv;
  g->num_edges = m;
  g->edge_feat_dim = ke;
  g->node_feats = (double*)calloc(n * kv ? n * kv : 1, sizeof(double));
  g->edge_feats = (double*)calloc(m * ke ? m * ke : 1, sizeof(double));
  g->srcs = (uint64_t*)calloc(m ? m : 1, sizeof(uint64_t));
  g->dsts = (uint64_t*)calloc(m ? m : 1, sizeof(uint64_t));
  if (!g->node_feats || !g->edge_feats || !g->srcs || !g->dsts) {
    acgo_free(g);
    return 2;
  }
  return 0;
}

static int grow_edges(acgo_graph* g, uint64_t m) {
  if (m <= g->num_edges) return 0;
  const uint64_t ke = g->edge_feat_dim;
  double* ef = (double*)realloc(g->edge_feats, sizeof(double) * (ke ? m * ke : 1));
  if (!ef) return 2;
  g->edge_feats = ef;
  uint64_t* s = (uint64_t*)realloc(g->srcs, sizeof(uint64_t) * m);
  if (!s) return 2;
  g->srcs = s;
  uint64_t* d = (uint64_t*)realloc(g->dsts, sizeof(uint64_t) * m);
  if (!d) return 2;
  g->dsts = d;
  g->num_edges = m;
  return 0;
}

int acgo_gen_er(uint64_t n, uint64_t m, uint64_t kv, uint64_t ke, uint64_t seed, acgo_graph* out) {
  if (!out || n == 0 || (n > 1 && m > n * (n - 1)) || (n == 1 && m > 0)) return 1;
  if (alloc_graph(out, n, kv, m, ke)) return 2;
  kset seen;
  if (kset_init(&seen, m)) return 2;
  uint64_t k = 0;
  for (uint64_t j = 0; j < m;) {
    const uint64_t x = draw(seed, S_ER, k++);
    const uint64_t u = below(x, n), v = below(mix64(x), n);
    if (u == v) continue;
    const int r = kset_insert(&seen, u * n + v);
    if (r < 0) {
      kset_free(&seen);
      return 2;
    }
    if (!r) continue;
    out->srcs[j] = u;
    out->dsts[j] = v;
    ++j;
  }
  kset_free(&seen);
  fill_normal(out->node_feats, n * kv, seed, S_NODE_FEAT, 0);
  fill_normal(out->edge_feats, m * ke, seed, S_EDGE_FEAT, 0);
  return 0;
}

/* R-MAT: edge_factor * 2^scale samples, quadrant probabilities (a, b, c,
 * 1 - a - b - c) per level; self-loops and repeated (src, dst) pairs dropped,
 * the first sample of each pair kept, edges in sampling order. */
int acgo_gen_rmat(int scale, int edge_factor, double a, double b, double c, uint64_t kv, uint64_t ke,
                  uint64_t seed, acgo_graph* out) {
  if (!out || scale < 1 || scale > 30 || edge_factor < 1 || a < 0 || b < 0 || c < 0 || a + b + c > 1.0)
    return 1;
  const uint64_t n = 1ull << scale, m0 = (uint64_t)edge_factor << scale;
  const double ab = a + b, abc = a + b + c;
  uint64_t* key = (uint64_t*)malloc(sizeof(uint64_t) * m0);
  if (!key) return 2;
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
    key[e] = (u << scale) | v;
  }
  kset seen;
  if (kset_init(&seen, m0)) {
    free(key);
    return 2;
  }
  uint64_t m = 0;
  for (uint64_t e = 0; e < m0; ++e) {
    const uint64_t u = key[e] >> scale, v = key[e] & (n - 1);
    if (u == v) continue;
    const int r = kset_insert(&seen, key[e]);
    if (r < 0) {
      kset_free(&seen);
      free(key);
      return 2;
    }
    if (r) key[m++] = key[e];  /* kept keys compacted in sampling order */
  }
  kset_free(&seen);
  if (alloc_graph(out, n, kv, m, ke)) {
    free(key);
    return 2;
  }
  for (uint64_t j = 0; j < m; ++j) {
    out->srcs[j] = key[j] >> scale;
    out->dsts[j] = key[j] & (n - 1);
  }
  free(key);
  fill_normal(out->node_feats, n * kv, seed, S_NODE_FEAT, 0);
  fill_normal(out->edge_feats, m * ke, seed, S_EDGE_FEAT, 0);
  return 0;
}

int acgo_fill_edges(acgo_graph* g, uint64_t m, uint64_t seed) {
  if (!g) return 1;
  const uint64_t n = g->num_nodes;
  if (m <= g->num_edges) return 0;
  if (n < 2 || m > n * (n - 1)) return 1;
  kset seen;
  if (kset_init(&seen, m)) return 2;
  for (uint64_t j = 0; j < g->num_edges; ++j)
    if (kset_insert(&seen, g->srcs[j] * n + g->dsts[j]) < 0) {
      kset_free(&seen);
      return 2;
    }
  uint64_t j = g->num_edges;
  if (grow_edges(g, m)) {
    kset_free(&seen);
    return 2;
  }
  uint64_t k = 0;
  while (j < m) {
    const uint64_t x = draw(seed, S_FILL, k++);
    const uint64_t u = below(x, n), v = below(mix64(x), n);
    if (u == v) continue;
    const int r = kset_insert(&seen, u * n + v);
    if (r < 0) {
      kset_free(&seen);
      return 2;
    }
    if (!r) continue;
    g->srcs[j] = u;
    g->dsts[j] = v;
    fill_normal(g->edge_feats + j * g->edge_feat_dim, g->edge_feat_dim, seed, S_FILL_FEAT,
                2 * j * g->edge_feat_dim);
    ++j;
  }
  kset_free(&seen);
  return 0;
}

/* Plant a pattern: a weakly connected set of pn data vertices grown by random
 * walks (the largest of up to 64 attempts), its walk tree plus random induced
 * edges up to pe pattern edges (new data edges with fresh features where the
 * set is short of vertices or edges), shuffled, relabelled by a random
 * permutation, features copied with N(0, noise^2) added.  Edges may be
 * appended to `data`. */
int acgo_plant(acgo_graph* data, uint64_t pn, uint64_t pe, double noise, uint64_t seed, acgo_graph* pat,
               uint64_t* truth_vertex, uint64_t* truth_edge) {
  if (!data || !pat) return 1;
  const uint64_t n = data->num_nodes, m = data->num_edges;
  if (pn == 0 || pn > n || pe > pn * (pn - 1)) return 1;
  int rc = 2;
  uint64_t *off = NULL, *nbr = NULL, *eid = NULL, *cur = NULL, *pedge = NULL, *perm = NULL;
  ulist S = {0}, tree = {0}, s2 = {0}, t2 = {0}, nsrc = {0}, ndst = {0}, chosen = {0}, extra = {0};
  kset have = {0}, taken = {0};
  off = (uint64_t*)calloc(n + 1, sizeof(uint64_t));
  nbr = (uint64_t*)malloc(sizeof(uint64_t) * (2 * m + 1));
  eid = (uint64_t*)malloc(sizeof(uint64_t) * (2 * m + 1));
  cur = (uint64_t*)malloc(sizeof(uint64_t) * (n + 1));
  if (!off || !nbr || !eid || !cur) goto done;
  /* undirected incidence lists: (neighbour, edge id) at both endpoints */
  for (uint64_t e = 0; e < m; ++e) {
    off[data->srcs[e] + 1]++;
    off[data->dsts[e] + 1]++;
  }
  for (uint64_t v = 0; v < n; ++v) off[v + 1] += off[v];
  memcpy(cur, off, sizeof(uint64_t) * n);
  for (uint64_t e = 0; e < m; ++e) {
    const uint64_t u = data->srcs[e], v = data->dsts[e];
    nbr[cur[u]] = v;
    eid[cur[u]++] = e;
    nbr[cur[v]] = u;
    eid[cur[v]++] = e;
  }
  uint64_t ctr = 0;
  for (int attempt = 0; attempt < 64 && S.n < pn; ++attempt) {
    s2.n = t2.n = 0;
    const uint64_t start = m ? data->srcs[below(draw(seed, S_WALK, ctr++), m)] : below(draw(seed, S_WALK, ctr++), n);
    if (ul_push(&s2, start)) goto done;
    for (uint64_t tries = 0; s2.n < pn && tries < 400 * pn; ++tries) {
      const uint64_t u = s2.v[below(draw(seed, S_WALK, ctr++), s2.n)];
      const uint64_t deg = off[u + 1] - off[u];
      if (!deg) continue;
      const uint64_t k = off[u] + below(draw(seed, S_WALK, ctr++), deg);
      const uint64_t w = nbr[k];
      if (ul_has(&s2, w)) continue;
      if (ul_push(&s2, w) || ul_push(&t2, eid[k])) goto done;
    }
    if (s2.n > S.n) {
      ul_swap(&S, &s2);
      ul_swap(&tree, &t2);
    }
  }
  /* still short (tiny components): connect fresh vertices by new edges;
     chosen holds data edge ids, or -(k + 1) for new edge k, as two's complement */
  while (S.n < pn) {
    const uint64_t w = below(draw(seed, S_NEW_EDGE, ctr++), n);
    if (ul_has(&S, w)) continue;
    const uint64_t u = S.v[below(draw(seed, S_NEW_EDGE, ctr++), S.n)];
    if (ul_push(&S, w) || ul_push(&nsrc, u) || ul_push(&ndst, w)) goto done;
    if (ul_push(&chosen, (uint64_t)(-(int64_t)nsrc.n))) goto done;
  }
  for (uint64_t i = 0; i < tree.n; ++i)
    if (ul_push(&chosen, tree.v[i])) goto done;
  if (chosen.n > pe) chosen.n = pe;
  /* induced data edges not chosen yet, in random order */
  if (kset_init(&have, 64) || kset_init(&taken, chosen.n + 1)) goto done;
  for (uint64_t i = 0; i < chosen.n; ++i)  /* data edges only (new ones are negative) */
    if ((int64_t)chosen.v[i] >= 0 && kset_insert(&taken, chosen.v[i]) < 0) goto done;
  for (uint64_t i = 0; i < S.n; ++i) {
    const uint64_t u = S.v[i];
    for (uint64_t k = off[u]; k < off[u + 1]; ++k) {
      const uint64_t e = eid[k];
      if (data->srcs[e] != u || !ul_has(&S, nbr[k]) || nbr[k] == u) continue;
      if (kset_insert(&have, u * n + nbr[k]) < 0) goto done;
      if (!kset_has(&taken, e) && ul_push(&extra, e)) goto done;
    }
  }
  if (extra.n) qsort(extra.v, extra.n, sizeof(uint64_t), cmp_u64);
  {
    uint64_t w = 0;
    for (uint64_t i = 0; i < extra.n; ++i)
      if (i == 0 || extra.v[i] != extra.v[i - 1]) extra.v[w++] = extra.v[i];
    extra.n = w;
  }
  for (uint64_t i = extra.n; i > 1; --i) {
    const uint64_t j = below(draw(seed, S_PICK, i), i), t = extra.v[i - 1];
    extra.v[i - 1] = extra.v[j];
    extra.v[j] = t;
  }
  for (uint64_t i = 0; i < extra.n && chosen.n < pe; ++i)
    if (ul_push(&chosen, extra.v[i])) goto done;
  for (uint64_t i = 0; i < nsrc.n; ++i)
    if (kset_insert(&have, nsrc.v[i] * n + ndst.v[i]) < 0) goto done;
  while (chosen.n < pe) {  /* new edges among the set */
    const uint64_t u = S.v[below(draw(seed, S_NEW_EDGE, ctr++), pn)];
    const uint64_t v = S.v[below(draw(seed, S_NEW_EDGE, ctr++), pn)];
    if (u == v) continue;
    const int r = kset_insert(&have, u * n + v);
    if (r < 0) goto done;
    if (!r) continue;
    if (ul_push(&nsrc, u) || ul_push(&ndst, v)) goto done;
    if (ul_push(&chosen, (uint64_t)(-(int64_t)nsrc.n))) goto done;
  }
  /* append the new data edges with fresh features */
  const uint64_t ke = data->edge_feat_dim, m_old = data->num_edges;
  if (nsrc.n) {
    if (grow_edges(data, m_old + nsrc.n)) goto done;
    for (uint64_t i = 0; i < nsrc.n; ++i) {
      data->srcs[m_old + i] = nsrc.v[i];
      data->dsts[m_old + i] = ndst.v[i];
    }
    fill_normal(data->edge_feats + m_old * ke, nsrc.n * ke, seed ^ m_old, S_NEW_FEAT, 0);
  }
  pedge = (uint64_t*)malloc(sizeof(uint64_t) * (chosen.n + 1));
  perm = (uint64_t*)malloc(sizeof(uint64_t) * pn);
  if (!pedge || !perm) goto done;
  for (uint64_t j = 0; j < chosen.n; ++j) {
    const int64_t c = (int64_t)chosen.v[j];
    pedge[j] = c >= 0 ? (uint64_t)c : m_old + (uint64_t)(-c - 1);
  }
  for (uint64_t i = chosen.n; i > 1; --i) {
    const uint64_t j = below(draw(seed, S_PICK, 1000003 + i), i), t = pedge[i - 1];
    pedge[i - 1] = pedge[j];
    pedge[j] = t;
  }
  /* relabel by a random permutation; features plus noise */
  for (uint64_t i = 0; i < pn; ++i) perm[i] = i;
  for (uint64_t i = pn; i > 1; --i) {
    const uint64_t j = below(draw(seed, S_PICK, 2000003 + i), i), t = perm[i - 1];
    perm[i - 1] = perm[j];
    perm[j] = t;
  }
  const uint64_t kv = data->node_feat_dim, np = chosen.n;
  if (alloc_graph(pat, pn, kv, np, ke)) goto done;
  fill_normal(pat->node_feats, pn * kv, seed, S_NOISE_V, 0);
  fill_normal(pat->edge_feats, np * ke, seed, S_NOISE_E, 0);
  for (uint64_t i = 0; i < pn; ++i) {
    const uint64_t dv = S.v[perm[i]];
    if (truth_vertex) truth_vertex[i] = dv;
    for (uint64_t k = 0; k < kv; ++k)
      pat->node_feats[i * kv + k] = data->node_feats[dv * kv + k] + noise * pat->node_feats[i * kv + k];
  }
  for (uint64_t j = 0; j < np; ++j) {
    const uint64_t e = pedge[j];
    if (truth_edge) truth_edge[j] = e;
    uint64_t ls = 0, ld = 0;
    for (uint64_t i = 0; i < pn; ++i) {
      if (S.v[perm[i]] == data->srcs[e]) ls = i;
      if (S.v[perm[i]] == data->dsts[e]) ld = i;
    }
    pat->srcs[j] = ls;
    pat->dsts[j] = ld;
    for (uint64_t k = 0; k < ke; ++k)
      pat->edge_feats[j * ke + k] = data->edge_feats[e * ke + k] + noise * pat->edge_feats[j * ke + k];
  }
  rc = 0;
done:
  free(off);
  free(nbr);
  free(eid);
  free(cur);
  free(pedge);
  free(perm);
  ul_free(&S);
  ul_free(&tree);
  ul_free(&s2);
  ul_free(&t2);
  ul_free(&nsrc);
  ul_free(&ndst);
  ul_free(&chosen);
  ul_free(&extra);
  kset_free(&have);
  kset_free(&taken);
  return rc;
}
