// acg_batch.cu -- many patterns against one data graph (acg_batch_*).
//
// The reference matches one pattern per run (main.cu:72-75); matching N
// patterns there means N runs, each rebuilding everything.  Here the data
// graph's preparation (CSR orderings, FP32 features, warp work splits) is done
// once, and the patterns are packed into groups, each matched as one disjoint
// union: every statistic of the algorithm is per pattern edge or per pattern
// vertex, so each member's mu is exactly its own match (each column keeps its
// member's quirk coverage, each vertex its member's iteration count).  Groups
// are at most 64 columns and 64 pattern vertices wide (the register-resident
// warp forms of the vertex-side kernels); patterns are sorted by iteration
// count before packing, so that a group's members iterate about as long as
// its longest.  All groups share one set of workspaces (the largest of each
// buffer over the groups) and the whole batch is captured into one CUDA graph,
// re-launched by every acg_batch_match with the same outputs and stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <memory>
#include <numeric>
#include <vector>

#include "acg.h"
#include "acg_plan.h"

using namespace acg;

struct acg_batch {
  acg_data* data = nullptr;
  int npat = 0;
  std::vector<int> pn;                    // vertices per pattern
  std::vector<std::vector<int>> members;  // pattern indices of each group
  std::vector<acg_plan*> plans;           // one per group
  std::vector<UnionOut> uo;               // per group (outputs set when captured)
  double* mu_u = nullptr;                 // [Dn][widest group] scratch
  std::vector<DevBuf> owned;              // shared workspaces, member features, scratch
  cudaStream_t own = nullptr;             // capture stream for callers on the null stream
  cudaGraphExec_t exec = nullptr;
  size_t nodes = 0;
  std::vector<double*> exec_outs;         // outputs the graph was captured with
  cudaStream_t exec_stream = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr, fence = nullptr;
  bool timed = false;
  acg_batch_info tune{};                  // autotune results (model, shape)
  double wide_iter_per_col = 0, wide_once_per_col = 0;  // patterns too wide to share a group
};

namespace {

constexpr int kGroupCols = 64;   // union columns (pattern edges) per group
constexpr int kGroupVerts = 64;  // union pattern vertices per group

void destroy(acg_batch* B) {
  if (!B) return;
  for (acg_plan* P : B->plans) acg_plan_destroy(P);
  if (B->exec) cudaGraphExecDestroy(B->exec);
  if (B->own) cudaStreamDestroy(B->own);
  for (cudaEvent_t e : {B->e0, B->e1, B->fence})
    if (e) cudaEventDestroy(e);
  dev_free_all(&B->owned);
  delete B;
}

struct HostPattern {
  int pn = 0, pe = 0, iters = 0;
  std::vector<uint64_t> ps, pd;
  const acg_graph* g = nullptr;
};

// The union spec of a group, with its member features copied into `owned`.
acg_status union_spec(acg_data* D, const std::vector<HostPattern>& hp, const std::vector<int>& mem,
                      std::vector<DevBuf>* owned, cudaStream_t s, PatternSpec* out) {
  PatternSpec& sp = *out;
  sp = PatternSpec{};
  sp.is_union = true;
  std::vector<int> p0(mem.size() + 1, 0);
  for (size_t i = 0; i < mem.size(); ++i) p0[i + 1] = p0[i] + hp[mem[i]].pn;
  sp.Pn = p0.back();
  // columns: every member's covered columns first, then the rest
  struct Col {
    int m, q;
    long long qlim;
  };
  std::vector<Col> cov, rest;
  for (size_t i = 0; i < mem.size(); ++i) {
    const HostPattern& h = hp[mem[i]];
    const long long lim = (long long)h.pn * D->Dn;
    for (int q = 0; q < h.pe; ++q) {
      const long long ql = std::max(0LL, lim - (long long)q * D->De);
      (ql > 0 ? cov : rest).push_back(Col{(int)i, q, ql});
    }
  }
  cov.insert(cov.end(), rest.begin(), rest.end());
  sp.Pe = (int)cov.size();
  std::vector<uint64_t> ps(sp.Pe), pd(sp.Pe);
  sp.qlim.resize(sp.Pe);
  sp.qmember.resize(sp.Pe);
  for (int u = 0; u < sp.Pe; ++u) {
    const Col& c = cov[u];
    const HostPattern& h = hp[mem[c.m]];
    ps[u] = (uint64_t)p0[c.m] + h.ps[c.q];
    pd[u] = (uint64_t)p0[c.m] + h.pd[c.q];
    sp.qlim[u] = c.qlim;
    sp.qmember[u] = c.m;  // a member's columns keep their order (covered ones are its first)
  }
  ACG_TRY(build_incidence(sp.Pn, sp.Pe, ps.data(), pd.data(), &sp.pat));
  sp.iters_p.resize(sp.Pn);
  for (size_t i = 0; i < mem.size(); ++i)
    std::fill(sp.iters_p.begin() + p0[i], sp.iters_p.begin() + p0[i + 1], hp[mem[i]].iters);
  // member features: vertices in member order, edges in union column order
  double *pv = nullptr, *pe = nullptr;
  ACG_TRY(dev_alloc(owned, sizeof(double) * (size_t)std::max(1, sp.Pn) * std::max(1, D->Kv), (void**)&pv, s));
  ACG_TRY(dev_alloc(owned, sizeof(double) * (size_t)std::max(1, sp.Pe) * std::max(1, D->Ke), (void**)&pe, s));
  for (size_t i = 0; i < mem.size(); ++i) {
    const HostPattern& h = hp[mem[i]];
    if (h.pn && D->Kv)
      ACG_CUDA_TRY(cudaMemcpyAsync(pv + (size_t)p0[i] * D->Kv, h.g->node_feats,
                                   sizeof(double) * h.pn * D->Kv, cudaMemcpyDeviceToDevice, s));
  }
  if (D->Ke)
    for (int u = 0; u < sp.Pe; ++u)
      ACG_CUDA_TRY(cudaMemcpyAsync(pe + (size_t)u * D->Ke,
                                   hp[mem[cov[u].m]].g->edge_feats + (size_t)cov[u].q * D->Ke,
                                   sizeof(double) * D->Ke, cudaMemcpyDeviceToDevice, s));
  sp.pv = pv;
  sp.pe = pe;
  return ACG_OK;
}

// ---------------------------------------------------------------- autotune
constexpr int kProbeIters = 3;

// One probe: the union of `mem` with every member running kProbeIters BP
// iterations, on its own (non-shared) workspaces, matched twice; the second
// match gives the time per iteration and the time outside the iterations.
acg_status probe(acg_data* D, const std::vector<HostPattern>& hp, const std::vector<int>& mem,
                 const acg_options& o, double* mu_scratch, cudaStream_t s, double* ms_iter,
                 double* ms_once) {
  std::vector<DevBuf> owned;
  PatternSpec sp;
  acg_status st = union_spec(D, hp, mem, &owned, s, &sp);
  acg_plan* P = nullptr;
  if (st == ACG_OK) {
    for (int& x : sp.iters_p) x = kProbeIters;
    st = plan_create_impl(D, std::move(sp), o, s, false, &P);
  }
  for (int k = 0; k < 2 && st == ACG_OK; ++k) st = run_match_any(P, mu_scratch, s, nullptr);
  if (st == ACG_OK) {
    if (cudaEventSynchronize(P->ev[4]) != cudaSuccess)
      st = set_error(ACG_ERR_CUDA, "autotune probe: %s", cudaGetErrorString(cudaGetLastError()));
    float t02 = 0, t23 = 0, t34 = 0, t01 = 0, t12 = 0;
    cudaEventElapsedTime(&t01, P->ev[0], P->ev[1]);
    cudaEventElapsedTime(&t12, P->ev[1], P->ev[2]);
    cudaEventElapsedTime(&t23, P->ev[2], P->ev[3]);
    cudaEventElapsedTime(&t34, P->ev[3], P->ev[4]);
    t02 = t01 + t12;
    *ms_iter = t23 / kProbeIters;
    *ms_once = t02 + t34;
  }
  if (P) acg_plan_destroy(P);
  cudaStreamSynchronize(s);  // the plan's work is done before its member features go
  dev_free_all(&owned);
  return st;
}

// The first patterns of `order` packed greedily up to `cols` columns.
std::vector<int> prefix_group(const std::vector<HostPattern>& hp, const std::vector<int>& order,
                              int cols) {
  std::vector<int> g;
  int c = 0, v = 0;
  for (int i : order) {
    if (hp[i].pe > kGroupCols || hp[i].pn > kGroupVerts) continue;
    if (!g.empty() && (c + hp[i].pe > cols || v + hp[i].pn > kGroupVerts || (int)g.size() == kMaxUnion))
      break;
    g.push_back(i);
    c += hp[i].pe;
    v += hp[i].pn;
  }
  return g;
}

int cols_of(const std::vector<HostPattern>& hp, const std::vector<int>& g) {
  int c = 0;
  for (int i : g) c += hp[i].pe;
  return c;
}

// Measure the cost model and the launch shape (see acg.h); fills B->tune and
// the chosen shape into *o.
acg_status autotune(acg_batch* B, const std::vector<HostPattern>& hp, const std::vector<int>& order,
                    acg_options* o, cudaStream_t s) {
  acg_data* D = B->data;
  std::vector<DevBuf> owned;
  double* mu = nullptr;
  acg_status st = dev_alloc(&owned, sizeof(double) * (size_t)D->Dn * kGroupVerts + 8, (void**)&mu, s);
  const std::vector<int> g64 = prefix_group(hp, order, kGroupCols);
  if (st == ACG_OK && g64.empty()) st = set_error(ACG_ERR_UNSUPPORTED, "autotune: no pattern fits a group");
  // launch shape: blocks per SM of the edge-side and the vertex-side passes
  // (0 = as many as fit)
  const int shapes[4][2] = {{0, 0}, {2, 0}, {0, 1}, {2, 1}};
  double best = 1e300, it64 = 0, once64 = 0;
  int bs = 0;
  for (int k = 0; k < 4 && st == ACG_OK; ++k) {
    acg_options oo = *o;
    oo.edge_blocks_per_sm = shapes[k][0];
    oo.vertex_blocks_per_sm = shapes[k][1];
    double mi = 0, mo = 0;
    st = probe(D, hp, g64, oo, mu, s, &mi, &mo);
    if (st == ACG_OK && mi < best) {
      best = mi;
      bs = k;
      it64 = mi;
      once64 = mo;
    }
  }
  if (st == ACG_OK) {
    o->edge_blocks_per_sm = shapes[bs][0];
    o->vertex_blocks_per_sm = shapes[bs][1];
    // the linear model from three widths (least squares in the columns)
    std::vector<double> xc, yi, yo;
    xc.push_back(cols_of(hp, g64));
    yi.push_back(it64);
    yo.push_back(once64);
    for (int w : {kGroupCols / 4, kGroupCols / 2}) {
      const std::vector<int> g = prefix_group(hp, order, w);
      double mi = 0, mo = 0;
      st = probe(D, hp, g, *o, mu, s, &mi, &mo);
      if (st != ACG_OK) break;
      xc.push_back(cols_of(hp, g));
      yi.push_back(mi);
      yo.push_back(mo);
    }
    if (st == ACG_OK) {
      auto fit = [&](const std::vector<double>& y, double* slope, double* icpt) {
        double mx = 0, my = 0;
        for (size_t i = 0; i < xc.size(); ++i) {
          mx += xc[i];
          my += y[i];
        }
        mx /= xc.size();
        my /= xc.size();
        double sxy = 0, sxx = 0;
        for (size_t i = 0; i < xc.size(); ++i) {
          sxy += (xc[i] - mx) * (y[i] - my);
          sxx += (xc[i] - mx) * (xc[i] - mx);
        }
        *slope = sxx > 0 ? std::max(0.0, sxy / sxx) : 0.0;
        *icpt = std::max(0.0, my - *slope * mx);
      };
      fit(yi, &B->tune.iter_ms_per_column, &B->tune.iter_ms_fixed);
      fit(yo, &B->tune.once_ms_per_column, &B->tune.once_ms_fixed);
      // patterns too wide to share a group run alone (the tile-form kernels):
      // a per-column cost from the widest of them
      int wi = -1;
      for (int i : order)
        if ((hp[i].pe > kGroupCols || hp[i].pn > kGroupVerts) && (wi < 0 || hp[i].pe > hp[wi].pe)) wi = i;
      if (wi >= 0 && hp[wi].pe > 0) {
        double mi = 0, mo = 0;
        st = probe(D, hp, {wi}, *o, mu, s, &mi, &mo);
        if (st == ACG_OK) {
          B->wide_iter_per_col = mi / hp[wi].pe;
          B->wide_once_per_col = mo / hp[wi].pe;
        }
      }
      B->tune.edge_blocks_per_sm = o->edge_blocks_per_sm;
      B->tune.vertex_blocks_per_sm = o->vertex_blocks_per_sm;
      B->tune.autotuned = 1;
    }
  }
  cudaStreamSynchronize(s);
  dev_free_all(&owned);
  return st;
}

// Groups as contiguous runs of `order` (sorted by iteration count) minimising
// the model's total: a run's cost is iters(last) * (a c + b) + (e c + f).
std::vector<std::vector<int>> plan_groups(const std::vector<HostPattern>& hp, const std::vector<int>& order,
                                          const acg_batch_info& m, double wide_iter, double wide_once,
                                          double* total) {
  const int n = (int)order.size();
  std::vector<double> best(n + 1, 1e300);
  std::vector<int> from(n + 1, 0);
  best[0] = 0;
  for (int i = 1; i <= n; ++i) {
    int cols = 0, verts = 0;
    bool alone = false;
    for (int j = i - 1; j >= 0; --j) {
      const HostPattern& h = hp[order[j]];
      cols += h.pe;
      verts += h.pn;
      alone = alone || h.pe > kGroupCols || h.pn > kGroupVerts;
      const int cnt = i - j;
      if (cnt > 1 && (alone || cols > kGroupCols || verts > kGroupVerts || cnt > kMaxUnion)) break;
      double cost = hp[order[i - 1]].iters * (m.iter_ms_per_column * cols + m.iter_ms_fixed) +
                    m.once_ms_per_column * cols + m.once_ms_fixed;
      if (alone && wide_iter > 0)  // a pattern that runs alone in the tile-form kernels
        cost = hp[order[i - 1]].iters * wide_iter * cols + wide_once * cols;
      if (best[j] + cost < best[i]) {
        best[i] = best[j] + cost;
        from[i] = j;
      }
    }
  }
  std::vector<std::vector<int>> groups;
  for (int i = n; i > 0; i = from[i]) groups.emplace_back(order.begin() + from[i], order.begin() + i);
  std::reverse(groups.begin(), groups.end());
  *total = best[n];
  return groups;
}

}  // namespace

extern "C" {

acg_status acg_batch_create(acg_data* D, const acg_graph* patterns, int32_t npatterns,
                            const acg_options* opt, void* stream, acg_batch** out) {
  clear_error();
  if (!out) return set_error(ACG_ERR_INVALID_ARGUMENT, "acg_batch_create: out is null");
  *out = nullptr;
  if (!D) return set_error(ACG_ERR_INVALID_ARGUMENT, "acg_batch_create: data is null");
  if (npatterns <= 0 || !patterns)
    return set_error(ACG_ERR_INVALID_ARGUMENT, "acg_batch_create: no patterns");
  acg_options o;
  ACG_TRY(resolve_options(opt, &o));
  o.kernel_timing = 0;
  cudaStream_t s = (cudaStream_t)stream;
  std::unique_ptr<acg_batch, void (*)(acg_batch*)> B(new acg_batch(), destroy);
  B->data = D;
  B->npat = npatterns;
  // host copies of the pattern endpoints, validated as acg_plan_create does
  std::vector<HostPattern> hp(npatterns);
  for (int i = 0; i < npatterns; ++i) {
    const acg_graph* g = &patterns[i];
    if (g->num_nodes == 0 || g->num_nodes > 128 || g->num_edges > 256 ||
        g->node_feat_dim != (uint64_t)D->Kv || g->edge_feat_dim != (uint64_t)D->Ke ||
        (g->num_nodes && D->Kv && !g->node_feats) || (g->num_edges && D->Ke && !g->edge_feats) ||
        (g->num_edges && (!g->srcs || !g->dsts)))
      return set_error(ACG_ERR_INVALID_ARGUMENT,
                       "pattern %d: empty, above 128 vertices / 256 edges, feature dimensions "
                       "unlike the data graph's, or null arrays", i);
    HostPattern& h = hp[i];
    h.g = g;
    h.pn = (int)g->num_nodes;
    h.pe = (int)g->num_edges;
    h.iters = o.num_iters < 0 ? h.pn : o.num_iters;
    h.ps.resize(h.pe);
    h.pd.resize(h.pe);
    if (h.pe) {
      ACG_CUDA_TRY(cudaMemcpyAsync(h.ps.data(), g->srcs, 8 * (size_t)h.pe, cudaMemcpyDeviceToHost, s));
      ACG_CUDA_TRY(cudaMemcpyAsync(h.pd.data(), g->dsts, 8 * (size_t)h.pe, cudaMemcpyDeviceToHost, s));
    }
    B->pn.push_back(h.pn);
  }
  ACG_CUDA_TRY(cudaStreamSynchronize(s));
  for (int i = 0; i < npatterns; ++i)
    for (int q = 0; q < hp[i].pe; ++q)
      if (hp[i].ps[q] >= (uint64_t)hp[i].pn || hp[i].pd[q] >= (uint64_t)hp[i].pn)
        return set_error(ACG_ERR_INDEX_OUT_OF_RANGE, "pattern %d edge %d endpoint >= %d", i, q, hp[i].pn);
  // groups: by iteration count, packed up to the column / vertex budget
  std::vector<int> order(npatterns);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return hp[a].iters < hp[b].iters; });
  if (o.autotune && D->Dn > 0) {
    ACG_TRY(autotune(B.get(), hp, order, &o, s));
    double total = 0;
    B->members = plan_groups(hp, order, B->tune, B->wide_iter_per_col, B->wide_once_per_col, &total);
    B->tune.predicted_ms = total;
  } else {
    std::vector<int> cur;
    int cols = 0, verts = 0;
    for (int i : order) {
      const bool alone = hp[i].pe > kGroupCols || hp[i].pn > kGroupVerts;
      if (!cur.empty() && (alone || cols + hp[i].pe > kGroupCols || verts + hp[i].pn > kGroupVerts ||
                           (int)cur.size() == kMaxUnion)) {
        B->members.push_back(cur);
        cur.clear();
        cols = verts = 0;
      }
      cur.push_back(i);
      cols += hp[i].pe;
      verts += hp[i].pn;
      if (alone) {
        B->members.push_back(cur);
        cur.clear();
        cols = verts = 0;
      }
    }
    if (!cur.empty()) B->members.push_back(cur);
  }
  // one deferred plan per group
  int widest = 1;
  for (const auto& mem : B->members) {
    PatternSpec sp;
    ACG_TRY(union_spec(D, hp, mem, &B->owned, s, &sp));
    widest = std::max(widest, sp.Pn);
    acg_plan* P = nullptr;
    ACG_TRY(plan_create_impl(D, std::move(sp), o, s, true, &P));
    B->plans.push_back(P);
    UnionOut u;
    u.n = (int)mem.size();
    u.p0[0] = 0;
    for (size_t i = 0; i < mem.size(); ++i) {
      u.out[i] = nullptr;
      u.p0[i + 1] = u.p0[i] + hp[mem[i]].pn;
    }
    B->uo.push_back(u);
  }
  // shared workspaces: the largest of each large buffer over the groups
  const size_t nbig = B->plans[0]->big.size();
  for (acg_plan* P : B->plans)
    if (P->big.size() != nbig) return set_error(ACG_ERR_INVALID_ARGUMENT, "batch: workspace layouts differ");
  for (size_t j = 0; j < nbig; ++j) {
    size_t bytes = 0;
    for (acg_plan* P : B->plans) bytes = std::max(bytes, P->big[j].first);
    void* buf = nullptr;
    ACG_TRY(dev_alloc(&B->owned, bytes, &buf, s));
    for (acg_plan* P : B->plans) *P->big[j].second = buf;
  }
  ACG_TRY(dev_alloc(&B->owned, sizeof(double) * (size_t)D->Dn * widest + 8, (void**)&B->mu_u, s));
  for (cudaEvent_t* e : {&B->e0, &B->e1})
    ACG_CUDA_TRY(cudaEventCreate(e));
  ACG_CUDA_TRY(cudaEventCreateWithFlags(&B->fence, cudaEventDisableTiming));
  ACG_CUDA_TRY(cudaStreamCreateWithFlags(&B->own, cudaStreamNonBlocking));
  ACG_CUDA_TRY(cudaStreamSynchronize(s));
  *out = B.release();
  return ACG_OK;
}

acg_status acg_batch_match(acg_batch* B, double* const* mu_out, void* stream) {
  clear_error();
  if (!B || !mu_out) return set_error(ACG_ERR_INVALID_ARGUMENT, "acg_batch_match: null argument");
  for (int i = 0; i < B->npat; ++i)
    if (!mu_out[i] && B->data->Dn > 0)
      return set_error(ACG_ERR_INVALID_ARGUMENT, "acg_batch_match: output %d is null", i);
  if (B->data->Dn == 0) return ACG_OK;
  // stream capture needs a stream other than the legacy null stream
  cudaStream_t caller = (cudaStream_t)stream;
  cudaStream_t s = caller ? caller : B->own;
  if (!caller) {
    ACG_CUDA_TRY(cudaEventRecord(B->fence, caller));
    ACG_CUDA_TRY(cudaStreamWaitEvent(s, B->fence, 0));
  }
  std::vector<double*> outs(mu_out, mu_out + B->npat);
  if (!B->exec || outs != B->exec_outs || s != B->exec_stream) {
    if (B->exec) {
      cudaGraphExecDestroy(B->exec);
      B->exec = nullptr;
    }
    for (size_t g = 0; g < B->members.size(); ++g)
      for (size_t i = 0; i < B->members[g].size(); ++i) B->uo[g].out[i] = mu_out[B->members[g][i]];
    ACG_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    acg_status st = ACG_OK;
    for (size_t g = 0; g < B->plans.size() && st == ACG_OK; ++g)
      st = run_match_any(B->plans[g], B->mu_u, s, &B->uo[g]);
    cudaGraph_t graph = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(s, &graph);
    if (st != ACG_OK) {
      if (graph) cudaGraphDestroy(graph);
      return st;
    }
    if (ce != cudaSuccess)
      return set_error(ACG_ERR_CUDA, "acg_batch_match: capture: %s", cudaGetErrorString(ce));
    cudaGraphGetNodes(graph, nullptr, &B->nodes);
    const cudaError_t ie = cudaGraphInstantiate(&B->exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess)
      return set_error(ACG_ERR_CUDA, "acg_batch_match: instantiate: %s", cudaGetErrorString(ie));
    B->exec_outs = outs;
    B->exec_stream = s;
  }
  ACG_CUDA_TRY(cudaEventRecord(B->e0, s));
  ACG_CUDA_TRY(cudaGraphLaunch(B->exec, s));
  ACG_CUDA_TRY(cudaEventRecord(B->e1, s));
  B->timed = true;
  if (!caller) {
    ACG_CUDA_TRY(cudaEventRecord(B->fence, s));
    ACG_CUDA_TRY(cudaStreamWaitEvent(caller, B->fence, 0));
  }
  return ACG_OK;
}

acg_status acg_batch_get_info(acg_batch* B, acg_batch_info* out) {
  clear_error();
  if (!B || !out) return set_error(ACG_ERR_INVALID_ARGUMENT, "acg_batch_get_info: null argument");
  *out = acg_batch_info{};
  out->patterns = B->npat;
  out->groups = (int32_t)B->members.size();
  out->graph_nodes = (int64_t)B->nodes;
  int widest_cols = 0;
  for (acg_plan* P : B->plans) widest_cols = std::max(widest_cols, P->Pe);
  out->widest_group_columns = widest_cols;
  out->autotuned = B->tune.autotuned;
  out->iter_ms_per_column = B->tune.iter_ms_per_column;
  out->iter_ms_fixed = B->tune.iter_ms_fixed;
  out->once_ms_per_column = B->tune.once_ms_per_column;
  out->once_ms_fixed = B->tune.once_ms_fixed;
  out->predicted_ms = B->tune.predicted_ms;
  out->edge_blocks_per_sm = B->tune.edge_blocks_per_sm;
  out->vertex_blocks_per_sm = B->tune.vertex_blocks_per_sm;
  if (B->timed) {
    ACG_CUDA_TRY(cudaEventSynchronize(B->e1));
    float ms = 0;
    cudaEventElapsedTime(&ms, B->e0, B->e1);
    out->ms_last = ms;
  }
  return ACG_OK;
}

acg_status acg_batch_destroy(acg_batch* B) {
  destroy(B);
  return ACG_OK;
}

}  // extern "C"
