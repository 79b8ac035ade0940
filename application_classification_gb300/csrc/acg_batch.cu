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
  for (int u = 0; u < sp.Pe; ++u) {
    const Col& c = cov[u];
    const HostPattern& h = hp[mem[c.m]];
    ps[u] = (uint64_t)p0[c.m] + h.ps[c.q];
    pd[u] = (uint64_t)p0[c.m] + h.pd[c.q];
    sp.qlim[u] = c.qlim;
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
  if (o.cnull)
    return set_error(ACG_ERR_UNSUPPORTED, "acg_batch_create: the cnull option is for single plans");
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
  {
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
